"""Generate the golden fixtures of the flow right-hand side from the FP64 CPU oracle.

The reference's own test suite pins no dΓ/dΣ values and the reference
(Julia) cannot run here, so these fixtures are the oracle's FP64 outputs on
seeded states; the oracle itself is pinned by tests/test_oracle_known_answers.py.
Run from the repository root:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

CASES = {
    # name: (lattice, size, J, loops, (num_sigma, num_omega, num_nu), eval, seed, noise)
    "square_L3_1l": ("square", 3, [[1.0]], 1, (11, 4, 3), 3, 21, 0.1),
    "square_L3_2l": ("square", 3, [[1.0]], 2, (11, 4, 3), 3, 22, 0.1),
    "honeycomb_L3_3l": ("honeycomb", 3, [[1.0], [0.5]], 3, (9, 3, 3), 2, 23, 0.1),
}


def compute(name):
    entry.load_package()
    import pffrg_gb300.workloads as wl

    O = entry.load_oracle()
    lattice, size, J, loops, (ns, no, nn), eval_, seed, noise = CASES[name]
    w = wl.Workload(name, lattice, size, "heisenberg", J, loops, 1.0, ns, no, nn, noise, seed, eval=eval_)
    lat, r, m, a = wl.build_state(w)
    P = O.Problem(r, m)
    da = np.zeros_like(a.buf)
    O.dsigma(P, w.Lam, a.buf, da)
    O.dgamma(P, loops, w.Lam, a.buf, da, eval_, sigma_corr=loops >= 3)
    return w, a.buf, da


def main():
    for name in CASES:
        w, a, da = compute(name)
        np.savez_compressed(Path(__file__).parent / f"{name}.npz", a=a, da=da, eval=w.eval, loops=w.loops)
        print(name, a.size, float(np.max(np.abs(da))))


if __name__ == "__main__":
    main()
