"""Golden fixtures of the flow right-hand side (tests/golden/, made by tests/golden/make_golden.py).

CPU: the oracle reproduces its committed outputs (pins it against accidental
change, across x86 and Arm builds).  GPU: the CUDA path reproduces them through
the C ABI (FP64, 1e-10 relative in the max norm).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden  # noqa: E402

NAMES = sorted(make_golden.CASES)


def rel(x, y):
    return float(np.max(np.abs(x - y)) / np.max(np.abs(y)))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(pkg, name):
    ref = np.load(GOLDEN / f"{name}.npz")
    w, a, da = make_golden.compute(name)
    assert np.array_equal(a, ref["a"])
    assert rel(da, ref["da"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(pkg, name):
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.action import Action
    from pffrg_gb300.flow import FlowContext

    ref = np.load(GOLDEN / f"{name}.npz")
    lattice, size, J, loops, (ns, no, nn), eval_, seed, noise = make_golden.CASES[name]
    w = wl.Workload(name, lattice, size, "heisenberg", J, loops, 1.0, ns, no, nn, noise, seed, eval=eval_)
    lat, r, m, a = wl.build_state(w)
    assert np.array_equal(a.buf, ref["a"])
    da = Action.empty_like(a)
    with FlowContext(r, m, precision="fp64") as ctx:
        ctx.compute_dsigma(w.Lam, a, da)
        ctx.compute_dgamma(w.Lam, a, da, eval_, loops=loops, sigma_corr=loops >= 3)
    assert rel(da.buf, ref["da"]) < 1e-10
