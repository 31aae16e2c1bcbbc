"""FP64 GPU against the CPU oracle where the benchmark's own code paths run.

The small-lattice parity tests (test_gpu_parity.py) have at most 8 sites and
therefore always run the 8-lane team shape with one site per lane.  These
tests pin the paths of the benchmark configurations to the oracle at the FP64
bar (1e-10 relative in the max norm):

* the benchmark state itself: pyrochlore L = 6 (48 sites, 8047 overlap
  rows), nearest-neighbour Heisenberg, 2 loops, 50/15/10 frequencies, Λ = 1,
  N(0, 0.05) seed 1 plus the bare coupling on the Ω = 0 t slice
  (src/Flow/compute.jl:115-174, flow_su2_t.jl:2-82), with the mixed path
  against the same oracle at the stated 1e-6;
* every built team shape that covers the sites, including those with several
  sites per lane and 16/32 lanes, on square L = 5 (12 sites), square L = 8
  (25 sites) and pyrochlore L = 6, each with the overlap rows staged in shared
  memory and read through L1/L2;
* a U(1)-DM state with many sites: kagome L = 8 XXZ + DM (82 sites, six
  components, 7772 overlap rows), 3 loops with the Σ corrections
  (compute.jl:177-287, flow_u1_dm_t.jl:2-115).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(8, 1), (16, 1), (32, 1), (16, 3), (16, 4), (32, 2), (32, 3), (32, 4), (32, 8)]


def rel_err(x, ref):
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def oracle_rhs(O, r, m, a, Lam, loops, eval_, symmetry="su2", sigma_corr=False):
    P = O.Problem(r, m, symmetry=symmetry)
    da = np.zeros_like(a.buf)
    O.dsigma(P, Lam, a.buf, da)
    O.dgamma(P, loops, Lam, a.buf, da, eval_, sigma_corr=sigma_corr)
    return da


def gpu_rhs(pkg, r, m, a, Lam, loops, eval_, precision="fp64", symmetry="su2", shape=None, staging=None,
            sigma_corr=False):
    import pffrg_gb300._capi as C
    from pffrg_gb300.flow import FlowContext

    with FlowContext(r, m, symmetry=symmetry, precision=precision) as ctx:
        if shape is not None:
            ctx.set_team_shape(*shape)
        if staging is not None:
            ctx.set_overlap_staging(staging)
        ctx.upload(C.SLOT_A, a)
        ctx.rhs(Lam, eval_, loops=loops, sigma_corr=sigma_corr)
        da = pkg.action.Action.empty_like(a)
        ctx.download(C.SLOT_DA, da)
        return da.buf.copy()


def test_benchmark_state_fp64_and_mixed_vs_oracle(pkg, O):
    import pffrg_gb300.workloads as wl

    w = wl.WORKLOADS["pyrochlore-L6-2l"]
    lat, r, m, a = wl.build_state(w)
    ref = oracle_rhs(O, r, m, a, w.Lam, w.loops, w.eval)
    got = gpu_rhs(pkg, r, m, a, w.Lam, w.loops, w.eval)
    e64 = rel_err(got, ref)
    mixed = gpu_rhs(pkg, r, m, a, w.Lam, w.loops, w.eval, precision="mixed")
    em = rel_err(mixed, ref)
    print(f"pyrochlore L=6 2-loop: FP64 GPU vs oracle {e64:.2e}, mixed vs oracle {em:.2e}")
    assert e64 < 1e-10
    assert em < 1e-6


CASES = [("square", 5, 2), ("square", 8, 2), ("pyrochlore", 6, 1)]


@pytest.mark.parametrize("lattice,size,loops", CASES)
def test_team_shapes_and_staging_vs_oracle(pkg, O, lattice, size, loops):
    import pffrg_gb300.workloads as wl

    w = wl.Workload("t", lattice, size, "heisenberg", [[1.0]], loops, 1.0, 10, 4, 3, 0.05, 1, bare_on_t=True,
                    eval=2)
    lat, r, m, a = wl.build_state(w)
    ref = oracle_rhs(O, r, m, a, w.Lam, loops, w.eval)
    ns = r.num_sites
    ran = 0
    for shape in SHAPES:
        if shape[0] * shape[1] < ns:
            continue
        for staging in (1, 2):
            got = gpu_rhs(pkg, r, m, a, w.Lam, loops, w.eval, shape=shape, staging=staging)
            e = rel_err(got, ref)
            assert e < 1e-10, (lattice, size, shape, staging, e)
            ran += 1
    assert ran >= 2 * (5 if ns > 16 else 6)


def test_kagome_L8_u1dm_3loop_vs_oracle(pkg, O):
    import pffrg_gb300.workloads as wl

    w = wl.Workload("t", "kagome", 8, "kagome-xxz-dm", [[1.0, 0.8, 0.2]], 3, 1.0, 10, 4, 3, 0.05, 11,
                    symmetry="u1-dm", eval=2)
    lat, r, m, a = wl.build_state(w)
    assert r.num_sites >= 32
    ref = oracle_rhs(O, r, m, a, w.Lam, 3, w.eval, symmetry="u1-dm", sigma_corr=True)
    for shape, staging in ((None, 1), (None, 2), ((32, 3), 0), ((32, 4), 0)):
        got = gpu_rhs(pkg, r, m, a, w.Lam, 3, w.eval, symmetry="u1-dm", shape=shape, staging=staging,
                      sigma_corr=True)
        e = rel_err(got, ref)
        print(f"kagome L=8 u1-dm 3-loop, shape {shape}, staging {staging}: FP64 GPU vs oracle {e:.2e}")
        assert e < 1e-10
    mixed = gpu_rhs(pkg, r, m, a, w.Lam, 3, w.eval, precision="mixed", symmetry="u1-dm", sigma_corr=True)
    assert rel_err(mixed, ref) < 1e-6
