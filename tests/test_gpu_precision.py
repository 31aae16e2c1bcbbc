"""Mixed path against the FP64 path on the GPU, team shapes, the autotuner and the χ clusters.

The FP64 path reproduces the oracle's adaptive decisions (test_gpu_parity.py), so the FP64 GPU
path is the comparator here: the mixed path (FP32 gathers, FP64 node setup, FP64 hand-off of
the Simpson subdomains whose decisions FP32 rounding could flip, FP64 Gauss-Kronrod integrals)
must agree with it to the stated 1e-6 relative in the max norm.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(x, ref):
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def rhs(pkg, r, m, a, Lam, eval_, loops, precision, handoff=None, shape=None):
    import pffrg_gb300._capi as C
    from pffrg_gb300.flow import FlowContext

    with FlowContext(r, m, precision=precision) as ctx:
        if handoff is not None:
            ctx.set_fp64_handoff(handoff)
        if shape is not None:
            ctx.set_team_shape(*shape)
        ctx.upload(C.SLOT_A, a)
        ctx.rhs(Lam, eval_, loops=loops)
        da = pkg.action.Action.empty_like(a)
        ctx.download(C.SLOT_DA, da)
        return da.buf.copy()


def test_mixed_small_lambda_flow_state(pkg):
    """A flow state near the breakdown (square L=3, Λ ≈ 0.1): without the hand-off the mixed path
    decides some Simpson subdomains a level apart from FP64 (errors up to the quadrature tolerance,
    7.7e-5 measured on 50/15/10 meshes); with it the two agree to FP32 arithmetic."""
    from pffrg_gb300.flow import get_eval
    from pffrg_gb300.launcher import launch

    keep = {}

    def measure(Lam, dLam, m, a, ctx):
        keep["state"] = (Lam, m, a.copy())
        return True

    res = launch("", "square", 3, "heisenberg", "su2", [[1.0]], num_sigma=30, num_omega=10, num_nu=8,
                 initial=50.0, final=0.1, ode_tol=(1e-3, 1e-3), parquet=False, precision="fp64",
                 correlations=False, measure=measure)
    from pffrg_gb300 import lattice as L

    Lam, m, a = keep["state"]
    assert Lam <= 0.11 and res.Lam[-1] == Lam
    r = L.get_reduced_lattice("heisenberg", [[1.0]], L.get_lattice("square", 3))
    ev = get_eval(Lam, 10, 100)
    ref = rhs(pkg, r, m, a, Lam, ev, 1, "fp64")
    got = rhs(pkg, r, m, a, Lam, ev, 1, "mixed")
    raw = rhs(pkg, r, m, a, Lam, ev, 1, "mixed", handoff=0.0)
    e, e0 = rel_err(got, ref), rel_err(raw, ref)
    print(f"Λ={Lam:.4f}: mixed vs FP64 {e:.2e} (without hand-off {e0:.2e})")
    assert e < 1e-6


def test_mixed_pyrochlore_benchmark_state(pkg):
    """The benchmark state (pyrochlore L=6, 2 loops, 50/15/10, N(0, 0.05) seed 1 + bare J on the Ω=0
    t slice) at Λ=1: mixed against FP64 within 1e-6."""
    import pffrg_gb300.workloads as wl

    w = wl.WORKLOADS["pyrochlore-L6-2l"]
    lat, r, m, a = wl.build_state(w)
    ref = rhs(pkg, r, m, a, w.Lam, w.eval, w.loops, "fp64")
    got = rhs(pkg, r, m, a, w.Lam, w.eval, w.loops, "mixed")
    e = rel_err(got, ref)
    print(f"pyrochlore L=6 benchmark state: mixed vs FP64 {e:.2e}")
    assert e < 1e-6


def test_team_shapes_agree_and_autotune(pkg):
    """Every built shape that covers the sites gives the FP64 result to rounding (the t-channel
    overlap sums are split over the lanes differently); the autotuner returns one of them."""
    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = wl.WORKLOADS["pyrochlore-L6-reduced"]
    lat, r, m, a = wl.build_state(w)
    shapes = [(16, 3), (16, 4), (32, 2), (32, 4)]
    outs = [rhs(pkg, r, m, a, w.Lam, w.eval, w.loops, "fp64", shape=s) for s in shapes]
    for s, o in zip(shapes[1:], outs[1:]):
        assert rel_err(o, outs[0]) < 1e-12, s
    with FlowContext(r, m, precision="mixed") as ctx:
        ctx.upload(C.SLOT_A, a)
        t, spl = ctx.autotune_team_shape(w.Lam, w.eval, loops=w.loops)
        assert t * spl >= r.num_sites and (t, spl) in [(16, 3), (16, 4), (32, 2), (32, 3)]
        with pytest.raises(Exception):
            ctx.set_team_shape(24, 2)  # not built


def test_chi_cluster_matches_single_block(pkg):
    """χ with every integral on a cluster of 8 or 16 blocks equals χ with one block per integral
    (same pop order, same cut order, same blocked total)."""
    import dataclasses

    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = dataclasses.replace(wl.WORKLOADS["square-L3-1l"], noise=0.1)
    lat, r, m, a = wl.build_state(w, num_sigma=20, num_omega=8, num_nu=6)
    chi_mesh = np.array([0.0, 0.5, 3.0])
    out = {}
    for prec in ("fp64", "mixed"):
        for cl, blocks in ((1 << 40, 8), (0, 8), (0, 16)):
            with FlowContext(r, m, precision=prec) as ctx:
                ctx.set_chi_integrand(prec)
                ctx.set_chi_cluster(cl, blocks)
                ctx.upload(C.SLOT_A, a)
                out[prec, cl, blocks] = ctx.chi_slot(0.3, C.SLOT_A, chi_mesh)
                st = ctx.read_stats()
        assert np.array_equal(out[prec, 0, 8], out[prec, 1 << 40, 8]), prec
        assert np.array_equal(out[prec, 0, 16], out[prec, 1 << 40, 8]), prec
        assert st["chi_evals"] > 0


def test_chi_mixed_vs_fp64(pkg):
    """χ of the mixed path (FP32 integrand with the float-float node setup) against χ of the FP64
    path on the same state, within the stated 1e-6 of max|χ|."""
    import dataclasses

    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = dataclasses.replace(wl.WORKLOADS["square-L3-1l"], noise=0.05)
    lat, r, m, a = wl.build_state(w, num_sigma=20, num_omega=8, num_nu=6)
    chi_mesh = np.array([0.0, 0.4, 2.0])
    out = {}
    for prec in ("fp64", "mixed"):
        with FlowContext(r, m, precision=prec) as ctx:
            ctx.set_chi_integrand(prec)  # the FP32 integrand (the default of a mixed context is FP64)
            ctx.upload(C.SLOT_A, a)
            out[prec] = ctx.chi_slot(1.0, C.SLOT_A, chi_mesh)
    e = rel_err(out["mixed"], out["fp64"])
    print(f"χ mixed vs FP64: {e:.2e}")
    assert e < 1e-6


def test_chi_remembered_capacities_identical(pkg):
    """χ of the same state twice in one context: the second call starts every integral at the capacity the
    first one needed and runs those that need a cluster on a second stream, alongside the others; the
    values and the evaluation counts are those of the first call."""
    import dataclasses

    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = dataclasses.replace(wl.WORKLOADS["square-L3-1l"], noise=0.1)
    lat, r, m, a = wl.build_state(w)
    chi_mesh = np.array([0.0, 0.1, 0.5, 2.0])
    with FlowContext(r, m, precision="fp64") as ctx:
        ctx.upload(C.SLOT_A, a)
        got = []
        for _ in range(3):
            got.append(ctx.chi_slot(0.15, C.SLOT_A, chi_mesh))
            st = ctx.read_stats()
            got.append((st["chi_evals"], st["chi_regions_max"]))
    print("χ evaluations, most regions of one integral:", got[1])
    assert got[1][1] > 32768  # some integrals need a cluster, so the later calls use the second stream
    assert np.array_equal(got[0], got[2]) and np.array_equal(got[0], got[4])
    assert got[1] == got[3] == got[5]
