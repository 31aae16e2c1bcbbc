"""The parquet fixed point on the device (pffrg_parquet) against the oracle's restatement of
launch_parquet! (src/Launcher/parquet.jl:43-80): the same number of iterations and the same
converged vertex and self energy, at the FP64 bar of 1e-10 relative in the max norm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(x, ref):
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.mark.parametrize("Lam", [5.0, 1.5])
def test_device_parquet_matches_oracle(pkg, O, Lam):
    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = wl.Workload("t", "square", 3, "heisenberg", [[1.0]], 1, Lam, 10, 4, 3, 0.0, 0)
    lat, r, m, a = wl.build_state(w)  # bare couplings: the reference's start of the iteration
    ref = a.buf.copy()
    it_ref, ea_ref, er_ref = O.parquet(O.Problem(r, m), Lam, ref, 3, ptol=(1e-8, 1e-8), max_iter=30)
    with FlowContext(r, m, precision="fp64") as ctx:
        ctx.upload(C.SLOT_A, a)
        it, ea, er = ctx.parquet(Lam, 3, parquet_tol=(1e-8, 1e-8), max_iter=30)
        got = pkg.action.Action.empty_like(a)
        ctx.download(C.SLOT_A, got)
    print(f"Λ={Lam}: {it} iterations (oracle {it_ref}), residual {ea:.2e} (oracle {ea_ref:.2e})")
    assert it == it_ref and 1 < it < 30
    assert rel_err(got.buf, ref) < 1e-10
    assert abs(ea - ea_ref) <= 1e-6 * max(ea_ref, 1e-300) or abs(ea - ea_ref) < 1e-14


def test_device_parquet_u1dm(pkg, O):
    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = wl.Workload("t", "triangular", 3, "triangular-dm-c3", [[1.0, 0.8, 0.3]], 1, 2.0, 8, 3, 3, 0.0, 0,
                    symmetry="u1-dm")
    lat, r, m, a = wl.build_state(w)
    ref = a.buf.copy()
    it_ref, _, _ = O.parquet(O.Problem(r, m, symmetry="u1-dm"), 2.0, ref, 2, ptol=(1e-8, 1e-8), max_iter=30)
    with FlowContext(r, m, symmetry="u1-dm", precision="fp64") as ctx:
        ctx.upload(C.SLOT_A, a)
        it, _, _ = ctx.parquet(2.0, 2, parquet_tol=(1e-8, 1e-8), max_iter=30)
        got = pkg.action.Action.empty_like(a)
        ctx.download(C.SLOT_A, got)
    assert it == it_ref
    assert rel_err(got.buf, ref) < 1e-10
