"""Failure paths of the C ABI, made on the host: no GPU fault, trap or hang is involved.

* A state with a NaN or an infinity: every entry point that computes a
  right-hand side returns PFFRG_E_NONFINITE (a finite check of each result on
  the device, read with the call's status word) instead of handing the values
  on; the flow driver stops with a reason.  The reference has no such check
  (a NaN passes its err >= 10 and Γmax >= 1000 tests, launcher_1l.jl:125-150).
* A chunk queue of the quadrature levels too small for the state returns
  PFFRG_E_LIMIT; the default queue then gives the regular result.
* A Gauss-Kronrod segment capacity of 16 overflows on the first call and is
  grown 8x at a time until the integrals fit: the result equals the
  default-capacity result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_state(noise=0.1, seed=7):
    import pffrg_gb300.workloads as wl

    w = wl.Workload("t", "square", 3, "heisenberg", [[1.0]], 1, 1.0, 12, 5, 4, noise, seed)
    return wl.build_state(w)


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_state_is_reported(pkg, bad):
    import pffrg_gb300._capi as C
    from pffrg_gb300.flow import FlowContext

    lat, r, m, a = small_state()
    q3 = a.Γ[0].ch_t.q3
    q3[0, 1, 1, 1] = bad
    da = pkg.action.Action.empty_like(a)
    with FlowContext(r, m, precision="fp64") as ctx:
        with pytest.raises(C.PffrgError) as ei:
            ctx.compute_dsigma(1.0, a, da)
            ctx.compute_dgamma(1.0, a, da, 3)
        assert ei.value.code == C.PFFRG_E_NONFINITE, str(ei.value)
        # the device-resident paths report it too, and the context stays usable afterwards
        ctx.upload(C.SLOT_A, a)
        for call in (lambda: ctx.rhs(1.0, 3), lambda: ctx.bs_step(1.0, 0.1, 3)):
            with pytest.raises(C.PffrgError) as ei:
                call()
            assert ei.value.code == C.PFFRG_E_NONFINITE, str(ei.value)
        lat, r, m, good = small_state()
        ctx.upload(C.SLOT_A, good)
        ctx.rhs(1.0, 3)
    with FlowContext(r, m, precision="mixed") as ctx:
        a.Γ[0].ch_t.q3[0, 1, 1, 1] = bad
        ctx.upload(C.SLOT_A, a)
        with pytest.raises(C.PffrgError) as ei:
            ctx.rhs(1.0, 3)
        assert ei.value.code == C.PFFRG_E_NONFINITE, str(ei.value)


def test_flow_stops_on_non_finite_rhs(pkg):
    """The Bogacki-Shampine loop on a state with a NaN ends with a reason and accepts no step."""
    import pffrg_gb300.frequency as F
    from pffrg_gb300.flow import FlowContext
    from pffrg_gb300.launcher import FlowResult, _flow

    lat, r, m, a = small_state()
    a.Γ[1].ch_s.q2_1[2, 0, 1] = np.nan
    res = FlowResult()
    p = (F.DEFAULT_P_SIGMA, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_CHI,
         F.DEFAULT_LINS, F.DEFAULT_BOUNDS)
    with FlowContext(r, m, precision="fp64") as ctx:
        _flow(ctx, r, m, a, res, loops=1, sigma_corr=False, Li=1.0, Lf=0.5, dLi=0.1, bmin=1e-4, bmax=0.1,
              min_eval=3, max_eval=3, sigma_tol=(1e-8, 1e-4), gamma_tol=(1e-8, 1e-4), ode_tol=(1e-3, 1e-3), p=p,
              cps=[], measure=None)
    assert res.reason == "right-hand side is not finite"
    assert not res.finished and not res.Lam


def test_tiny_chunk_queue_reports_limit(pkg):
    import pffrg_gb300._capi as C
    from pffrg_gb300.flow import FlowContext

    lat, r, m, a = small_state()
    with FlowContext(r, m, precision="fp64") as ctx:
        ctx.upload(C.SLOT_A, a)
        ctx.rhs(1.0, 3)
        ref = pkg.action.Action.empty_like(a)
        ctx.download(C.SLOT_DA, ref)
        ctx.set_capacities(queue_chunks=8)
        with pytest.raises(C.PffrgError) as ei:
            ctx.rhs(1.0, 3)
        assert ei.value.code == C.PFFRG_E_LIMIT and "queue" in str(ei.value)
        ctx.set_capacities()
        ctx.rhs(1.0, 3)
        got = pkg.action.Action.empty_like(a)
        ctx.download(C.SLOT_DA, got)
    assert np.array_equal(got.buf, ref.buf)


def test_tiny_gauss_kronrod_capacity_grows(pkg):
    import pffrg_gb300._capi as C
    from pffrg_gb300.flow import FlowContext

    lat, r, m, a = small_state()
    out = []
    for gk in (0, 16):
        with FlowContext(r, m, precision="fp64") as ctx:
            ctx.set_capacities(gk_segments=gk)
            da = pkg.action.Action.empty_like(a)
            ctx.compute_dsigma(1.0, a, da)
            ctx.compute_dgamma(1.0, a, da, 3)
            ctx.upload(C.SLOT_A, a)
            ctx.rhs(0.2, 3)
            d2 = pkg.action.Action.empty_like(a)
            ctx.download(C.SLOT_DA, d2)
            out.append((da.buf.copy(), d2.buf.copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    with FlowContext(r, m, precision="fp64") as ctx:
        with pytest.raises(C.PffrgError):
            ctx.set_capacities(gk_segments=4)
