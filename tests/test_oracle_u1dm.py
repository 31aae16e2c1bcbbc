"""The U(1)-DM restatement of the oracle (flow_u1_dm_*.jl, BSE/SDE_u1_dm.jl,
action_u1_dm.jl, correlation_u1_dm.jl) checked by two exact identities.

1. An SU(2)-symmetric vertex written in U(1)-DM components (Γxx = Γzz = Γspin,
   Γdd = Γdens, ΓDM = Γzd = Γdz = 0) must flow exactly like the SU(2) vertex
   with S = 1/2.  The adaptive rules stop on norms over all components, which
   differ between the two layouts, so the tolerances accept the first estimate
   (atol = 1e10): both sides then sample the same nodes and agree to rounding.
2. A π rotation of the spin frame about x flips the sign of ΓDM, Γzd and Γdz
   and keeps the others: the right-hand side must commute with that flip
   exactly (every term of every bubble has the matching parity).
"""
import numpy as np
import pytest

FIRST = (1e10, 1e-4)  # accept the first quadrature estimate everywhere


def _embed(pkg, a, r, m):
    from pffrg_gb300 import action as A

    b = A.get_action_empty("u1-dm", r, m)
    b.Σ[:] = a.Σ
    for dst, src in [(0, 0), (1, 0), (3, 1)]:
        b.Γ[dst].bare[:] = a.Γ[src].bare
        for cd, cs in zip(b.Γ[dst].channels, a.Γ[src].channels):
            for q in ("q1", "q2_1", "q2_2", "q3"):
                getattr(cd, q)[:] = getattr(cs, q)
    return b


def _compare(pkg, d2, d6, a2, a6):
    from pffrg_gb300 import action as A

    x2 = A.Action.empty_like(a2)
    x2.buf[:] = d2
    x6 = A.Action.empty_like(a6)
    x6.buf[:] = d6
    err = np.max(np.abs(x6.Σ - x2.Σ))
    for dst, src in [(0, 0), (1, 0), (3, 1)]:
        for cd, cs in zip(x6.Γ[dst].channels, x2.Γ[src].channels):
            for q in ("q1", "q2_1", "q2_2", "q3"):
                err = max(err, np.max(np.abs(getattr(cd, q) - getattr(cs, q))))
    off = max(np.max(np.abs(getattr(ch, q))) for c in (2, 4, 5) for ch in x6.Γ[c].channels
              for q in ("q1", "q2_1", "q2_2", "q3"))
    return err, off, np.max(np.abs(d2))


@pytest.mark.parametrize("lattice", ["square", "kagome"])
def test_u1dm_reduces_to_su2_flow(pkg, O, lattice):
    import pffrg_gb300.workloads as wl

    w = wl.Workload("t", lattice, 3, "heisenberg", [[1.0]], 1, 1.0, 8, 4, 3, 0.1, 7)
    lat, r, m, a = wl.build_state(w)
    b = _embed(pkg, a, r, m)
    P2, P6 = O.Problem(r, m), O.Problem(r, m, symmetry="u1-dm")
    for loops in (1, 2, 3):
        d2, d6 = np.zeros_like(a.buf), np.zeros_like(b.buf)
        O.dsigma(P2, 1.0, a.buf, d2, *FIRST)
        O.dgamma(P2, loops, 1.0, a.buf, d2, 2, gtol=FIRST, sigma_corr=loops >= 3, stol=FIRST)
        O.dsigma(P6, 1.0, b.buf, d6, *FIRST)
        O.dgamma(P6, loops, 1.0, b.buf, d6, 2, gtol=FIRST, sigma_corr=loops >= 3, stol=FIRST)
        err, off, scale = _compare(pkg, d2, d6, a, b)
        assert off == 0.0
        assert err <= 1e-13 * scale, (loops, err, scale)


def test_u1dm_reduces_to_su2_parquet_and_chi(pkg, O):
    import pffrg_gb300.workloads as wl

    w = wl.Workload("t", "kagome", 3, "heisenberg", [[1.0]], 1, 1.0, 8, 4, 3, 0.1, 7)
    lat, r, m, a = wl.build_state(w)
    b = _embed(pkg, a, r, m)
    P2, P6 = O.Problem(r, m), O.Problem(r, m, symmetry="u1-dm")
    # compute_Σ! then compute_Γ! (SDE.jl:58-96, compute.jl:2-54)
    d2, d6 = np.zeros_like(a.buf), np.zeros_like(b.buf)
    c2 = O.sde(P2, 1.0, a.buf, d2, 2, FIRST, FIRST)
    c6 = O.sde(P6, 1.0, b.buf, d6, 2, FIRST, FIRST)
    err, off, scale = _compare(pkg, d2, d6, a, b)
    assert off == 0.0 and err <= 1e-13 * scale
    d2, d6 = np.zeros_like(a.buf), np.zeros_like(b.buf)
    O.bse(P2, 1.0, a.buf, d2, c2, 2, FIRST)
    O.bse(P6, 1.0, b.buf, d6, c6, 2, FIRST)
    err, off, scale = _compare(pkg, d2, d6, a, b)
    assert off == 0.0 and err <= 1e-13 * scale
    # χxx = χzz = χ (S = 1/2) and χxy = 0 (correlation_u1_dm.jl vs correlation_su2.jl)
    chi_mesh = np.array([0.0, 0.5])
    x2 = O.chi(P2, 1.0, a.buf, chi_mesh, FIRST)
    xx, zz, xy = O.chi(P6, 1.0, b.buf, chi_mesh, FIRST)
    s = np.max(np.abs(x2))
    assert np.max(np.abs(xx - x2)) <= 1e-13 * s
    assert np.max(np.abs(zz - x2)) <= 1e-13 * s
    assert np.max(np.abs(xy)) == 0.0


def _flip(b):
    c = b.copy()
    for k in (2, 4, 5):
        c.Γ[k].bare[:] *= -1
        for ch in c.Γ[k].channels:
            for q in ("q1", "q2_1", "q2_2", "q3"):
                getattr(ch, q)[:] *= -1
    return c


@pytest.mark.parametrize("loops", [1, 2, 3])
def test_u1dm_spin_flip_covariance(pkg, O, loops):
    import pffrg_gb300.workloads as wl

    w = wl.Workload("t", "triangular", 3, "triangular-dm-c3", [[1.0, 0.8, 0.3]], 1, 1.0, 8, 4, 3, 0.1, 5,
                    symmetry="u1-dm")
    lat, r, m, b = wl.build_state(w)
    P = O.Problem(r, m, symmetry="u1-dm")
    fb = _flip(b)
    d1, d2 = np.zeros_like(b.buf), np.zeros_like(b.buf)
    O.dsigma(P, 1.0, b.buf, d1)
    O.dgamma(P, loops, 1.0, b.buf, d1, 2, sigma_corr=loops >= 3)
    O.dsigma(P, 1.0, fb.buf, d2)
    O.dgamma(P, loops, 1.0, fb.buf, d2, 2, sigma_corr=loops >= 3)
    x1 = type(b).empty_like(b)
    x1.buf[:] = d1
    want = _flip(x1)
    want.buf[:b.layout.num_sigma] = d1[:b.layout.num_sigma]
    # bare entries of an output are left untouched by the right-hand side: compare the rest
    mask = b.gamma_mask().copy()
    mask[:b.layout.num_sigma] = True
    assert np.max(np.abs(d1[mask])) > 0
    assert np.array_equal(d2[mask], want.buf[mask])
    # the DM part is really exercised: nonzero ΓDM, Γzd, Γdz output
    assert all(np.max(np.abs(x1.Γ[k].ch_s.q3)) > 0 for k in (2, 4, 5))
