"""The CPU oracle and the host-side set-up against the reference's own known answers.

Each test restates a check of the reference's test suite (file:line cited)
so that the oracle the GPU is compared with is itself pinned to the
reference's behaviour.
"""
import math

import numpy as np
import pytest

# src/Lattice/test.jl:21-31: sites within bond distance 8
SITE_COUNTS = {"square": 145, "honeycomb": 109, "kagome": 163, "triangular": 217, "cubic": 833, "fcc": 2057,
               "bcc": 1241, "hyperhoneycomb": 319, "hyperkagome": 415, "pyrochlore": 1029, "diamond": 525}


@pytest.mark.parametrize("name", sorted(SITE_COUNTS))
def test_lattice_site_counts(pkg, name):
    lat = pkg.lattice.get_lattice(name, 8)
    assert len(lat.sites) == SITE_COUNTS[name]


@pytest.mark.parametrize("name,size,expected", [("square", 3, 6), ("square", 5, 12), ("honeycomb", 3, None),
                                                ("kagome", 3, None), ("pyrochlore", 3, None)])
def test_reduction_invariants(pkg, name, size, expected):
    lat = pkg.lattice.get_lattice(name, size)
    r = pkg.lattice.get_reduced_lattice("heisenberg", [[1.0]], lat)
    if expected is not None:
        assert r.num_sites == expected
    # multiplicities partition the lattice, exchange is an involution, the origin is site 1
    assert int(r.mult.sum()) == len(lat.sites)
    ex = r.exchange - 1
    assert np.all(ex[ex] == np.arange(r.num_sites))
    assert r.irreducible[0] == 0 and r.mult[0] == 1
    offs, rows = r.overlap_csr()
    assert rows.shape[1] == 3 and np.all(rows[:, :2] >= 1) and np.all(rows[:, :2] <= r.num_sites)
    assert np.all(rows[:, 2] >= 1) and offs[-1] == len(rows)


def test_bare_norms_su2(pkg):
    """src/Action/test.jl:316-329: square L=5 Heisenberg, |Γ_spin.bare| = 0.25, |Γ_dens.bare| = 0."""
    from pffrg_gb300 import action as A, frequency as F, lattice as L

    lat = L.get_lattice("square", 5)
    r = L.get_reduced_lattice("heisenberg", [[1.0]], lat)
    m = F.Mesh(31, 31, 31, 31, *[F.get_mesh(0.5, 1.0, 30, 0.4)] * 6)
    a = A.get_action_empty("su2", r, m)
    A.init_action(lat, r, a)
    assert np.linalg.norm(a.Γ[0].bare) == pytest.approx(0.25)
    assert np.linalg.norm(a.Γ[1].bare) == pytest.approx(0.0)


def test_bare_norms_u1_dm(pkg):
    """src/Action/test.jl:334-351: triangular-dm-c3 L=5, |Γxx| = |Γzz| = |ΓDM| = sqrt(1/8), others 0."""
    from pffrg_gb300 import action as A, frequency as F, lattice as L

    lat = L.get_lattice("triangular", 5)
    r = L.get_reduced_lattice("triangular-dm-c3", [[1.0, 1.0, 1.0]], lat)
    m = F.Mesh(31, 31, 31, 31, *[F.get_mesh(0.5, 1.0, 30, 0.4)] * 6)
    a = A.get_action_empty("u1-dm", r, m)
    A.init_action(lat, r, a)
    for c in range(3):
        assert np.linalg.norm(a.Γ[c].bare) == pytest.approx(math.sqrt(0.125))
    for c in range(3, 6):
        assert np.linalg.norm(a.Γ[c].bare) == pytest.approx(0.0)


def test_mesh_endpoints(pkg):
    """src/Frequency/test.jl:15-19."""
    rng = np.random.default_rng(0)
    x = pkg.frequency.get_mesh(float(rng.random()), 1.0, 30, 0.4)
    assert len(x) == 31 and x[0] == 0.0 and x[-1] == pytest.approx(1.0)
    assert np.all(np.diff(x) > 0)
    with pytest.raises(ValueError):
        pkg.frequency.get_mesh(1.0, 0.5, 30, 0.4)


def _square_problem(pkg, O, n=30):
    from pffrg_gb300 import frequency as F, lattice as L

    lat = L.get_lattice("square", 3)
    r = L.get_reduced_lattice("heisenberg", [[1.0]], lat)
    mesh = F.get_mesh(0.37, 1.0, n, 0.4)
    m = F.Mesh(n + 1, n + 1, n + 1, n + 1, mesh, mesh, mesh, mesh, mesh, mesh)
    return lat, r, m, O.Problem(r, m)


def test_buffer_kernel_dispatch(pkg, O):
    """src/Frequency/test.jl:22-46: kernel 4/3/2/1/0 of get_buffer_{s,t,u}."""
    lat, r, m, P = _square_problem(pkg, O)
    inf = math.inf
    w, v, vp = 0.3, 0.6, 0.2
    for ch in (1, 2, 3):
        assert O.buffer_kernel(P, ch, w, v, vp) == 4
        assert O.buffer_kernel(P, ch, w, inf, vp) == 3
        assert O.buffer_kernel(P, ch, w, v, inf) == 2
        assert O.buffer_kernel(P, ch, w, inf, inf) == 1
        assert O.buffer_kernel(P, ch, inf, inf, inf) == 0
        # sign folding keeps the kernel
        assert O.buffer_kernel(P, ch, -w, -v, -vp) == 4


def test_interpolation_multilinear_exact(pkg, O):
    """src/Action/test.jl:2-303: a multilinear f(w, v, v') is reproduced exactly, on and off the mesh."""
    from pffrg_gb300 import action as A

    lat, r, m, P = _square_problem(pkg, O)
    a = A.get_action_empty("su2", r, m)
    rng = np.random.default_rng(1)
    Ns = r.num_sites
    coef = rng.random((8, 3, 2, Ns))
    x = m.omega_s
    xe = x[-1]

    def f(ch, c, w, v, vp):
        k = coef[:, ch, c, :]
        return (k[0] * w * v * vp + k[1] * w * v + k[2] * w * vp + k[3] * v * vp + k[4] * w + k[5] * v + k[6] * vp
                + k[7])

    for c in range(2):
        for ch, chan in enumerate(a.Γ[c].channels):
            for iw, w in enumerate(x):
                chan.q1[:, iw] = f(ch, c, w, xe, xe)
                for iv, v in enumerate(x):
                    chan.q2_1[:, iw, iv] = f(ch, c, w, v, xe)
                    chan.q2_2[:, iw, iv] = f(ch, c, w, xe, v)
                    for ivp, vp in enumerate(x):
                        chan.q3[:, iw, iv, ivp] = f(ch, c, w, v, vp)
    inf = math.inf
    for ch in range(3):
        for c in range(2):
            for (w, v, vp) in [(x[3], x[7], x[11]), (0.123, 0.456, 0.789), (0.9, 0.05, 0.33)]:
                assert np.allclose(O.vertex_channel(P, a.buf, c, ch + 1, w, v, vp), f(ch, c, w, v, vp), rtol=1e-12)
                assert np.allclose(O.vertex_channel(P, a.buf, c, ch + 1, w, inf, vp), f(ch, c, w, xe, vp), rtol=1e-12)
                assert np.allclose(O.vertex_channel(P, a.buf, c, ch + 1, w, v, inf), f(ch, c, w, v, xe), rtol=1e-12)
                assert np.allclose(O.vertex_channel(P, a.buf, c, ch + 1, w, inf, inf), f(ch, c, w, xe, xe), rtol=1e-12)
            assert np.allclose(O.vertex_channel(P, a.buf, c, ch + 1, inf, inf, inf), 0.0)


def test_sigma_interpolation(pkg, O):
    """src/Action/test.jl:80-84: Σ on the mesh and its 1/w extrapolation."""
    from pffrg_gb300 import action as A

    lat, r, m, P = _square_problem(pkg, O)
    a = A.get_action_empty("su2", r, m)
    rng = np.random.default_rng(2)
    a.Σ[:] = rng.random(m.num_sigma)
    a.Σ[0] = 0.0
    for k in (0, 5, 17, m.num_sigma - 1):
        assert O.get_sigma(P, a.buf, m.sigma[k]) == pytest.approx(a.Σ[k])
        assert O.get_sigma(P, a.buf, -m.sigma[k]) == pytest.approx(-a.Σ[k])
    outer = m.sigma[-1] + 0.7
    assert O.get_sigma(P, a.buf, outer) == pytest.approx(a.Σ[-1] * m.sigma[-1] / outer)


@pytest.mark.parametrize("log_mesh", [False, True])
def test_integrators_vs_gauss_kronrod(O, log_mesh):
    """src/Flow/test.jl:44-61: integrate_lin!/integrate_log! (eval 100, tol 1e-8) against the adaptive
    Gauss-Kronrod rule on x^i exp(-x^2) sin(2 pi x), i = 1..100 on [1, 5], compared with Julia's ≈
    (rtol = sqrt(eps))."""
    got = O.test_integrators(100, 1.0, 5.0, 100, 1e-8, 1e-8, log_mesh)
    ref = np.array([O.test_quadgk(i + 1, 1.0, 5.0, 1e-8, 1e-8) for i in range(100)])
    assert np.allclose(got, ref, rtol=math.sqrt(np.finfo(float).eps), atol=0.0)


def test_gauss_kronrod_against_scipy(O):
    scipy = pytest.importorskip("scipy.integrate")
    for p in (1, 3, 7):
        ref = scipy.quad(lambda x: x ** p * math.exp(-x * x) * math.sin(2 * math.pi * x), 1.0, 5.0,
                         epsabs=1e-14, epsrel=1e-13, limit=200)[0]
        assert O.test_quadgk(p, 1.0, 5.0, 1e-12, 1e-12) == pytest.approx(ref, rel=1e-10)


def test_symmetrize(pkg, O):
    """symmetrize! (action_su2.jl:141-173): q3[i,w,v,v'] = q3[x(i),w,v',v] for v < v'."""
    from pffrg_gb300 import action as A, frequency as F, lattice as L

    lat = L.get_lattice("square", 3)
    r = L.get_reduced_lattice("heisenberg", [[1.0]], lat)
    m = F.initial_mesh(1.0, 6, 4, 5, 3)
    a = A.get_action_empty("su2", r, m)
    a.buf[:] = np.random.default_rng(3).normal(size=a.buf.size)
    P = O.Problem(r, m)
    O.symmetrize(P, a.buf)
    ex = r.exchange - 1
    for c in range(2):
        for ch, chan in enumerate(a.Γ[c].channels):
            q = chan.q3
            for v in range(m.num_nu):
                for vp in range(v + 1, m.num_nu):
                    src = np.arange(r.num_sites) if ch == 2 else ex
                    assert np.array_equal(q[:, :, v, vp], q[src, :, vp, v])


def test_layout_matches_oracle(pkg, O):
    import pffrg_gb300.workloads as wl

    lat, r, m, a = wl.build_state(wl.WORKLOADS["square-L3-1l"], num_sigma=8, num_omega=4, num_nu=3)
    assert O.Problem(r, m).action_size == a.layout.size


def test_eval_schedule(pkg):
    """eval = min(max(ceil(min_eval / sqrt(Λ)), min_eval), max_eval) (launcher_1l.jl:78)."""
    from pffrg_gb300.flow import get_eval

    assert get_eval(50.0, 10, 100) == 10
    assert get_eval(1.0, 10, 100) == 10
    assert get_eval(0.25, 10, 100) == 20
    assert get_eval(1e-4, 10, 100) == 100


def test_workload_is_seeded(pkg):
    import pffrg_gb300.workloads as wl

    s1 = wl.build_state(wl.WORKLOADS["square-L3-1l"], num_sigma=8, num_omega=4, num_nu=3)[3]
    s2 = wl.build_state(wl.WORKLOADS["square-L3-1l"], num_sigma=8, num_omega=4, num_nu=3)[3]
    assert np.array_equal(s1.buf, s2.buf)
    assert s1.Σ[0] == 0.0


@pytest.mark.parametrize("which", [0, 1])
@pytest.mark.parametrize("tol", [(1e-10, 1e-4), (1e-14, 1e-9)])
def test_hcubature_against_scipy(O, which, tol):
    """The Genz-Malik cubature behind integrate_χ_boxes (correlation_lib.jl:2-30) on two smooth
    integrands over a rectangle, against scipy's nested adaptive quadrature."""
    scipy = pytest.importorskip("scipy.integrate")
    x0, x1, y0, y1 = 0.1, 0.9, 0.2, 0.7
    if which == 0:
        f = lambda y, x: math.exp(-(x * x + 2 * y * y)) * math.cos(3 * x * y)  # noqa: E731
    else:
        f = lambda y, x: 1.0 / math.sqrt(x * x + y * y + 1e-3)  # noqa: E731
    ref = scipy.dblquad(f, x0, x1, y0, y1, epsabs=1e-14, epsrel=1e-13)[0]
    got = O.test_hcubature(which, x0, x1, y0, y1, *tol)
    assert got == pytest.approx(ref, rel=30 * tol[1])


def test_chi_constant_vertex(pkg, O):
    """compute_χ! (correlation_su2.jl:58-86) for a frequency-independent vertex and Σ = 0 factorises:
    χ_i(w) = -(2S)^2 Γ_i I(w)^2 / (2π)^2 for i > 1 and χ_1(w) = 2S I(w) / (4π) (no on-site coupling),
    with I(w) = ∫ G0(v - w/2) G0(v + w/2) dv and G0(v) = -expm1(-v^2/Λ^2) / v (bubbles.jl:2-14)."""
    scipy = pytest.importorskip("scipy.integrate")
    import dataclasses

    import pffrg_gb300.workloads as wl

    w = dataclasses.replace(wl.WORKLOADS["square-L3-1l"], noise=0.0)
    lat, r, m, a = wl.build_state(w, num_sigma=10, num_omega=5, num_nu=4)
    Lam, S = 0.8, 0.5
    chi_mesh = np.array([0.0, 0.4, 3.0])
    P = O.Problem(r, m)
    got = O.chi(P, Lam, a.buf, chi_mesh, (1e-12, 1e-9))

    def G0(v):
        return 0.0 if abs(v) <= 1e-8 else -math.expm1(-v * v / (Lam * Lam)) / v

    spin = a.Γ[0].bare
    assert spin[0] == 0.0 and a.Γ[1].bare[0] == 0.0
    for k, wv in enumerate(chi_mesh):
        g = lambda v: G0(v - 0.5 * wv) * G0(v + 0.5 * wv)  # noqa: E731
        I = sum(scipy.quad(g, lo, hi, epsabs=1e-14, epsrel=1e-12, limit=400)[0]
                for lo, hi in [(-np.inf, -10.0), (-10.0, 0.0), (0.0, 10.0), (10.0, np.inf)])
        want = -(2 * S) ** 2 * spin * I * I / (2 * math.pi) ** 2
        want[0] = 2 * S * I / (4 * math.pi)
        assert np.allclose(got[:, k], want, rtol=1e-7, atol=1e-12)
