"""Mesh scans and resampling: the oracle's numpy restatement of resample_from_to (Action.jl:360-557,
channel.jl:416-466, mesh.jl:86-122, param.jl:25-87) pinned by the reference's own known answers
(src/Frequency/test.jl: mesh bounds; src/Action/test.jl:80-154: Σ on the mesh and beyond it, exact
interpolation of functions linear in each frequency), and the package's host resampling checked
against it.  The device scans and resampling are checked against the oracle in test_gpu_flow.py."""
import numpy as np
import pytest


def _params():
    from pffrg_gb300 import frequency as F

    return (F.DEFAULT_P_SIGMA, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU,
            F.DEFAULT_P_CHI, F.DEFAULT_LINS, F.DEFAULT_BOUNDS)


def oracle_view(a):
    """Σ and the vertex of a package Action as the oracle's plain arrays (views, so writes land in a)."""
    keys = ("q1", "q2_1", "q2_2", "q3")
    G = [{x: {q: getattr(ch, q) for q in keys} for x, ch in zip("stu", v.channels)} for v in a.Γ]
    return a.Σ, G


def mesh_dict(m):
    return {k: np.asarray(getattr(m, k)) for k in ("sigma", "omega_s", "nu_s", "omega_t", "nu_t", "chi")}


def test_mesh_bounds_known_answer(O):
    """src/Frequency/test.jl:10-21: get_mesh(δ, 1, 30, 0.4) runs from 0 to 1."""
    rng = np.random.default_rng(0)
    for _ in range(5):
        lst = O.get_mesh(rng.uniform(0.05, 0.95), 1.0, 30, 0.4)
        assert len(lst) == 31 and lst[0] == 0.0 and abs(lst[-1] - 1.0) < 1e-14
        assert np.all(np.diff(lst) > 0)


def test_sigma_known_answers(O):
    """src/Action/test.jl:80-83: on the mesh Σ is returned, beyond it Σ[end] σ[end] / w."""
    rng = np.random.default_rng(1)
    mesh = O.get_mesh(0.3, 5.0, 20, 0.4)
    S = rng.normal(size=21)
    S[0] = 0.0  # Σ is odd in w
    for k in range(21):
        assert O.sigma_at(mesh[k], mesh, S) == pytest.approx(S[k], rel=1e-14, abs=1e-14)
        assert O.sigma_at(-mesh[k], mesh, S) == pytest.approx(-S[k], rel=1e-14, abs=1e-14)
    outer = 7.5
    assert O.sigma_at(outer, mesh, S) == pytest.approx(S[-1] * mesh[-1] / outer, rel=1e-14)


def test_resample_linear_functions_exact(O):
    """src/Action/test.jl:125-154: interpolation reproduces a function linear in each frequency at
    points inside the old meshes, and the last values beyond them."""
    rng = np.random.default_rng(2)
    ns, nO, nn = 3, 8, 6
    O_old, n_old = O.get_mesh(0.5, 10.0, nO - 1, 0.4), O.get_mesh(0.4, 8.0, nn - 1, 0.4)
    O_new, n_new = O.get_mesh(0.7, 9.0, nO - 1, 0.4), O.get_mesh(0.2, 7.0, nn - 1, 0.4)
    c = rng.normal(size=(ns, 8))

    def f(s, w, v, vp):
        return (c[s, 0] + c[s, 1] * w + c[s, 2] * v + c[s, 3] * vp + c[s, 4] * w * v + c[s, 5] * w * vp +
                c[s, 6] * v * vp + c[s, 7] * w * v * vp)

    S = np.arange(ns)[:, None, None, None]
    q3 = f(S, O_old[None, :, None, None], n_old[None, None, :, None], n_old[None, None, None, :])
    ch = {"q1": q3[:, :, -1, -1].copy(), "q2_1": q3[:, :, :, -1].copy(), "q2_2": q3[:, :, -1, :].copy(), "q3": q3}
    new = {k: np.zeros_like(v) for k, v in ch.items()}
    O.resample_channel(O_old, n_old, ch, O_new, n_new, new)
    want = f(S, O_new[None, :, None, None], n_new[None, None, :, None], n_new[None, None, None, :])
    assert np.allclose(new["q3"], want, rtol=1e-12, atol=1e-12)
    assert np.allclose(new["q2_1"], f(S[:, :, :, 0], O_new[None, :, None], n_new[None, None, :], n_old[-1]),
                       rtol=1e-12, atol=1e-12)
    assert np.allclose(new["q1"], f(S[:, :, 0, 0], O_new[None, :], n_old[-1], n_old[-1]), rtol=1e-12, atol=1e-12)
    # beyond the old Ω mesh: the last value
    new2 = {k: np.zeros_like(v) for k, v in ch.items()}
    O.resample_channel(O_old, n_old, ch, O_old * 1.5, n_old, new2)
    assert np.array_equal(new2["q1"][:, -1], ch["q1"][:, -1])


@pytest.mark.parametrize("symmetry", ["su2", "u1-dm"])
@pytest.mark.parametrize("Lam", [0.3, 8.0])
def test_host_resample_matches_oracle(pkg, O, symmetry, Lam):
    """launcher.resample_from_to (the package's host path: scans, meshes, interpolation) against the
    oracle's restatement, below lins[1] (scanned meshes) and above it (scaled meshes)."""
    import pffrg_gb300.workloads as wl
    from pffrg_gb300 import launcher as LA

    if symmetry == "su2":
        w = wl.WORKLOADS["square-L3-1l"]
    else:
        w = wl.Workload("t", "kagome", 3, "kagome-xxz-dm", [[1.0, 0.8, 0.2]], 1, 1.0, 10, 5, 4, 0.1, 3,
                        symmetry="u1-dm")
    lat, r, m, a = wl.build_state(w, num_sigma=12, num_omega=6, num_nu=5)
    a.Σ[:] = m.sigma / (1.0 + m.sigma ** 2)
    rng = np.random.default_rng(5)
    chi = [rng.normal(size=(r.num_sites, m.num_chi)) for _ in range(1 if symmetry == "su2" else 3)]
    P = _params()
    host = a.copy()
    m_host = LA.resample_from_to(Lam, *P, m, a, host, chi)
    ref = a.copy()
    S_old, G_old = oracle_view(a)
    S_new, G_new = oracle_view(ref)
    m_ref = O.resample_from_to(Lam, *P, mesh_dict(m), S_old, G_old, S_new, G_new, chi)
    for k, v in m_ref.items():
        assert np.allclose(getattr(m_host, k), v, rtol=1e-15, atol=0.0), k
    assert np.max(np.abs(host.buf - ref.buf)) <= 1e-13 * np.max(np.abs(ref.buf))


def test_host_scan_bit_exact_vs_oracle(pkg, O):
    """launcher.scan (whose δb loop reads only the two trial-mesh points that Δ uses) returns exactly
    the oracle's scan, which rebuilds the whole trial mesh every step as the reference does, on cuts
    that decay, peak at a finite frequency or are noise."""
    from pffrg_gb300 import frequency as F
    from pffrg_gb300 import launcher as LA

    rng = np.random.default_rng(0)
    for t in range(300):
        n = int(rng.integers(6, 40))
        x = F.get_mesh(rng.uniform(0.1, 3.0), rng.uniform(5.0, 50.0), n - 1, 0.4)
        kind = t % 3
        if kind == 0:
            y = np.exp(-x / rng.uniform(0.1, 5.0)) * rng.normal()
        elif kind == 1:
            y = rng.normal(size=n)
        else:
            y = 1.0 / (1.0 + (x - rng.uniform(0.0, 3.0)) ** 2)
        p = (0.4, rng.uniform(0.005, 0.05), rng.uniform(0.05, 0.2), 0.05 * rng.uniform(0.1, 5.0),
             40.0 * rng.uniform(0.1, 5.0))
        assert LA.scan(x, y, *p) == O.scan(x, y, *p), t
