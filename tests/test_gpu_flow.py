"""The device Bogacki-Shampine step and the launch! driver against the oracle.

The reference step (launcher_1l.jl:83-116) is restated here in numpy on top
of the oracle's right-hand side; the device step (pffrg_bs_step) must give the
same 3rd-order solution and error ratio in FP64 (1e-10 relative).
"""
import numpy as np
import pytest
from test_oracle_resample import mesh_dict, oracle_view

pytestmark = pytest.mark.gpu


def oracle_bs_step(O, P, a, Lam, dLam, loops, eval_, ode_tol=(1e-8, 1e-2)):
    m = np.zeros(a.buf.size, dtype=bool)
    m[: a.layout.num_sigma] = True
    m |= a.gamma_mask()
    q3 = a.q3_mask()

    def rhs(state, lam):
        out = np.zeros_like(state)
        O.dsigma(P, lam, state, out)
        O.dgamma(P, loops, lam, state, out, eval_, sigma_corr=loops >= 3)
        return out

    x = a.buf
    da = x.copy()
    aerr = x.copy()
    k = rhs(x, Lam)
    da[m] += -2.0 * dLam / 9.0 * k[m]
    aerr[m] += -7.0 * dLam / 24.0 * k[m]
    inter = x.copy()
    inter[m] += -0.5 * dLam * k[m]
    k = rhs(inter, Lam - 0.5 * dLam)
    da[m] += -1.0 * dLam / 3.0 * k[m]
    aerr[m] += -1.0 * dLam / 4.0 * k[m]
    inter = x.copy()
    inter[m] += -0.75 * dLam * k[m]
    k = rhs(inter, Lam - 0.75 * dLam)
    da[m] += -4.0 * dLam / 9.0 * k[m]
    aerr[m] += -1.0 * dLam / 3.0 * k[m]
    inter[m] = da[m]
    k = rhs(inter, Lam - dLam)
    aerr[m] += -1.0 * dLam / 8.0 * k[m]
    aerr[m] -= inter[m]
    delta = np.max(np.abs(aerr[q3]))
    scale = ode_tol[0] + max(np.max(np.abs(inter[q3])), np.max(np.abs(x[q3]))) * ode_tol[1]
    return inter, delta / scale


@pytest.mark.parametrize("loops", [1, 2])
def test_bs_step_matches_oracle(pkg, O, loops):
    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.action import Action
    from pffrg_gb300.flow import FlowContext

    w = wl.Workload("bs", "square", 3, "heisenberg", [[1.0]], loops, 2.0, 11, 4, 3, 0.05, 31)
    lat, r, m, a = wl.build_state(w)
    P = O.Problem(r, m)
    ref_next, ref_err = oracle_bs_step(O, P, a, 2.0, 0.1, loops, 3)
    with FlowContext(r, m, precision="fp64") as ctx:
        ctx.upload(C.SLOT_A, a)
        err, amax = ctx.bs_step(2.0, 0.1, 3, loops=loops)
        nxt = Action.empty_like(a)
        ctx.download(C.SLOT_NEXT, nxt)
    mask = np.zeros(a.buf.size, dtype=bool)
    mask[: m.num_sigma] = True
    mask |= a.gamma_mask()
    rel = np.max(np.abs(nxt.buf[mask] - ref_next[mask])) / np.max(np.abs(ref_next[mask]))
    assert rel < 1e-10
    assert err == pytest.approx(ref_err, rel=1e-9)
    assert amax == pytest.approx(np.max(np.abs(ref_next[a.q3_mask()])), rel=1e-12)


def test_launch_runs_to_final(pkg, O):
    from pffrg_gb300 import lattice as L
    from pffrg_gb300.launcher import launch

    seen = []
    last = {}

    def measure(Lam, dLam, m, a, ctx):
        seen.append(Lam)
        last.update(m=m, buf=a.buf.copy())
        return True

    res = launch("t", "square", 3, "heisenberg", "su2", [[1.0]], num_sigma=10, num_omega=4, num_nu=3, num_chi=4,
                 initial=5.0, final=3.0, parquet=False, precision="fp64", measure=measure)
    assert res.finished and res.Lam[-1] <= 3.0 + 1e-12
    assert seen == res.Lam and all(np.diff(res.Lam) < 0)
    assert res.integrand_evals > 0
    # χ of every accepted step (measure, Launcher.jl:23-35); the last one against the oracle
    assert [c[0] for c in res.chi] == res.Lam
    Lam, chi_mesh, chi = res.chi[-1]
    r = L.get_reduced_lattice("heisenberg", [[1.0]], L.get_lattice("square", 3))
    ref = O.chi(O.Problem(r, last["m"]), Lam, last["buf"], chi_mesh)
    assert np.max(np.abs(chi - ref)) <= 1e-6 * np.max(np.abs(ref))
    # the on-site static χ grows as Λ decreases (the flow stops otherwise)
    onsite = [c[2][0, 0] for c in res.chi]
    assert all(x > 0 for x in onsite) and all(np.diff(onsite) > -0.005 * np.array(onsite[:-1]))


def test_parquet_converges(pkg):
    from pffrg_gb300.launcher import launch

    res = launch("t", "square", 3, "heisenberg", "su2", [[1.0]], num_sigma=10, num_omega=4, num_nu=3, num_chi=4,
                 initial=5.0, final=5.0, parquet=True, precision="fp64", parquet_tol=(1e-8, 1e-6))
    assert 1 <= res.parquet_iterations < 50


def test_launch_writes_and_resumes_files(pkg, tmp_path):
    """launch! with output files (measure, Launcher.jl:2-60): Σ and χ of every accepted step in *_obs,
    checkpoints in *_cp (ct = 0: every step), the finished flags; an interrupted run resumes from its
    last checkpoint with overwrite = false (Launcher.jl:704-760)."""
    from pffrg_gb300 import disk as D, hdf5 as H
    from pffrg_gb300.launcher import launch

    kw = dict(num_sigma=10, num_omega=4, num_nu=3, num_chi=4, initial=5.0, parquet=False, precision="fp64",
              ct=0.0)
    f = str(tmp_path / "run")
    last = {}

    def keep(Lam, dLam, m, a, ctx):
        last.update(Lam=Lam, m=m, buf=a.buf.copy())

    res = launch(f, "square", 3, "heisenberg", "su2", [[1.0]], final=3.0, measure=keep, **kw)
    assert res.finished
    with H.File(f + "_obs", "r") as o, H.File(f + "_cp", "r") as c:
        assert o.read("finished") is True and c.read("finished") is True
        cut = sorted((float(k) for k in o.keys("χ")), reverse=True)
        assert np.allclose(cut, res.Lam)
        assert o.read("reduced_lattice/model") == "heisenberg"
        # the last checkpoint holds the accepted state before resampling, on its meshes
        Lam, dLam, m, a = D.read_checkpoint(c, 0.0)
        assert Lam == res.Lam[-1] == last["Lam"]
        assert np.array_equal(a.buf, last["buf"]) and np.array_equal(m.omega_s, last["m"].omega_s)

    # interrupted after two accepted steps, then resumed
    g = str(tmp_path / "cut")

    class Stop(Exception):
        pass

    seen = []

    def crash(Lam, dLam, m, a, ctx):
        seen.append(Lam)
        if len(seen) == 2:
            raise Stop()

    with pytest.raises(Stop):
        launch(g, "square", 3, "heisenberg", "su2", [[1.0]], final=3.0, measure=crash, **kw)
    with H.File(g + "_cp", "r") as c:
        assert "finished" not in c
        assert min(float(k) for k in c.keys("a")) == pytest.approx(seen[-1])
    res2 = launch(g, "square", 3, "heisenberg", "su2", [[1.0]], final=3.0, overwrite=False, **kw)
    assert res2.finished and res2.Lam[-1] <= 3.0 + 1e-12 and res2.Lam[0] < seen[-1]
    res3 = launch(g, "square", 3, "heisenberg", "su2", [[1.0]], final=3.0, overwrite=False, **kw)
    assert res3.reason == "calculation has finished already"


def test_sweep_matches_single_runs(pkg):
    """Concurrent instances (own context and stream each) give exactly the single-run results."""
    from pffrg_gb300.launcher import launch
    from pffrg_gb300.sweep import launch_sweep, square_j1j2_sweep

    # different sizes launch the same pass kernels with different shared memory from several threads
    inst = square_j1j2_sweep(8, sizes=(3, 4, 5, 6, 8))
    kw = dict(num_sigma=10, num_omega=4, num_nu=3, num_chi=4, initial=5.0, final=4.0, parquet=False,
              precision="mixed")
    res = launch_sweep(inst, workers=8, **kw)
    for i, r in zip(inst, res):
        single = launch("", i.name, i.size, i.model, i.symmetry, i.J, **kw)
        assert r.Lam == single.Lam
        assert np.array_equal(r.action.buf, single.action.buf)


@pytest.mark.parametrize("symmetry", ["su2", "u1-dm"])
def test_device_resample_matches_host(pkg, O, symmetry):
    """Mesh scans from the device cuts and the device resampling (pffrg_scan_cuts, pffrg_resample)
    against the host path of resample_from_to (Action.jl:483-557) and the oracle's restatement."""
    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300 import frequency as F
    from pffrg_gb300 import launcher as LA
    from pffrg_gb300.action import Action
    from pffrg_gb300.flow import FlowContext

    if symmetry == "su2":
        w = wl.WORKLOADS["square-L3-1l"]
    else:
        w = wl.Workload("t", "kagome", 3, "kagome-xxz-dm", [[1.0, 0.8, 0.2]], 1, 1.0, 10, 5, 4, 0.1, 3,
                        symmetry="u1-dm")
    lat, r, m, a = wl.build_state(w, num_sigma=12, num_omega=6, num_nu=5)
    # a smooth self energy (the scans read argmax |Σ|; a noisy one can place it where the reference's
    # own mesh rule has no valid linear bound)
    a.Σ[:] = m.sigma / (1.0 + m.sigma ** 2)
    P = (F.DEFAULT_P_SIGMA, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_CHI,
         F.DEFAULT_LINS, F.DEFAULT_BOUNDS)
    chi = [np.random.default_rng(5).normal(size=(r.num_sites, m.num_chi))]
    for Lam in (0.3, 8.0):  # scanned meshes below lins[1], scaled ones above
        host = a.copy()  # the flow resamples a copy of the accepted state (bare couplings kept)
        m_host = LA.resample_from_to(Lam, *P, m, a, host, chi)
        with FlowContext(r, m, symmetry=symmetry, precision="fp64") as ctx:
            ctx.upload(C.SLOT_NEXT, a)
            sig, arg, cuts = ctx.scan_cuts(C.SLOT_NEXT)
            for c, v in enumerate(a.Γ):
                for ch, chan in enumerate(v.channels):
                    want = int(np.argmax(np.abs(chan.q3).reshape(-1, order="F")))
                    assert arg[3 * c + ch] == want
                    assert np.array_equal(cuts[3 * c + ch], LA.channel_cuts(chan.q3))
            cl = [[cuts[3 * c + ch] for ch in range(3)] for c in range(len(a.Γ))]
            m_dev = LA.new_meshes(Lam, *P, m, sig, cl, chi)
            for name in ("sigma", "omega_s", "nu_s", "omega_t", "nu_t", "chi"):
                assert np.array_equal(getattr(m_dev, name), getattr(m_host, name))
            ctx.resample(C.SLOT_NEXT, C.SLOT_A, m_dev)
            dev = Action.empty_like(a)
            ctx.download(C.SLOT_A, dev)
        assert np.max(np.abs(dev.buf - host.buf)) <= 1e-13 * np.max(np.abs(host.buf))
        ref = a.copy()
        S_old, G_old = oracle_view(a)
        S_new, G_new = oracle_view(ref)
        m_ref = O.resample_from_to(Lam, *P, mesh_dict(m), S_old, G_old, S_new, G_new, chi)
        for name, v in m_ref.items():
            assert np.allclose(getattr(m_dev, name), v, rtol=1e-15, atol=0.0), name
        assert np.max(np.abs(dev.buf - ref.buf)) <= 1e-13 * np.max(np.abs(ref.buf))


def test_flow_matches_oracle_flow(pkg, O):
    """The whole flow loop against the oracle: launch! in FP64 on the GPU (device steps, device scans and
    resampling, χ after every step) and the same loop of launcher_1l.jl:56-198 restated here on the
    oracle's right-hand side, host scans and resampling (launcher.resample_from_to) and the oracle's χ.
    Square L = 3, 10/4/3 frequencies, Λ 5 → 0.7 (step control rejects steps from Λ ≈ 0.93 on; with these
    small meshes the flow turns unstable near 0.6): both take the same accepted and rejected steps (the
    cutoffs agree to 1e-8, the error ratios differing in the last digits), and χ(ω = 0) agrees at every
    accepted cutoff within the stated 1e-6 of max|χ|."""
    from pffrg_gb300 import action as A
    from pffrg_gb300 import frequency as F
    from pffrg_gb300 import lattice as L
    from pffrg_gb300.flow import get_eval
    from pffrg_gb300.launcher import launch, resample_from_to

    kw = dict(num_sigma=10, num_omega=4, num_nu=3, num_chi=4, initial=5.0, final=0.7, parquet=False,
              ode_tol=(1e-3, 1e-3))
    res = launch("", "square", 3, "heisenberg", "su2", [[1.0]], precision="fp64", **kw)
    # the same loop on the oracle
    lat = L.get_lattice("square", 3)
    r = L.get_reduced_lattice("heisenberg", [[1.0]], lat)
    p = (F.DEFAULT_P_SIGMA, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_OMEGA, F.DEFAULT_P_NU, F.DEFAULT_P_CHI,
         F.DEFAULT_LINS, F.DEFAULT_BOUNDS)
    m = F.initial_mesh(5.0, 10, 4, 3, 4, *p)
    a = A.get_action_empty("su2", r, m)
    A.init_action(lat, r, a)
    Lam, Lf, bmin, bmax = 5.0, 0.7, 1e-4, 0.1
    dLam = bmax * Lam
    cps = [5.0, 0.7]
    lams, chis, rejected = [], [], 0
    chi_prev = np.zeros((r.num_sites, 4))
    while Lam > Lf:
        P = O.Problem(r, m)
        inter, err = oracle_bs_step(O, P, a, Lam, dLam, 1, get_eval(Lam, 10, 100), ode_tol=(1e-3, 1e-3))
        assert err < 10.0

        def next_dlam(dl, lam):
            dl = max(bmin, min(bmax * lam, 0.85 * (1.0 / err) ** (1.0 / 3.0) * dl))
            lower = [c for c in cps if c - lam < 0.0]
            return min(dl, lam - (lower[0] if lower else 0.0))

        if err <= 1.0 or dLam <= bmin:
            Lam -= dLam
            dLam = next_dlam(dLam, Lam)
            chi = O.chi(P, Lam, inter, m.chi)
            lams.append(Lam)
            chis.append(chi[:, 0].copy())
            assert chi[0, 0] / chi_prev[0, 0] >= 0.995 if chi_prev[0, 0] else True
            chi_prev = chi
            a_inter = A.Action.empty_like(a)
            a_inter.buf[:] = inter
            a_new = a_inter.copy()  # the resampling keeps the bare couplings of the state
            m = resample_from_to(Lam, *p, m, a_inter, a_new, [chi])
            a = a_new
        else:
            dLam = next_dlam(dLam, Lam)
            rejected += 1
    assert rejected > 0
    n = min(len(res.Lam), len(lams))
    assert np.allclose(res.Lam[:n], lams[:n], rtol=1e-8, atol=0.0)
    for (Lg, mesh, cg), c in zip(res.chi, chis):
        assert np.max(np.abs(cg[:, 0] - c)) <= 1e-6 * np.max(np.abs(c)), Lg
    assert res.finished and len(res.Lam) == len(lams), (res.reason, len(res.Lam), len(lams))
    assert res.rejected == rejected
