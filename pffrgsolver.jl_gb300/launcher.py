"""launch!: the FRG flow driver above the GPU right-hand side (host side).

Restates src/Launcher/Launcher.jl:565-773 (launch!), the Bogacki-Shampine
loop of src/Launcher/launcher_{1l,2l,ml}.jl (the four stages and the error
ratio run on the device through ``pffrg_bs_step``), the parquet warm start of
src/Launcher/parquet.jl:1-100, and the mesh scan/resampling between steps
(src/Action/Action.jl:361-527, src/Action/channel.jl:416-471).  Observables
go to ``measure`` callbacks and, when ``launch`` is given a file name, to the
reference's ``*_obs`` / ``*_cp`` HDF5 files (through ``disk`` and ``hdf5``).
"""
from __future__ import annotations

import bisect
import math
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import action as A
from . import disk, hdf5
from . import frequency as F
from . import lattice as L
from . import _capi
from .flow import FlowContext, get_eval


# ---------------------------------------------------------------------------
# interpolation helpers on sorted meshes (param.jl:26-87), vectorised
# ---------------------------------------------------------------------------
def params(vals: np.ndarray, x: np.ndarray):
    """Lower/upper indices and weights of get_param for every value in vals."""
    vals = np.asarray(vals, dtype=np.float64)
    n = len(x)
    hi = np.searchsorted(x, vals, side="left")
    top = vals >= x[-1]
    hi = np.where(top, n - 1, hi)
    hi = np.clip(hi, 0, n - 1)
    lo = np.where(top, n - 1, np.where(vals < x[hi], hi - 1, hi))
    lo = np.clip(lo, 0, n - 1)
    wl = np.ones_like(vals)
    wu = np.zeros_like(vals)
    m = lo < hi
    d = np.where(m, 1.0 / np.where(m, x[hi] - x[lo], 1.0), 0.0)
    wl = np.where(m, d * (x[hi] - vals), 1.0)
    wu = np.where(m, d * (vals - x[lo]), 0.0)
    return lo, hi, wl, wu


def _interp1(v: float, x: list, y: list) -> float:
    """y interpolated at one value v on the sorted list x: get_param (param.jl:26-87) and its linear
    read-out, scalar (the same arithmetic as params for one value)."""
    n = len(x)
    if v >= x[n - 1]:
        return 1.0 * y[n - 1] + 0.0 * y[n - 1]
    hi = bisect.bisect_left(x, v)
    lo = max(hi - 1 if v < x[hi] else hi, 0)
    if lo < hi:
        d = 1.0 / (x[hi] - x[lo])
        return d * (x[hi] - v) * y[lo] + d * (v - x[lo]) * y[hi]
    return 1.0 * y[lo] + 0.0 * y[hi]


def get_sigma(w: float, sigma_mesh: np.ndarray, Sig: np.ndarray) -> float:
    """get_Σ (Action.jl:8-26)."""
    if abs(w) <= sigma_mesh[-1]:
        lo, hi, wl, wu = params(np.array([abs(w)]), sigma_mesh)
        return float(np.sign(w) * (wl[0] * Sig[lo[0]] + wu[0] * Sig[hi[0]]))
    return float(sigma_mesh[-1] * Sig[-1] / w)


# ---------------------------------------------------------------------------
# mesh scanning (Action.jl:361-449) and resampling (Action.jl:451-527, channel.jl:416-471)
# ---------------------------------------------------------------------------
def scan(x, y, p0, p1, p2, p3, p4) -> float:
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    num_lin = int(math.ceil(p0 * (len(x) - 1)))
    # a) first extremum at finite frequency, δa where the channel has decayed to 75 % of it
    da = math.inf
    idx = 0
    slope = (y[1] - y[0]) / (x[1] - x[0])
    for i in range(1, len(x) - 1):
        s = (y[i + 1] - y[i]) / (x[i + 1] - x[i])
        if np.sign(s) != np.sign(slope):
            idx = i
            break
        slope = s
    if idx > 0:
        for i in range(idx + 1, len(x)):
            if abs(y[i] / y[idx]) <= 0.75:
                da = max(x[i], num_lin * x[idx] / math.ceil(0.5 * num_lin))
                break
    # b) finite value at the origin: p1 < Δ < p2
    db = num_lin * x[1]
    if abs(y[0]) / np.max(np.abs(y)) > 1e-2:
        xl, yl = x.tolist(), y.tolist()
        yp0 = _interp1(0.0, xl, yl)  # the trial meshes all start at 0
        delta = abs(y[1] - y[0]) / max(abs(y[1]), abs(y[0]))
        while not (p1 < delta < p2):
            if delta >= p2:
                db *= 0.98
            elif delta <= p1:
                db *= 1.02
            if db >= x[-1]:
                break
            # Δ reads only the first two points of the trial mesh get_mesh(δb, x[end], len(x) - 1, p0):
            # 0 and its first linear point δb / num_lin (the same values as building the whole mesh
            # and interpolating y on it; the loop can take a few hundred 2 % steps, so it stays scalar)
            yp1 = _interp1(1 * (db / num_lin), xl, yl)
            delta = abs(yp1 - yp0) / max(abs(yp1), abs(yp0))
    # c) merge and bound
    return min(max(num_lin * p3, min(da, db)), p4)


def channel_cuts(q3):
    """The cuts through max |q3| that scan_channel reads (Action.jl:452-480): q3[s, :, v, v'],
    q3[s, w, k, k] - q3[s, w, end, end], q3[s, w, :, v'] - q3[s, w, end, v'], q3[s, w, v, :] - q3[s, w, v, end]."""
    idx = np.unravel_index(int(np.argmax(np.abs(q3).reshape(-1, order="F"))), q3.shape, order="F")
    s, w, v, vp = idx
    nu = q3.shape[2]
    cut_O = q3[s, :, v, vp]
    cut_1 = np.array([q3[s, w, k, k] - q3[s, w, -1, -1] for k in range(nu)])
    cut_2 = q3[s, w, :, vp] - q3[s, w, -1, vp]
    cut_3 = q3[s, w, v, :] - q3[s, w, v, -1]
    return np.concatenate([cut_O, cut_1, cut_2, cut_3])


def scan_channel(Lam, p_O, p_n, Om, nu, q3):
    """(Ω_lin, ν_lin) of one channel from cuts through its maximum (Action.jl:452-480)."""
    return scan_cuts(Lam, p_O, p_n, Om, nu, channel_cuts(q3))


def scan_cuts(Lam, p_O, p_n, Om, nu, cuts):
    """scan_channel on its four cuts (as returned by channel_cuts or the device)."""
    NO, Nn = len(Om), len(nu)
    cut_O, cut_1 = cuts[:NO], cuts[NO:NO + Nn]
    cut_2, cut_3 = cuts[NO + Nn:NO + 2 * Nn], cuts[NO + 2 * Nn:NO + 3 * Nn]
    O_lin = scan(Om, cut_O, p_O[0], p_O[1], p_O[2], p_O[3] * Lam, p_O[4] * Lam)
    n1 = scan(nu, cut_1, p_n[0], p_n[1], p_n[2], p_n[3] * Lam, p_n[4] * Lam)
    n2 = scan(nu, cut_2, p_n[0], p_n[1], p_n[2], p_n[3] * Lam, p_n[4] * Lam)
    n3 = scan(nu, cut_3, p_n[0], p_n[1], p_n[2], p_n[3] * Lam, p_n[4] * Lam)
    return O_lin, min(n1, n2, n3)


def _resample_channel(Om_old, nu_old, ch_old, Om_new, nu_new, ch_new):
    """Trilinear resampling of one channel (channel.jl:416-471)."""
    l1, h1, a1, b1 = params(Om_new, Om_old)
    l2, h2, a2, b2 = params(nu_new, nu_old)
    q1 = ch_old.q1
    ch_new.q1[...] = a1[None, :] * q1[:, l1] + b1[None, :] * q1[:, h1]
    for name in ("q2_1", "q2_2"):
        q = getattr(ch_old, name)
        out = (a1[None, :, None] * a2[None, None, :] * q[:, l1][:, :, l2]
               + b1[None, :, None] * a2[None, None, :] * q[:, h1][:, :, l2]
               + a1[None, :, None] * b2[None, None, :] * q[:, l1][:, :, h2]
               + b1[None, :, None] * b2[None, None, :] * q[:, h1][:, :, h2])
        getattr(ch_new, name)[...] = out
    q3 = ch_old.q3
    out = np.zeros_like(ch_new.q3)
    W1 = (a1, b1)
    I1 = (l1, h1)
    W2 = (a2, b2)
    I2 = (l2, h2)
    for k3 in range(2):  # corner order of get_q3 (channel.jl:226-242)
        for k2 in range(2):
            for k1 in range(2):
                w = W1[k1][:, None, None] * W2[k2][None, :, None] * W2[k3][None, None, :]
                out += w[None] * q3[:, I1[k1]][:, :, I2[k2]][:, :, :, I2[k3]]
    ch_new.q3[...] = out


def resample_from_to(Lam, p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds, m_old: F.Mesh, a_old: A.Action,
                     a_new: A.Action, chi=None) -> F.Mesh:
    """New meshes at cutoff Λ and the action resampled onto them (Action.jl:483-548), on the host."""
    cuts = [[channel_cuts(ch.q3) for ch in v.channels] for v in a_old.Γ]
    m_new = new_meshes(Lam, p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds, m_old, a_old.Σ, cuts, chi)
    for k, w in enumerate(m_new.sigma):
        a_new.Σ[k] = get_sigma(w, m_old.sigma, a_old.Σ)
    for vo, vn in zip(a_old.Γ, a_new.Γ):
        _resample_channel(m_old.omega_s, m_old.nu_s, vo.ch_s, m_new.omega_s, m_new.nu_s, vn.ch_s)
        _resample_channel(m_old.omega_t, m_old.nu_t, vo.ch_t, m_new.omega_t, m_new.nu_t, vn.ch_t)
        _resample_channel(m_old.omega_s, m_old.nu_s, vo.ch_u, m_new.omega_s, m_new.nu_s, vn.ch_u)
    return m_new


def new_meshes(Lam, p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds, m_old: F.Mesh, Sigma, cuts,
               chi=None) -> F.Mesh:
    """The meshes of resample_from_to (Action.jl:499-544) from Σ, the cuts of every component's
    s, t, u channel (cuts[c][ch]) and χ."""
    s_lin = lins[1] * Lam
    Os_lin = lins[2] * Lam
    ns_lin = lins[3] * Lam
    Ot_lin = lins[2] * Lam
    nt_lin = lins[3] * Lam
    c_lin = lins[4] * Lam
    if Lam < lins[0]:
        s_lin = p_sigma[1] * m_old.sigma[int(np.argmax(np.abs(Sigma)))]
        Os, ns, Ot, nt = [], [], [], []
        for cs in cuts:
            o1, n1 = scan_cuts(Lam, p_Os, p_ns, m_old.omega_s, m_old.nu_s, cs[0])
            o2, n2 = scan_cuts(Lam, p_Os, p_ns, m_old.omega_s, m_old.nu_s, cs[2])
            Os.append(min(o1, o2))
            ns.append(min(n1, n2))
            o3, n3 = scan_cuts(Lam, p_Ot, p_nt, m_old.omega_t, m_old.nu_t, cs[1])
            Ot.append(o3)
            nt.append(n3)
        Os_lin, ns_lin, Ot_lin, nt_lin = min(Os), min(ns), min(Ot), min(nt)
        if chi is not None:
            lst = []
            for c in chi:
                row = int(np.unravel_index(int(np.argmax(np.abs(c).reshape(-1, order="F"))), c.shape, order="F")[0])
                lst.append(scan(m_old.chi, c[row, :], p_chi[0], p_chi[1], p_chi[2], p_chi[3] * Lam, p_chi[4] * Lam))
            c_lin = min(lst)
    b = max(Lam, bounds[0])
    sigma = F.get_mesh(s_lin, bounds[1] * b, m_old.num_sigma - 1, p_sigma[0]) * p_sigma[2]
    Os_m = F.get_mesh(Os_lin, bounds[2] * b, m_old.num_omega - 1, p_Os[0]) * p_Os[5]
    ns_m = F.get_mesh(ns_lin, bounds[3] * b, m_old.num_nu - 1, p_ns[0]) * p_ns[5]
    Ot_m = F.get_mesh(Ot_lin, bounds[2] * b, m_old.num_omega - 1, p_Ot[0]) * p_Ot[5]
    nt_m = F.get_mesh(nt_lin, bounds[3] * b, m_old.num_nu - 1, p_nt[0]) * p_nt[5]
    chi_m = F.get_mesh(c_lin, bounds[4] * b, m_old.num_chi - 1, p_chi[0]) * p_chi[5]
    return F.Mesh(m_old.num_sigma, m_old.num_omega, m_old.num_nu, m_old.num_chi, sigma, Os_m, ns_m, Ot_m, nt_m, chi_m)


# ---------------------------------------------------------------------------
# launch!
# ---------------------------------------------------------------------------
@dataclass
class FlowResult:
    Lam: list = field(default_factory=list)       # accepted cutoffs
    chi: list = field(default_factory=list)       # (Λ, χ mesh, χ[Ns, num_chi]) per measurement
    dLam: list = field(default_factory=list)
    err: list = field(default_factory=list)
    abs_max: list = field(default_factory=list)
    rejected: int = 0
    steps: list = field(default_factory=list)     # (Λ before, dΛ taken) of every accepted step
    # wall seconds per part of the loop (the reference's timers, src/Flow/timers.jl): ODE steps on the
    # device, correlations, host transfers and resampling
    timers: dict = field(default_factory=lambda: {"steps": 0.0, "chi": 0.0, "transfer": 0.0, "resample": 0.0})
    rhs_evals: int = 0
    integrand_evals: int = 0
    parquet_iterations: int = 0
    parquet_residuals: list = field(default_factory=list)  # absolute residual of every parquet iteration
    seconds: float = 0.0
    finished: bool = False
    reason: str = ""
    mesh: F.Mesh | None = None
    action: A.Action | None = None


class _Output:
    """The ``f_obs`` / ``f_cp`` files of a run and the reference's measure (Launcher.jl:2-60):
    Σ and χ of every accepted step to ``*_obs`` (once per cutoff), checkpoints to ``*_cp`` when ``ct``
    hours have passed since the last one (``ct = 0``: now), or at every step within the last half
    hour of the wall time ``wt``."""

    def __init__(self, f: str, symmetry: str, wt: float, ct: float):
        self.obs, self.cp = f + "_obs", f + "_cp"
        self.symmetry, self.wt, self.ct = symmetry, wt, ct
        self.t0 = self.t = time.time()

    def exists(self) -> bool:
        return os.path.isfile(self.obs) and os.path.isfile(self.cp)

    def finished(self) -> bool:
        with hdf5.File(self.obs, "r") as o, hdf5.File(self.cp, "r") as c:
            return "finished" in o and "finished" in c

    def start(self, r, euclidean: bool) -> None:
        for p in (self.obs, self.cp):
            if os.path.isfile(p):
                os.remove(p)
        for p in (self.obs, self.cp):
            with hdf5.File(p, "cw") as fh:
                disk.save_lattice(fh, r, euclidean)

    def measure(self, Lam, dLam, m, a, chi, ct=None, wt=None) -> None:
        ct = self.ct if ct is None else ct
        wt = self.wt if wt is None else wt
        with hdf5.File(self.obs, "cw") as o, hdf5.File(self.cp, "cw") as c:
            if f"χ/{hdf5.julia_float_str(Lam)}" not in o:
                disk.save_self(o, Lam, m, a)
                disk.save_chi(o, Lam, self.symmetry, m, chi)
            now = time.time()
            h0 = (now - self.t0) / 3600.0
            has_cp = f"a/{hdf5.julia_float_str(Lam)}" in c
            if wt - h0 > 0.5:
                if (now - self.t) / 3600.0 >= ct:
                    if not has_cp:
                        disk.checkpoint(c, Lam, dLam, m, a)
                    self.t = now
            elif 0.1 < wt - h0 <= 0.5 and not has_cp:
                disk.checkpoint(c, Lam, dLam, m, a)

    def finish(self) -> None:
        for p in (self.obs, self.cp):
            with hdf5.File(p, "cw") as fh:
                if "finished" not in fh:
                    fh["finished"] = True


def launch(f: str, name: str, size: int, model: str, symmetry: str, J, *, A_rep: float = 0.0, S: float = 0.5,
           euclidean: bool = False, num_sigma: int = 25, num_omega: int = 15, num_nu: int = 10, num_chi: int = 10,
           p_sigma=F.DEFAULT_P_SIGMA, p_Os=F.DEFAULT_P_OMEGA, p_ns=F.DEFAULT_P_NU, p_Ot=F.DEFAULT_P_OMEGA,
           p_nt=F.DEFAULT_P_NU, p_chi=F.DEFAULT_P_CHI, lins=F.DEFAULT_LINS, bounds=F.DEFAULT_BOUNDS,
           max_iter: int = 50, min_eval: int = 10, max_eval: int = 100, sigma_tol=(1e-8, 1e-4),
           gamma_tol=(1e-8, 1e-4), chi_tol=(1e-8, 1e-4), parquet_tol=(1e-8, 1e-4), ode_tol=(1e-8, 1e-2),
           loops: int = 1, parquet: bool = True, sigma_corr: bool = True, initial: float = 5.0,
           final: float = 0.05, bmin: float = 1e-4, bmax: float = 0.1, cps=(), overwrite: bool = True,
           wt: float = 23.5, ct: float = 1.0, precision: str = "mixed", device: int = 0, measure=None,
           correlations: bool = True, warm_start=None, verbose: bool = False, schedule=None) -> FlowResult:
    """Run the FRG flow from ``initial`` to ``final`` (launch!, Launcher.jl:565-773).

    After every accepted step the static correlations χ of the new state are
    computed on the GPU (``correlations``; measure, Launcher.jl:2-60), the flow
    stops when the dominant on-site χ falls by more than 0.5 %, and χ steers
    the χ mesh of the resampling.  ``measure(Λ, dΛ, m, a, ctx)`` is an extra
    user callback after every accepted step; returning False stops the flow.

    With a non-empty ``f`` the run writes the reference's ``f_obs`` / ``f_cp``
    HDF5 files; ``overwrite = False`` resumes from the last checkpoint of
    existing files (Launcher.jl:704-760).  ``warm_start`` (a fitted
    ``warmstart.ParquetWarmStart``) starts the parquet iteration from its
    predicted vertex instead of the bare couplings.  ``schedule`` (another
    run's ``steps``) replays that run's accepted (Λ, dΛ) sequence instead of
    choosing step sizes: the two runs then differ by their arithmetic only.
    """
    t0 = time.perf_counter()
    if symmetry not in A.SYMMETRIES:
        raise ValueError(f"Symmetry {symmetry} unknown. Valid arguments are su2 and u1-dm.")
    res = FlowResult()
    out = _Output(f, symmetry, wt, ct) if f else None
    p = (p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds)
    if overwrite or out is None:
        flat = [float(x) for j in J for x in j] + [float(A_rep)]
        nrm = math.sqrt(sum(x * x for x in flat))
        Jn = [[float(x) / nrm for x in j] for j in J]
        A_n = A_rep / nrm
        lat = L.get_lattice(name, size, euclidean=euclidean)
        r = L.get_reduced_lattice(model, Jn, lat)
        m = F.initial_mesh(initial, num_sigma, num_omega, num_nu, num_chi, p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi,
                           lins, bounds)
        a = A.get_action_empty(symmetry, r, m, S=S)
        A.init_action(lat, r, a)
        A.add_repulsion(A_n, a)
        if out:
            out.start(r, euclidean)
        Li, dLi = initial, bmax * initial
    else:
        if not out.exists():
            res.reason = "found no existing output files"
            return res
        if out.finished():
            res.finished = True
            res.reason = "calculation has finished already"
            return res
        with hdf5.File(out.cp, "r") as c:
            lat, r = disk.read_lattice(c)
            Li, dLi, m_old, a_inter = disk.read_checkpoint(c, 0.0)
        with hdf5.File(out.obs, "r") as o:
            chi = disk.read_chi_all(o, Li, verbose=False)[1]
        a = a_inter.copy()
        m = resample_from_to(Li, *p, m_old, a_inter, a, chi)
        parquet = False
    ctx = FlowContext(r, m, symmetry=symmetry, S=S, precision=precision, device=device)
    try:
        if parquet:
            if warm_start is not None:
                from .warmstart import coupling_features, vertex_mask

                mask = vertex_mask(a)
                a.buf[mask] = warm_start.predict(coupling_features(J))
            res.parquet_iterations = launch_parquet(ctx, r, m, a, initial, max_iter, min_eval, max_eval, sigma_tol,
                                                    gamma_tol, parquet_tol, verbose=verbose,
                                                    residuals=res.parquet_residuals)
            if out:
                # the parquet solution is measured and checkpointed (parquet.jl:96-98)
                ctx.upload(_capi.SLOT_NEXT, a)
                chi0 = ctx.chi_slot(initial, _capi.SLOT_NEXT, m.chi, chi_tol)
                out.measure(initial, dLi, m, a, chi0, ct=0.0, wt=math.inf)
        _flow(ctx, r, m, a, res, loops=loops, sigma_corr=sigma_corr and loops >= 3, Li=Li, Lf=final,
              dLi=dLi, bmin=bmin, bmax=bmax, min_eval=min_eval, max_eval=max_eval, sigma_tol=sigma_tol,
              gamma_tol=gamma_tol, ode_tol=ode_tol, p=p, cps=list(cps), measure=measure,
              chi_tol=chi_tol if correlations or out else None, out=out, verbose=verbose, schedule=schedule)
        if out:
            out.finish()
    finally:
        ctx.close()
    res.seconds = time.perf_counter() - t0
    return res


def _flow(ctx: FlowContext, r, m, a, res: FlowResult, *, loops, sigma_corr, Li, Lf, dLi, bmin, bmax, min_eval,
          max_eval, sigma_tol, gamma_tol, ode_tol, p, cps, measure, chi_tol=None, out=None, verbose=False,
          schedule=None):
    """Bogacki-Shampine loop of launch_1l!/2l!/ml! (launcher_1l.jl:56-198) with device stages.

    ``schedule`` (the ``steps`` of another run: (Λ, dΛ) of each accepted step) replays that run's
    step sequence: every step takes the scheduled dΛ and is accepted, and the flow ends after the
    last one; the measurements are those of this run's arithmetic on the other run's cutoffs."""
    p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds = p
    Lam, dLam = Li, dLi
    step_i = 0
    cps = sorted(set(list(cps) + [Li, Lf]), reverse=True)
    for c in cps:
        if c < Lam:
            dLam = min(dLam, 0.85 * (Lam - c))
            break
    if schedule is not None:
        if not schedule:
            return
        dLam = schedule[0][1]
    ctx.upload(_capi.SLOT_A, a)
    a_next = A.Action.empty_like(a)
    a_new = A.Action.empty_like(a)
    ncomp = 1 if ctx.symmetry == "su2" else 3
    chi = [np.zeros((r.num_sites, m.num_chi), order="F") for _ in range(ncomp)]  # get_χ_empty

    def measure_chi(ct=None):
        # compute_χ! on the new state and the monotonicity test of measure (Launcher.jl:23-35):
        # the static on-site value of the component with the largest |χ|; observables and
        # checkpoints go to the output files
        nonlocal chi
        chi_prev = chi
        t0 = time.perf_counter()
        got = ctx.chi_slot(Lam, _capi.SLOT_NEXT, m.chi, chi_tol)
        res.timers["chi"] += time.perf_counter() - t0
        chi = [got] if ncomp == 1 else got
        res.chi.append((Lam, np.array(m.chi), got))
        if out:
            t1 = time.perf_counter()
            out.measure(Lam, dLam, m, a_next, chi, ct=ct)
            res.timers["files"] = res.timers.get("files", 0.0) + time.perf_counter() - t1
        idx = int(np.argmax([np.max(np.abs(c)) for c in chi]))
        with np.errstate(divide="ignore", invalid="ignore"):
            return bool(np.float64(chi[idx][0, 0]) / np.float64(chi_prev[idx][0, 0]) >= 0.995)

    while Lam > Lf:
        eval_ = get_eval(Lam, min_eval, max_eval)
        t0 = time.perf_counter()
        try:
            err, amax = ctx.bs_step(Lam, dLam, eval_, loops=loops, gamma_tol=gamma_tol, sigma_tol=sigma_tol,
                                    sigma_corr=sigma_corr, ode_tol=ode_tol)
        except _capi.PffrgError as e:
            if e.code != _capi.PFFRG_E_NONFINITE:
                raise
            # a stage derivative with NaN or infinite entries: stop as the reference's sanity checks
            # stop an unstable integration (launcher_1l.jl:125-128), with the state of the last step
            res.reason = "right-hand side is not finite"
            break
        t_step = time.perf_counter() - t0
        res.timers["steps"] += t_step
        res.rhs_evals += 4
        res.integrand_evals += ctx.last_integrand_evals
        if verbose:
            print(f"Λ = {Lam:.6g}  dΛ = {dLam:.3g}  eval = {eval_}  err = {err:.3g}  Γmax = {amax:.4g}  "
                  f"step {t_step:.3f} s  nodes {ctx.last_integrand_evals}", flush=True)
        if err >= 10.0:
            res.reason = "integration has become unstable"
            break

        def next_dlam(dl):
            dl = max(bmin, min(bmax * Lam, 0.85 * (1.0 / err) ** (1.0 / 3.0) * dl))
            lower = [c for c in cps if c - Lam < 0.0]
            lam_cp = lower[0] if lower else 0.0
            return min(dl, Lam - lam_cp)

        if err <= 1.0 or dLam <= bmin or schedule is not None:
            res.steps.append((Lam, dLam))
            Lam -= dLam
            dLam = next_dlam(dLam)
            if schedule is not None:
                # replay: the next step of the given sequence, whatever the error ratio says
                step_i += 1
                if step_i >= len(schedule):
                    Lf = Lam
                else:
                    dLam = schedule[step_i][1]
            res.Lam.append(Lam)
            res.dLam.append(dLam)
            res.err.append(err)
            res.abs_max.append(amax)
            if measure or out:
                # the callback and the checkpoints see the accepted state on the host
                t0 = time.perf_counter()
                ctx.download(_capi.SLOT_NEXT, a_next)
                res.timers["transfer"] += time.perf_counter() - t0
            if amax >= 1000.0:
                res.reason = "vertex has diverged"
                if chi_tol is not None:
                    measure_chi(ct=0.0)
                if measure:
                    measure(Lam, dLam, m, a_next, ctx)
                break
            # at a requested checkpoint the measurement checkpoints now (launcher_1l.jl:154-167)
            at_cp = any(math.isclose(Lam, c, rel_tol=1.49e-8) for c in cps)
            monotone = measure_chi(ct=0.0 if at_cp else None) if chi_tol is not None else True
            if measure and measure(Lam, dLam, m, a_next, ctx) is False:
                monotone = False
            if not monotone:
                res.reason = "flowing correlations show non-monotonicity"
                if out:
                    out.measure(Lam, dLam, m, a_next, chi, ct=0.0)
                break
            # new meshes and the resampled state (launcher_1l.jl:177): the scans read Σ and the cuts
            # through each channel's maximum from the device, the meshes are built on the host and
            # the action is interpolated onto them on the device
            t0 = time.perf_counter()
            sig, _, cuts = ctx.scan_cuts(_capi.SLOT_NEXT)
            C = len(a.Γ)
            cut_lists = [[cuts[3 * c + ch] for ch in range(3)] for c in range(C)]
            m = new_meshes(Lam, p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds, m, sig, cut_lists,
                           chi if chi_tol is not None else None)
            ctx.resample(_capi.SLOT_NEXT, _capi.SLOT_A, m)
            res.timers["resample"] += time.perf_counter() - t0
        else:
            dLam = next_dlam(dLam)
            res.rejected += 1
    else:
        res.finished = True
    res.mesh = m
    if res.Lam:
        ctx.download(_capi.SLOT_A, a_new)
        res.action = a_new
    else:
        res.action = a


def launch_parquet(ctx: FlowContext, r, m, a: A.Action, Lam: float, max_iter: int, min_eval: int, max_eval: int,
                   sigma_tol, gamma_tol, parquet_tol, beta=None, verbose: bool = False, residuals=None) -> int:
    """Parquet fixed point of the SDE and the BSEs at cutoff Λ (parquet.jl:1-100); returns iterations.

    The iteration runs on the device (``pffrg_parquet``): ``a`` is uploaded once, the SDE / BSE
    evaluations, the residuals and the damping stay on the device, and the converged iterate is
    downloaded into ``a`` at the end."""
    beta = min(Lam, 1.0) if beta is None else beta
    eval_ = get_eval(Lam, min_eval, max_eval)
    ctx.upload(_capi.SLOT_A, a)
    it, abs_err, rel_err, hist = ctx.parquet(Lam, eval_, gamma_tol, sigma_tol, parquet_tol, beta, max_iter,
                                             history=True)
    ctx.download(_capi.SLOT_A, a)
    if residuals is not None:
        residuals.extend(float(x) for x in hist)
    if verbose:
        print(f"parquet: {it} iterations, residual {abs_err:.3e} (relative {rel_err:.3e})", flush=True)
    return it
