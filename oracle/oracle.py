"""ctypes binding of the CPU FP64 oracle (liboracle_pffrg.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
legs load it as the checker and the CPU baseline.  The product path never
imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle_pffrg.so"

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


class _Problem(ctypes.Structure):
    _fields_ = [
        ("num_sites", ctypes.c_int64),
        ("exchange", _i64p),
        ("mult", _i64p),
        ("overlap_offsets", _i64p),
        ("overlap_rows", _i64p),
        ("num_sigma", ctypes.c_int64),
        ("num_omega", ctypes.c_int64),
        ("num_nu", ctypes.c_int64),
        ("sigma", _f64p),
        ("omega_s", _f64p),
        ("nu_s", _f64p),
        ("omega_t", _f64p),
        ("nu_t", _f64p),
        ("symmetry", ctypes.c_int32),
        ("S", ctypes.c_double),
        ("num_threads", ctypes.c_int32),
        ("task_stride", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("integrand_evals", ctypes.c_int64),
        ("gathered_values", ctypes.c_int64),
        ("overlap_terms", ctypes.c_int64),
        ("sigma_evals", ctypes.c_int64),
        ("reevals", ctypes.c_int64),
        ("level_hist", ctypes.c_int64 * 24),
    ]


def build(force: bool = False) -> Path:
    """Compile the oracle with g++ (OpenMP, FP contraction off for cross-machine determinism)."""
    src = HERE / "pffrg_oracle.cpp"
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= src.stat().st_mtime:
        return LIB_PATH
    LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", str(LIB_PATH), str(src)]
    subprocess.run(cmd, check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.POINTER(_Problem)
        L.oracle_action_size.argtypes = [P]
        L.oracle_action_size.restype = ctypes.c_int64
        L.oracle_corrs.argtypes = [P, ctypes.c_int, ctypes.c_double, _f64p, _f64p, ctypes.c_double,
                                   ctypes.c_double, _f64p]
        L.oracle_dsigma.argtypes = [P, ctypes.c_double, _f64p, _f64p, ctypes.c_double, ctypes.c_double]
        L.oracle_dgamma.argtypes = [P, ctypes.c_int, ctypes.c_double, _f64p, _f64p, _f64p, _f64p, _f64p,
                                    _f64p, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double]
        L.oracle_bse.argtypes = [P, ctypes.c_double, _f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double]
        L.oracle_sde.argtypes = [P, ctypes.c_double, _f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.oracle_chi.argtypes = [P, ctypes.c_double, _f64p, _f64p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                 _f64p]
        L.oracle_symmetrize.argtypes = [P, _f64p]
        L.oracle_symmetrize_add_to.argtypes = [P, _f64p, _f64p]
        L.oracle_buffer_kernel.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.oracle_gamma_comp.argtypes = [P, _f64p, ctypes.c_int] + [ctypes.c_double] * 9 + [ctypes.c_int, _f64p]
        L.oracle_vertex_channel.argtypes = [P, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double, _f64p]
        L.oracle_get_sigma.argtypes = [P, _f64p, ctypes.c_double]
        L.oracle_get_sigma.restype = ctypes.c_double
        L.oracle_test_integrators.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_int, _f64p]
        L.oracle_test_quadgk.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double]
        L.oracle_test_quadgk.restype = ctypes.c_double
        L.oracle_test_hcubature.argtypes = [ctypes.c_int] + [ctypes.c_double] * 6
        L.oracle_test_hcubature.restype = ctypes.c_double
        L.oracle_last_stats.argtypes = [ctypes.POINTER(Stats)]
        _lib = L
    return _lib


def _f(x: np.ndarray):
    assert x.dtype == np.float64 and x.flags.c_contiguous
    return x.ctypes.data_as(_f64p)


def _opt(x):
    return _f(x) if x is not None else None


class Problem:
    """Lattice tables + meshes + model, kept alive for the oracle calls."""

    def __init__(self, r, m, symmetry: str = "su2", S: float = 0.5, num_threads: int = 0, task_stride: int = 1):
        offs, rows = r.overlap_csr()
        self._keep = dict(
            exchange=np.ascontiguousarray(r.exchange, dtype=np.int64),
            mult=np.ascontiguousarray(r.mult, dtype=np.int64),
            offs=np.ascontiguousarray(offs, dtype=np.int64),
            rows=np.ascontiguousarray(rows.reshape(-1), dtype=np.int64),
            sigma=np.ascontiguousarray(m.sigma, dtype=np.float64),
            omega_s=np.ascontiguousarray(m.omega_s, dtype=np.float64),
            nu_s=np.ascontiguousarray(m.nu_s, dtype=np.float64),
            omega_t=np.ascontiguousarray(m.omega_t, dtype=np.float64),
            nu_t=np.ascontiguousarray(m.nu_t, dtype=np.float64),
        )
        k = self._keep
        ip = lambda x: x.ctypes.data_as(_i64p)  # noqa: E731
        self.s = _Problem(r.num_sites, ip(k["exchange"]), ip(k["mult"]), ip(k["offs"]), ip(k["rows"]),
                          m.num_sigma, m.num_omega, m.num_nu, _f(k["sigma"]), _f(k["omega_s"]),
                          _f(k["nu_s"]), _f(k["omega_t"]), _f(k["nu_t"]), 0 if symmetry == "su2" else 1,
                          float(S), int(num_threads), int(task_stride))
        self.ref = ctypes.byref(self.s)

    @property
    def action_size(self) -> int:
        return int(lib().oracle_action_size(self.ref))


def stats() -> dict:
    st = Stats()
    lib().oracle_last_stats(ctypes.byref(st))
    out = {k: int(getattr(st, k)) for k, _ in Stats._fields_ if k != "level_hist"}
    out["level_hist"] = [int(x) for x in st.level_hist]
    return out


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with code {rc}")


def corrs(P: Problem, kind: int, Lam: float, a: np.ndarray, da: np.ndarray | None, atol: float,
          rtol: float) -> np.ndarray:
    out = np.zeros(6 * int(P.s.num_omega))
    _check(lib().oracle_corrs(P.ref, kind, Lam, _f(a), _opt(da), atol, rtol, _f(out)), "corrs")
    return out.reshape((2, 3, int(P.s.num_omega)), order="F")


def dsigma(P: Problem, Lam: float, a: np.ndarray, da: np.ndarray, atol=1e-8, rtol=1e-4) -> None:
    _check(lib().oracle_dsigma(P.ref, Lam, _f(a), _f(da), atol, rtol), "dsigma")


def dgamma(P: Problem, loops: int, Lam: float, a: np.ndarray, da: np.ndarray, eval_: int, gtol=(1e-8, 1e-4),
           sigma_corr: bool = False, stol=(1e-8, 1e-4), scratch=None) -> dict:
    n = a.size
    if scratch is None:
        scratch = [np.zeros(n) for _ in range(4)]
    _check(lib().oracle_dgamma(P.ref, loops, Lam, _f(a), _f(da), *[_f(s) for s in scratch], eval_, gtol[0],
                               gtol[1], int(sigma_corr), stol[0], stol[1]), "dgamma")
    return stats()


def sde(P: Problem, Lam: float, a1: np.ndarray, a2: np.ndarray, eval_: int, gtol=(1e-8, 1e-4),
        stol=(1e-8, 1e-4)) -> np.ndarray:
    c = np.zeros(6 * int(P.s.num_omega))
    _check(lib().oracle_sde(P.ref, Lam, _f(a1), _f(a2), _f(c), eval_, gtol[0], gtol[1], stol[0], stol[1]), "sde")
    return c


def bse(P: Problem, Lam: float, a1: np.ndarray, a2: np.ndarray, corrs_buf: np.ndarray, eval_: int,
        gtol=(1e-8, 1e-4)) -> None:
    _check(lib().oracle_bse(P.ref, Lam, _f(a1), _f(a2), _f(corrs_buf), eval_, gtol[0], gtol[1]), "bse")


def _masks(P: Problem):
    """(vertex mask without bare, q3 mask) of a packed action of P's layout."""
    ns, nsig, no, nn = (int(P.s.num_sites), int(P.s.num_sigma), int(P.s.num_omega), int(P.s.num_nu))
    ncomp = 2 if int(P.s.symmetry) == 0 else 6
    k1, k2, k3 = ns * no, ns * no * nn, ns * no * nn * nn
    chan = k1 + 2 * k2 + k3
    size = nsig + ncomp * (ns + 3 * chan)
    gm = np.zeros(size, dtype=bool)
    q3 = np.zeros(size, dtype=bool)
    for c in range(ncomp):
        base = nsig + c * (ns + 3 * chan) + ns
        gm[base:base + 3 * chan] = True
        for ch in range(3):
            o = base + ch * chan + k1 + 2 * k2
            q3[o:o + k3] = True
    return gm, q3


def parquet(P: Problem, Lam: float, a: np.ndarray, eval_: int, gtol=(1e-8, 1e-4), stol=(1e-8, 1e-4),
            ptol=(1e-8, 1e-4), beta=None, max_iter: int = 50):
    """launch_parquet!'s fixed point (src/Launcher/parquet.jl:43-80) with the oracle's compute_Σ! and
    compute_Γ!: a (packed) is replaced by the iterate; returns (iterations, abs residual, rel residual)."""
    beta = min(Lam, 1.0) if beta is None else beta
    gm, q3 = _masks(P)
    nsig = int(P.s.num_sigma)
    ap = np.zeros_like(a)
    abs_err = rel_err = np.inf
    count = 1
    while abs_err >= ptol[0] and rel_err >= ptol[1] and count <= max_iter:
        s_abs = s_rel = np.inf
        s_count = 1
        corrs_buf = None
        while s_abs >= ptol[0] and s_rel >= ptol[1] and s_count <= max_iter:
            corrs_buf = sde(P, Lam, a, ap, eval_, gtol, stol)
            s_abs = float(np.max(np.abs(ap[:nsig] - a[:nsig])))
            s_rel = s_abs / max(float(np.max(np.abs(a[:nsig]))), float(np.max(np.abs(ap[:nsig]))))
            a[:nsig] = (1.0 - beta) * a[:nsig] + beta * ap[:nsig]
            s_count += 1
        bse(P, Lam, a, ap, corrs_buf, eval_, gtol)
        abs_err = float(np.max(np.abs(ap[q3] - a[q3])))
        rel_err = abs_err / max(float(np.max(np.abs(a[q3]))), float(np.max(np.abs(ap[q3]))))
        a[gm] = (1.0 - beta) * a[gm] + beta * ap[gm]
        count += 1
    return count - 1, abs_err, rel_err


def chi(P: Problem, Lam: float, a: np.ndarray, chi_mesh: np.ndarray, tol=(1e-8, 1e-4)):
    """compute_χ!: χ[site, w] on the χ mesh (Fortran-ordered [Ns, num_chi]); for u1-dm the list
    [χxx, χzz, χxy] of such arrays (correlation_u1_dm.jl:152-190)."""
    cm = np.ascontiguousarray(chi_mesh, dtype=np.float64)
    ncomp = 1 if int(P.s.symmetry) == 0 else 3
    ns = int(P.s.num_sites)
    out = np.zeros(ncomp * ns * len(cm))
    _check(lib().oracle_chi(P.ref, Lam, _f(a), _f(cm), len(cm), tol[0], tol[1], _f(out)), "chi")
    mats = [out[k * ns * len(cm):(k + 1) * ns * len(cm)].reshape((ns, len(cm)), order="F") for k in range(ncomp)]
    return mats[0] if ncomp == 1 else mats


def symmetrize(P: Problem, a: np.ndarray) -> None:
    _check(lib().oracle_symmetrize(P.ref, _f(a)), "symmetrize")


def symmetrize_add_to(P: Problem, a_l: np.ndarray, a: np.ndarray) -> None:
    _check(lib().oracle_symmetrize_add_to(P.ref, _f(a_l), _f(a)), "symmetrize_add_to")


def buffer_kernel(P: Problem, ch: int, w: float, v: float, vp: float) -> int:
    return int(lib().oracle_buffer_kernel(P.ref, ch, w, v, vp))


def gamma_comp(P: Problem, a: np.ndarray, comp: int, s_args, t_args, u_args, mask: int = 7) -> np.ndarray:
    out = np.zeros(int(P.s.num_sites))
    _check(lib().oracle_gamma_comp(P.ref, _f(a), comp, *s_args, *t_args, *u_args, mask, _f(out)), "gamma_comp")
    return out


def vertex_channel(P: Problem, a: np.ndarray, comp: int, ch: int, w: float, v: float, vp: float) -> np.ndarray:
    out = np.zeros(int(P.s.num_sites))
    _check(lib().oracle_vertex_channel(P.ref, _f(a), comp, ch, w, v, vp, _f(out)), "vertex_channel")
    return out


def get_sigma(P: Problem, a: np.ndarray, w: float) -> float:
    return float(lib().oracle_get_sigma(P.ref, _f(a), w))


def test_integrators(n: int, a: float, b: float, eval_: int, atol: float, rtol: float, log_mesh: bool) -> np.ndarray:
    out = np.zeros(n)
    _check(lib().oracle_test_integrators(n, a, b, eval_, atol, rtol, int(log_mesh), _f(out)), "integrators")
    return out


def test_quadgk(power: int, a: float, b: float, atol: float, rtol: float) -> float:
    return float(lib().oracle_test_quadgk(power, a, b, atol, rtol))


def num_threads() -> int:
    return os.cpu_count() or 1


def test_hcubature(which: int, x0: float, x1: float, y0: float, y1: float, atol: float, rtol: float) -> float:
    return float(lib().oracle_test_hcubature(which, x0, x1, y0, y1, atol, rtol))


# ---------------------------------------------------------------------------
# Mesh scans and resampling, restated in numpy from the reference (independent of the package's
# own host and device code, which the tests check against it)
# ---------------------------------------------------------------------------
def get_mesh(linear: float, upper: float, num: int, p: float) -> np.ndarray:
    """get_mesh (src/Frequency/mesh.jl:86-122): 0, num_lin linear points of width linear / num_lin,
    then num - num_lin points growing by (upper / linear)^(1 / num_log)."""
    assert linear > 0.0 and upper > 0.0 and linear < upper
    num_lin = int(np.ceil(p * num))
    num_log = num - num_lin
    assert num_log > 0
    h = linear / num_lin
    xi = (upper / linear) ** (1.0 / num_log)
    mesh = np.zeros(num + 1)
    for i in range(1, num_lin + 1):
        mesh[i] = i * h
    for i in range(1, num_log + 1):
        mesh[num_lin + i] = xi ** i * linear
    return mesh


def get_param(val: float, lst: np.ndarray):
    """get_indices + get_param (src/Frequency/param.jl:25-87), 0-based indices: the neighbours of val in
    the sorted list (both the last entry at or beyond it) and the linear weights."""
    n = len(lst)
    if val >= lst[n - 1]:
        lo = hi = n - 1
    else:
        i = 0
        while val > lst[i]:
            i += 1
        lo = hi = i
        if val < lst[i]:
            lo -= 1
    if lo < hi:
        d = 1.0 / (lst[hi] - lst[lo])
        return lo, hi, d * (lst[hi] - val), d * (val - lst[lo])
    return lo, hi, 1.0, 0.0


def _sign(x: float) -> float:
    return 0.0 if x == 0.0 else (np.nan if x != x else (1.0 if x > 0.0 else -1.0))


def scan(x: np.ndarray, y: np.ndarray, p0: float, p1: float, p2: float, p3: float, p4: float) -> float:
    """scan (src/Action/Action.jl:369-446): the linear extent of a new mesh from a cut y(x)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(x)
    num_lin = int(np.ceil(p0 * (n - 1)))
    with np.errstate(divide="ignore", invalid="ignore"):
        # a) the first peak at a finite frequency and where the cut has fallen to 75 % of it
        da = np.inf
        idx = 0
        slope = np.float64(y[1] - y[0]) / np.float64(x[1] - x[0])
        for i in range(1, n - 1):
            s = np.float64(y[i + 1] - y[i]) / np.float64(x[i + 1] - x[i])
            if _sign(s) != _sign(slope):
                idx = i
                break
            slope = s
        if idx > 0:
            for i in range(idx + 1, n):
                if abs(np.float64(y[i]) / np.float64(y[idx])) <= 0.75:
                    da = max(x[i], num_lin * x[idx] / np.ceil(0.5 * num_lin))
                    break
        # b) a finite value at the origin: the relative step to the first frequency within (p1, p2)
        db = num_lin * x[1]
        if abs(y[0]) / np.max(np.abs(y)) > 1e-2:
            D = abs(y[1] - y[0]) / max(abs(y[1]), abs(y[0]))
            while not (p1 < D < p2):
                if D >= p2:
                    db *= 0.98
                elif D <= p1:
                    db *= 1.02
                if db >= x[-1]:
                    break
                xp = get_mesh(db, x[-1], n - 1, p0)
                yp = np.empty_like(y)
                for i in range(n):
                    lo, hi, wl, wh = get_param(xp[i], x)
                    yp[i] = wl * y[lo] + wh * y[hi]
                D = abs(yp[1] - yp[0]) / max(abs(yp[1]), abs(yp[0]))
    return min(max(num_lin * p3, min(da, db)), p4)


def scan_channel(Lam: float, p_O, p_n, O: np.ndarray, nu: np.ndarray, q3: np.ndarray):
    """scan_channel (src/Action/Action.jl:449-480): scans of the cuts through max |q3| (q3[site, Ω, ν, ν'],
    the first maximum in column-major order)."""
    s, w, v, vp = np.unravel_index(int(np.argmax(np.abs(q3).reshape(-1, order="F"))), q3.shape, order="F")
    cut_O = q3[s, :, v, vp]
    cut_1 = np.array([q3[s, w, k, k] - q3[s, w, -1, -1] for k in range(len(nu))])
    cut_2 = np.array([q3[s, w, k, vp] - q3[s, w, -1, vp] for k in range(len(nu))])
    cut_3 = np.array([q3[s, w, v, k] - q3[s, w, v, -1] for k in range(len(nu))])
    O_lin = scan(O, cut_O, p_O[0], p_O[1], p_O[2], p_O[3] * Lam, p_O[4] * Lam)
    n_lin = min(scan(nu, c, p_n[0], p_n[1], p_n[2], p_n[3] * Lam, p_n[4] * Lam) for c in (cut_1, cut_2, cut_3))
    return O_lin, n_lin


def sigma_at(w: float, sigma_mesh: np.ndarray, Sigma: np.ndarray) -> float:
    """get_Σ (src/Action/Action.jl:8-26): odd in w, interpolated on the mesh, 1 / w beyond it."""
    if abs(w) <= sigma_mesh[-1]:
        lo, hi, wl, wh = get_param(abs(w), sigma_mesh)
        return _sign(w) * (wl * Sigma[lo] + wh * Sigma[hi])
    return sigma_mesh[-1] * Sigma[-1] / w


def resample_channel(O_old, n_old, ch_old: dict, O_new, n_new, ch_new: dict) -> None:
    """resample_from_to! of a channel (src/Action/channel.jl:416-466): q1, q2_1, q2_2, q3 at the new
    meshes by linear, bilinear and trilinear interpolation in the reference's term order."""
    q1, q21, q22, q3 = (ch_old[k] for k in ("q1", "q2_1", "q2_2", "q3"))
    pO = [get_param(x, O_old) for x in O_new]
    pn = [get_param(x, n_old) for x in n_new]
    for w, (l1, h1, a1, b1) in enumerate(pO):
        ch_new["q1"][:, w] = a1 * q1[:, l1]
        ch_new["q1"][:, w] += b1 * q1[:, h1]
    for v, (l2, h2, a2, b2) in enumerate(pn):
        for w, (l1, h1, a1, b1) in enumerate(pO):
            for key, q in (("q2_1", q21), ("q2_2", q22)):
                val = a1 * a2 * q[:, l1, l2]
                val += b1 * a2 * q[:, h1, l2]
                val += a1 * b2 * q[:, l1, h2]
                val += b1 * b2 * q[:, h1, h2]
                ch_new[key][:, w, v] = val
    for vp, (l3, h3, a3, b3) in enumerate(pn):
        for v, (l2, h2, a2, b2) in enumerate(pn):
            for w, (l1, h1, a1, b1) in enumerate(pO):
                val = a1 * a2 * a3 * q3[:, l1, l2, l3]
                val += b1 * a2 * a3 * q3[:, h1, l2, l3]
                val += a1 * b2 * a3 * q3[:, l1, h2, l3]
                val += b1 * b2 * a3 * q3[:, h1, h2, l3]
                val += a1 * a2 * b3 * q3[:, l1, l2, h3]
                val += b1 * a2 * b3 * q3[:, h1, l2, h3]
                val += a1 * b2 * b3 * q3[:, l1, h2, h3]
                val += b1 * b2 * b3 * q3[:, h1, h2, h3]
                ch_new["q3"][:, w, v, vp] = val


def resample_from_to(Lam: float, p_sigma, p_Os, p_ns, p_Ot, p_nt, p_chi, lins, bounds, m_old: dict,
                     Sigma_old: np.ndarray, G_old: list, Sigma_new: np.ndarray, G_new: list, chi: list) -> dict:
    """resample_from_to (src/Action/Action.jl:483-548).  Meshes are dicts with sigma, omega_s, nu_s,
    omega_t, nu_t, chi; a vertex is a list of components, each {"s"|"t"|"u": {"q1", "q2_1", "q2_2",
    "q3": arrays [site, Ω(, ν(, ν'))]}}; chi is the list of χ[site, ω] arrays.  Fills Sigma_new and
    G_new and returns the new meshes."""
    s_lin, Os_lin, ns_lin = lins[1] * Lam, lins[2] * Lam, lins[3] * Lam
    Ot_lin, nt_lin, chi_lin = lins[2] * Lam, lins[3] * Lam, lins[4] * Lam
    if Lam < lins[0]:
        s_lin = p_sigma[1] * m_old["sigma"][int(np.argmax(np.abs(Sigma_old)))]
        Os_l, ns_l, Ot_l, nt_l = [], [], [], []
        for comp in G_old:
            a_s = scan_channel(Lam, p_Os, p_ns, m_old["omega_s"], m_old["nu_s"], comp["s"]["q3"])
            a_u = scan_channel(Lam, p_Os, p_ns, m_old["omega_s"], m_old["nu_s"], comp["u"]["q3"])
            Os_l.append(min(a_s[0], a_u[0]))
            ns_l.append(min(a_s[1], a_u[1]))
            a_t = scan_channel(Lam, p_Ot, p_nt, m_old["omega_t"], m_old["nu_t"], comp["t"]["q3"])
            Ot_l.append(a_t[0])
            nt_l.append(a_t[1])
        Os_lin, ns_lin, Ot_lin, nt_lin = min(Os_l), min(ns_l), min(Ot_l), min(nt_l)
        chi_l = []
        for c in chi:
            site = np.unravel_index(int(np.argmax(np.abs(c).reshape(-1, order="F"))), c.shape, order="F")[0]
            chi_l.append(scan(m_old["chi"], c[site, :], p_chi[0], p_chi[1], p_chi[2], p_chi[3] * Lam,
                              p_chi[4] * Lam))
        chi_lin = min(chi_l)
    up = max(Lam, bounds[0])
    m_new = {
        "sigma": get_mesh(s_lin, bounds[1] * up, len(m_old["sigma"]) - 1, p_sigma[0]) * p_sigma[2],
        "omega_s": get_mesh(Os_lin, bounds[2] * up, len(m_old["omega_s"]) - 1, p_Os[0]) * p_Os[5],
        "nu_s": get_mesh(ns_lin, bounds[3] * up, len(m_old["nu_s"]) - 1, p_ns[0]) * p_ns[5],
        "omega_t": get_mesh(Ot_lin, bounds[2] * up, len(m_old["omega_t"]) - 1, p_Ot[0]) * p_Ot[5],
        "nu_t": get_mesh(nt_lin, bounds[3] * up, len(m_old["nu_t"]) - 1, p_nt[0]) * p_nt[5],
        "chi": get_mesh(chi_lin, bounds[4] * up, len(m_old["chi"]) - 1, p_chi[0]) * p_chi[5],
    }
    for k, w in enumerate(m_new["sigma"]):
        Sigma_new[k] = sigma_at(w, m_old["sigma"], Sigma_old)
    for old, new in zip(G_old, G_new):
        resample_channel(m_old["omega_s"], m_old["nu_s"], old["s"], m_new["omega_s"], m_new["nu_s"], new["s"])
        resample_channel(m_old["omega_t"], m_old["nu_t"], old["t"], m_new["omega_t"], m_new["nu_t"], new["t"])
        resample_channel(m_old["omega_s"], m_old["nu_s"], old["u"], m_new["omega_s"], m_new["nu_s"], new["u"])
    return m_new
