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
