"""ctypes binding of libpffrg_gpu.so (structs mirror include/pffrg_gpu.h).

This is the product path: there is no CPU fallback.  If the library has not
been built, or no CUDA device is usable, the calls raise.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libpffrg_gpu.so"

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)

PFFRG_FP64 = 0
PFFRG_MIXED = 1
PFFRG_SU2 = 0
PFFRG_U1_DM = 1
PFFRG_E_ARGS, PFFRG_E_CUDA, PFFRG_E_LIMIT, PFFRG_E_NONFINITE = 1, 2, 3, 4
SLOT_A, SLOT_DA, SLOT_INTER, SLOT_ERR, SLOT_NEXT = range(5)

EXPORTED = [
    "pffrg_create", "pffrg_destroy", "pffrg_last_error", "pffrg_set_mesh", "pffrg_set_precision",
    "pffrg_dsigma", "pffrg_dgamma", "pffrg_sde", "pffrg_bse", "pffrg_action_size", "pffrg_upload",
    "pffrg_download", "pffrg_rhs", "pffrg_bs_step", "pffrg_accept", "pffrg_last_integrand_evals",
    "pffrg_host_alloc", "pffrg_host_free", "pffrg_set_timing", "pffrg_read_stats", "pffrg_chi", "pffrg_chi_slot",
    "pffrg_set_async_waves", "pffrg_set_team_shape", "pffrg_autotune_team_shape", "pffrg_set_fp64_handoff",
    "pffrg_set_chi_cluster", "pffrg_set_chi_integrand",
    "pffrg_scan_cuts",
    "pffrg_resample", "pffrg_set_capacities", "pffrg_set_overlap_staging",
    "pffrg_parquet",
]


class Stats(ctypes.Structure):
    _fields_ = [("integrand_evals", ctypes.c_int64), ("algorithmic_values", ctypes.c_int64),
                ("pass_ms", ctypes.c_double), ("rhs_ms", ctypes.c_double), ("pass_launches", ctypes.c_int64),
                ("launches", ctypes.c_int64), ("chi_evals", ctypes.c_int64), ("chi_regions_max", ctypes.c_int64),
                ("chi_rounds", ctypes.c_int64), ("chi_rounds_max", ctypes.c_int64)]


class LatticeView(ctypes.Structure):
    _fields_ = [("num_sites", ctypes.c_int64), ("exchange", _i64p), ("mult", _i64p),
                ("overlap_offsets", _i64p), ("overlap_rows", _i64p)]


class MeshView(ctypes.Structure):
    _fields_ = [("num_sigma", ctypes.c_int64), ("num_omega", ctypes.c_int64), ("num_nu", ctypes.c_int64),
                ("sigma", _f64p), ("omega_s", _f64p), ("nu_s", _f64p), ("omega_t", _f64p), ("nu_t", _f64p)]


class ActionView(ctypes.Structure):
    _fields_ = [("sigma", _f64p), ("bare", _f64p * 6), ("q1", (_f64p * 3) * 6), ("q2_1", (_f64p * 3) * 6),
                ("q2_2", (_f64p * 3) * 6), ("q3", (_f64p * 3) * 6)]


class PffrgError(RuntimeError):
    """A nonzero status of the library; ``code`` is the PFFRG_E_* value (0 when unknown)."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


_lib = None


def load():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise PffrgError(f"{LIB_PATH} not found: build it with __graft_entry__.build() "
                         "(there is no CPU fallback)")
    L = ctypes.CDLL(str(LIB_PATH))
    vp = ctypes.c_void_p
    L.pffrg_create.argtypes = [ctypes.POINTER(LatticeView), ctypes.POINTER(MeshView), ctypes.c_int,
                               ctypes.c_double, ctypes.c_int, ctypes.c_int]
    L.pffrg_create.restype = vp
    L.pffrg_destroy.argtypes = [vp]
    L.pffrg_last_error.argtypes = [vp]
    L.pffrg_last_error.restype = ctypes.c_char_p
    L.pffrg_set_mesh.argtypes = [vp, ctypes.POINTER(MeshView)]
    L.pffrg_set_precision.argtypes = [vp, ctypes.c_int]
    AV = ctypes.POINTER(ActionView)
    d = ctypes.c_double
    L.pffrg_dsigma.argtypes = [vp, d, AV, AV, d, d]
    L.pffrg_dgamma.argtypes = [vp, ctypes.c_int, d, AV, AV, ctypes.c_int, d, d, ctypes.c_int, d, d]
    L.pffrg_sde.argtypes = [vp, d, AV, AV, ctypes.c_int, d, d, d, d]
    L.pffrg_bse.argtypes = [vp, d, AV, AV, ctypes.c_int, d, d]
    L.pffrg_action_size.argtypes = [vp]
    L.pffrg_action_size.restype = ctypes.c_int64
    L.pffrg_upload.argtypes = [vp, ctypes.c_int, AV]
    L.pffrg_download.argtypes = [vp, ctypes.c_int, AV]
    L.pffrg_rhs.argtypes = [vp, ctypes.c_int, d, ctypes.c_int, ctypes.c_int, ctypes.c_int, d, d, d, d, ctypes.c_int]
    L.pffrg_bs_step.argtypes = [vp, ctypes.c_int, d, d, ctypes.c_int, d, d, d, d, ctypes.c_int, d, d,
                                ctypes.POINTER(d), ctypes.POINTER(d)]
    L.pffrg_accept.argtypes = [vp]
    dp = ctypes.POINTER(ctypes.c_double)
    L.pffrg_set_async_waves.argtypes = [vp, ctypes.c_int]
    L.pffrg_set_team_shape.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.pffrg_set_fp64_handoff.argtypes = [vp, ctypes.c_double]
    L.pffrg_set_chi_cluster.argtypes = [vp, ctypes.c_int64, ctypes.c_int]
    L.pffrg_set_chi_integrand.argtypes = [vp, ctypes.c_int]
    L.pffrg_set_capacities.argtypes = [vp, ctypes.c_int64, ctypes.c_int64]
    L.pffrg_parquet.argtypes = [vp, d, ctypes.c_int, d, d, d, d, d, d, d, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(d), ctypes.POINTER(d), ctypes.POINTER(d)]
    L.pffrg_set_overlap_staging.argtypes = [vp, ctypes.c_int]
    ip = ctypes.POINTER(ctypes.c_int)
    L.pffrg_autotune_team_shape.argtypes = [vp, ctypes.c_int, d, ctypes.c_int, ctypes.c_int, ctypes.c_int, d, d, d, d,
                                            ip, ip]
    L.pffrg_scan_cuts.argtypes = [vp, ctypes.c_int, dp, ctypes.POINTER(ctypes.c_int64), dp]
    L.pffrg_resample.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(MeshView)]
    L.pffrg_chi.argtypes = [vp, d, AV, dp, ctypes.c_int, d, d, dp]
    L.pffrg_chi_slot.argtypes = [vp, d, ctypes.c_int, dp, ctypes.c_int, d, d, dp]
    L.pffrg_last_integrand_evals.argtypes = [vp]
    L.pffrg_last_integrand_evals.restype = ctypes.c_int64
    L.pffrg_host_alloc.argtypes = [ctypes.c_int64]
    L.pffrg_host_alloc.restype = vp
    L.pffrg_host_free.argtypes = [vp]
    L.pffrg_set_timing.argtypes = [vp, ctypes.c_int]
    L.pffrg_read_stats.argtypes = [vp, ctypes.POINTER(Stats), ctypes.c_int]
    _lib = L
    return L


def lattice_view(r):
    """LatticeView of a ReducedLattice; the returned keep-alive tuple must outlive the view."""
    offs, rows = r.overlap_csr()
    keep = (np.ascontiguousarray(r.exchange, dtype=np.int64), np.ascontiguousarray(r.mult, dtype=np.int64),
            np.ascontiguousarray(offs, dtype=np.int64), np.ascontiguousarray(rows.reshape(-1), dtype=np.int64))
    v = LatticeView(r.num_sites, *[k.ctypes.data_as(_i64p) for k in keep])
    return v, keep


def mesh_view(m):
    keep = tuple(np.ascontiguousarray(x, dtype=np.float64) for x in (m.sigma, m.omega_s, m.nu_s, m.omega_t, m.nu_t))
    v = MeshView(m.num_sigma, m.num_omega, m.num_nu, *[k.ctypes.data_as(_f64p) for k in keep])
    return v, keep


def action_view(a) -> ActionView:
    """ActionView whose pointers alias the packed buffer of an Action (one copy per transfer)."""
    buf = a.buf
    base = buf.ctypes.data
    lay = a.layout
    v = ActionView()
    v.sigma = ctypes.cast(base, _f64p)
    for c in range(lay.num_comps):
        v.bare[c] = ctypes.cast(base + 8 * lay.bare_offset(c), _f64p)
        for ch in range(3):
            v.q1[c][ch] = ctypes.cast(base + 8 * lay.kernel_offset(c, ch, 0), _f64p)
            v.q2_1[c][ch] = ctypes.cast(base + 8 * lay.kernel_offset(c, ch, 1), _f64p)
            v.q2_2[c][ch] = ctypes.cast(base + 8 * lay.kernel_offset(c, ch, 2), _f64p)
            v.q3[c][ch] = ctypes.cast(base + 8 * lay.kernel_offset(c, ch, 3), _f64p)
    return v
