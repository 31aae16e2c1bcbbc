"""Flow right-hand side on the GPU, behind the reference's function names.

``FlowContext`` owns one libpffrg_gpu context (device memory, stream) for a
lattice, a mesh size and a symmetry.  Its methods mirror the reference's
internal API (same argument meaning, outputs written in place):

* compute_dΣ!       src/Flow/flow_self.jl:2-20           -> ``compute_dsigma``
* compute_dΓ_1l!    src/Flow/compute.jl:57-112            -> ``compute_dgamma(loops=1)``
* compute_dΓ_2l!    src/Flow/compute.jl:115-174           -> ``compute_dgamma(loops=2)``
* compute_dΓ_ml!    src/Flow/compute.jl:177-287 (+ compute_dΣ_corr!, flow_self.jl:23-51)
* compute_Σ!        src/Flow/SDE.jl:58-96                 -> ``compute_sigma_sde``
* compute_Γ!        src/Flow/compute.jl:2-54              -> ``compute_gamma_bse``

A nonzero status from the library raises ``PffrgError`` with the library's
message (the reference raises AssertionErrors on the same conditions).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .action import Action


class FlowContext:
    def __init__(self, r, m, symmetry: str = "su2", S: float = 0.5, precision: str = "fp64", device: int = 0):
        self.lib = _capi.load()
        self._lat, self._lat_keep = _capi.lattice_view(r)
        self._mesh, self._mesh_keep = _capi.mesh_view(m)
        self.symmetry = symmetry
        self.S = S
        prec = _capi.PFFRG_FP64 if precision == "fp64" else _capi.PFFRG_MIXED
        sym = _capi.PFFRG_SU2 if symmetry == "su2" else _capi.PFFRG_U1_DM
        h = self.lib.pffrg_create(ctypes.byref(self._lat), ctypes.byref(self._mesh), sym, S, prec, device)
        if not h:
            raise _capi.PffrgError(self.lib.pffrg_last_error(None).decode())
        self.h = h
        self.num_sites = r.num_sites
        self._layout = (m.num_sigma, m.num_omega, m.num_nu, 2 if symmetry == "su2" else 6)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pffrg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------
    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.pffrg_last_error(self.h).decode()
            raise _capi.PffrgError(f"{what}: code {rc}: {msg}", rc)

    @property
    def action_size(self) -> int:
        return int(self.lib.pffrg_action_size(self.h))

    def set_mesh(self, m) -> None:
        self._mesh, self._mesh_keep = _capi.mesh_view(m)
        self._check(self.lib.pffrg_set_mesh(self.h, ctypes.byref(self._mesh)), "set_mesh")

    def scan_cuts(self, slot: int):
        """(Σ, argmax[3 C], cuts[3 C, NΩ + 3 Nν]) of the action in `slot` for the mesh scans."""
        lay = self._layout
        sig = np.zeros(lay[0])
        arg = np.zeros(3 * lay[3], dtype=np.int64)
        cuts = np.zeros((3 * lay[3], lay[1] + 3 * lay[2]))
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.pffrg_scan_cuts(self.h, slot, sig.ctypes.data_as(dp),
                                             arg.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                             cuts.ctypes.data_as(dp)), "scan_cuts")
        return sig, arg, cuts

    def resample(self, src_slot: int, dst_slot: int, m) -> None:
        """Interpolate the action in src_slot onto the meshes m into dst_slot; m becomes the context's."""
        self._mesh, self._mesh_keep = _capi.mesh_view(m)
        self._check(self.lib.pffrg_resample(self.h, src_slot, dst_slot, ctypes.byref(self._mesh)), "resample")

    def set_precision(self, precision: str) -> None:
        p = _capi.PFFRG_FP64 if precision == "fp64" else _capi.PFFRG_MIXED
        self._check(self.lib.pffrg_set_precision(self.h, p), "set_precision")

    @property
    def last_integrand_evals(self) -> int:
        return int(self.lib.pffrg_last_integrand_evals(self.h))

    def set_timing(self, on: bool) -> None:
        self._check(self.lib.pffrg_set_timing(self.h, int(on)), "set_timing")

    def read_stats(self, reset: bool = False) -> dict:
        st = _capi.Stats()
        self._check(self.lib.pffrg_read_stats(self.h, ctypes.byref(st), int(reset)), "read_stats")
        return {k: getattr(st, k) for k, _ in _capi.Stats._fields_}

    # ---- reference-facing calls (host arrays in, host arrays out) ----
    def compute_dsigma(self, Lam: float, a: Action, da: Action, sigma_tol=(1e-8, 1e-4)) -> None:
        av, dv = _capi.action_view(a), _capi.action_view(da)
        self._check(self.lib.pffrg_dsigma(self.h, Lam, ctypes.byref(av), ctypes.byref(dv), *sigma_tol), "dsigma")

    def compute_dgamma(self, Lam: float, a: Action, da: Action, eval_: int, gamma_tol=(1e-8, 1e-4),
                       loops: int = 1, sigma_corr: bool = False, sigma_tol=(1e-8, 1e-4)) -> None:
        av, dv = _capi.action_view(a), _capi.action_view(da)
        self._check(self.lib.pffrg_dgamma(self.h, loops, Lam, ctypes.byref(av), ctypes.byref(dv), eval_,
                                          gamma_tol[0], gamma_tol[1], int(sigma_corr), sigma_tol[0], sigma_tol[1]),
                    "dgamma")

    def compute_sigma_sde(self, Lam: float, a1: Action, a2: Action, eval_: int, gamma_tol=(1e-8, 1e-4),
                          sigma_tol=(1e-8, 1e-4)) -> None:
        v1, v2 = _capi.action_view(a1), _capi.action_view(a2)
        self._check(self.lib.pffrg_sde(self.h, Lam, ctypes.byref(v1), ctypes.byref(v2), eval_, gamma_tol[0],
                                       gamma_tol[1], sigma_tol[0], sigma_tol[1]), "sde")

    def compute_gamma_bse(self, Lam: float, a1: Action, a2: Action, eval_: int, gamma_tol=(1e-8, 1e-4)) -> None:
        v1, v2 = _capi.action_view(a1), _capi.action_view(a2)
        self._check(self.lib.pffrg_bse(self.h, Lam, ctypes.byref(v1), ctypes.byref(v2), eval_, *gamma_tol), "bse")

    def compute_chi(self, Lam: float, a: Action, chi_mesh, chi_tol=(1e-8, 1e-4)):
        """compute_χ! (correlation_su2.jl:58-86): χ[i, w] as an [Ns, num_chi] array (column-major);
        for u1-dm the list [χxx, χzz, χxy] of such arrays (correlation_u1_dm.jl:152-190)."""
        av = _capi.action_view(a)
        return self._chi(lambda mp, n, out: self.lib.pffrg_chi(self.h, Lam, ctypes.byref(av), mp, n, chi_tol[0],
                                                                chi_tol[1], out), chi_mesh)

    def chi_slot(self, Lam: float, slot: int, chi_mesh, chi_tol=(1e-8, 1e-4)) -> np.ndarray:
        """χ of the device-resident action in `slot`."""
        return self._chi(lambda mp, n, out: self.lib.pffrg_chi_slot(self.h, Lam, slot, mp, n, chi_tol[0],
                                                                     chi_tol[1], out), chi_mesh)

    def _chi(self, call, chi_mesh):
        mesh = np.ascontiguousarray(chi_mesh, dtype=np.float64)
        ncomp = 1 if self.symmetry == "su2" else 3
        n = self.num_sites * len(mesh)
        out = np.zeros(ncomp * n, dtype=np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(call(mesh.ctypes.data_as(dp), len(mesh), out.ctypes.data_as(dp)), "chi")
        mats = [out[k * n:(k + 1) * n].reshape((self.num_sites, len(mesh)), order="F") for k in range(ncomp)]
        return mats[0] if ncomp == 1 else mats

    def set_async_waves(self, on: bool) -> None:
        """Device-driven quadrature levels (default) or the host-driven loop; same results."""
        self._check(self.lib.pffrg_set_async_waves(self.h, int(bool(on))), "set_async_waves")

    def set_fp64_handoff(self, eps: float = 1e-6) -> None:
        """Mixed path: Simpson subdomains whose test FP32 rounding (relative eps) could flip are
        evaluated again in FP64, so the adaptive decisions are the FP64 path's (0: off)."""
        self._check(self.lib.pffrg_set_fp64_handoff(self.h, float(eps)), "set_fp64_handoff")

    def autotune_team_shape(self, Lam: float, eval_: int, loops: int = 1, a_slot: int = _capi.SLOT_A,
                            da_slot: int = _capi.SLOT_DA, gamma_tol=(1e-8, 1e-4), sigma_tol=(1e-8, 1e-4)):
        """Time one right-hand side per candidate team shape on the device-resident action in
        a_slot (da_slot is overwritten), keep the fastest and return it as (lanes, sites per lane)."""
        t, s = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.pffrg_autotune_team_shape(self.h, loops, Lam, a_slot, da_slot, eval_, gamma_tol[0],
                                                       gamma_tol[1], sigma_tol[0], sigma_tol[1], ctypes.byref(t),
                                                       ctypes.byref(s)), "autotune_team_shape")
        return t.value, s.value

    def set_chi_integrand(self, precision: str = "fp64") -> None:
        """χ integrand of a mixed context in FP64 (default) or mixed (FP32, float-float setup)."""
        code = {"fp64": _capi.PFFRG_FP64, "mixed": _capi.PFFRG_MIXED}[precision]
        self._check(self.lib.pffrg_set_chi_integrand(self.h, code), "set_chi_integrand")

    def set_chi_cluster(self, min_regions: int = 32768, blocks: int = 8) -> None:
        """χ cubature passes with at least min_regions of region capacity run each integral on a
        cluster of `blocks` (8 or 16) blocks (min_regions 0: always); results are identical."""
        self._check(self.lib.pffrg_set_chi_cluster(self.h, int(min_regions), int(blocks)), "set_chi_cluster")

    def set_capacities(self, queue_chunks: int = 0, gk_segments: int = 0) -> None:
        """Chunk-queue capacity of the quadrature levels and first Gauss-Kronrod segment capacity
        (0: the defaults); a level beyond the queue raises PffrgError with PFFRG_E_LIMIT."""
        self._check(self.lib.pffrg_set_capacities(self.h, int(queue_chunks), int(gk_segments)), "set_capacities")

    def set_overlap_staging(self, mode: int = 0) -> None:
        """Overlap rows of the t-channel sums: 0 staged by size, 1 through L1/L2, 2 staged when
        they fit a block's shared memory.  Results agree to rounding."""
        self._check(self.lib.pffrg_set_overlap_staging(self.h, int(mode)), "set_overlap_staging")

    def set_team_shape(self, lanes: int = 0, sites_per_lane: int = 0) -> None:
        """Team shape of the quadrature passes (lanes x sites per lane; 0, 0: chosen from the
        number of sites).  Results agree to rounding."""
        self._check(self.lib.pffrg_set_team_shape(self.h, int(lanes), int(sites_per_lane)), "set_team_shape")

    # ---- device-resident interface ----
    def upload(self, slot: int, a: Action) -> None:
        v = _capi.action_view(a)
        self._check(self.lib.pffrg_upload(self.h, slot, ctypes.byref(v)), "upload")

    def download(self, slot: int, a: Action) -> None:
        v = _capi.action_view(a)
        self._check(self.lib.pffrg_download(self.h, slot, ctypes.byref(v)), "download")

    def rhs(self, Lam: float, eval_: int, loops: int = 1, a_slot: int = _capi.SLOT_A, da_slot: int = _capi.SLOT_DA,
            gamma_tol=(1e-8, 1e-4), sigma_tol=(1e-8, 1e-4), sigma_corr: bool = False) -> None:
        self._check(self.lib.pffrg_rhs(self.h, loops, Lam, a_slot, da_slot, eval_, gamma_tol[0], gamma_tol[1],
                                       sigma_tol[0], sigma_tol[1], int(sigma_corr)), "rhs")

    def bs_step(self, Lam: float, dLam: float, eval_: int, loops: int = 1, gamma_tol=(1e-8, 1e-4),
                sigma_tol=(1e-8, 1e-4), sigma_corr: bool = False, ode_tol=(1e-8, 1e-2)):
        err = ctypes.c_double()
        amax = ctypes.c_double()
        self._check(self.lib.pffrg_bs_step(self.h, loops, Lam, dLam, eval_, gamma_tol[0], gamma_tol[1], sigma_tol[0],
                                           sigma_tol[1], int(sigma_corr), ode_tol[0], ode_tol[1], ctypes.byref(err),
                                           ctypes.byref(amax)), "bs_step")
        return float(err.value), float(amax.value)

    def parquet(self, Lam: float, eval_: int, gamma_tol=(1e-8, 1e-4), sigma_tol=(1e-8, 1e-4),
                parquet_tol=(1e-8, 1e-4), beta=None, max_iter: int = 50, history: bool = False):
        """launch_parquet!'s fixed point (parquet.jl:43-80) on the action in slot A, in place on the
        device; returns (iterations, absolute residual, relative residual) and, with ``history``, the
        absolute residual of every iteration as a fourth item."""
        beta = min(Lam, 1.0) if beta is None else beta
        it, ea, er = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        hist = np.zeros(max(1, max_iter))
        self._check(self.lib.pffrg_parquet(self.h, Lam, eval_, gamma_tol[0], gamma_tol[1], sigma_tol[0], sigma_tol[1],
                                           parquet_tol[0], parquet_tol[1], beta, max_iter, ctypes.byref(it),
                                           ctypes.byref(ea), ctypes.byref(er),
                                           hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "parquet")
        if history:
            return it.value, ea.value, er.value, hist[:it.value].copy()
        return it.value, ea.value, er.value

    def accept(self) -> None:
        self._check(self.lib.pffrg_accept(self.h), "accept")


def get_eval(Lam: float, min_eval: int, max_eval: int) -> int:
    """Subdomains per integration range (launcher_1l.jl:78)."""
    return int(min(max(int(np.ceil(min_eval / np.sqrt(Lam))), min_eval), max_eval))
