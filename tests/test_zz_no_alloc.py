"""The no-allocation one-loop dΓ entry point against the regular one.

pffrg_dgamma_1l_noalloc serves callers that cannot allocate device memory --
hosts whose device memory belongs to another framework's pool allocator, and
embedders with a device-memory budget fixed at start-up -- by keeping all of
its scratch in one static device array.  The first test calls it through the
C ABI on device-resident actions, twice in a row on different states
(different lattices and mesh sizes, so stale scratch from the first call
would show in the second), and compares each result with the regular
pffrg_dgamma(loops = 1) FP64 path within the FP64 parity tolerance of the
other GPU tests (1e-10 relative in the max norm); a repeated call must leave
the device's free memory unchanged.  The others check its PFFRG_E_LIMIT
paths: a problem larger than the array, and boundary integrals that outgrow
the array's Gauss-Kronrod segments.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # lattice, size, positive frequencies (σ, Ω, ν), eval, seed
    ("square", 3, (11, 4, 3), 4, 3),
    ("kagome", 3, (9, 3, 3), 3, 5),
]
LIMIT = 3  # PFFRG_E_LIMIT


def _lib():
    import pffrg_gb300._capi as C

    lib = C.load()
    lib.pffrg_dgamma_1l_noalloc.argtypes = [ctypes.POINTER(C.LatticeView), ctypes.POINTER(C.MeshView),
                                            ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    lib.pffrg_noalloc_last_error.restype = ctypes.c_char_p
    lib.pffrg_noalloc_scratch_bytes.restype = ctypes.c_int64
    return lib


def _call(lib, r, m, a, a_dev, da_dev, Lam, eval_, tol):
    import torch

    import pffrg_gb300._capi as C

    lv, lkeep = C.lattice_view(r)
    mv, mkeep = C.mesh_view(m)
    stream = torch.cuda.current_stream().cuda_stream
    return lib.pffrg_dgamma_1l_noalloc(ctypes.byref(lv), ctypes.byref(mv), a.S, Lam, a_dev.data_ptr(),
                                       da_dev.data_ptr(), eval_, tol[0], tol[1], stream)


def test_noalloc_matches_dgamma(pkg):
    import torch

    import pffrg_gb300.workloads as wl
    from pffrg_gb300.action import Action
    from pffrg_gb300.flow import FlowContext

    lib = _lib()
    assert lib.pffrg_noalloc_scratch_bytes() == 128 << 20

    Lam, tol = 1.0, (1e-8, 1e-4)
    for lattice, size, (ns, no, nn), eval_, seed in CASES:
        w = wl.Workload("noalloc", lattice, size, "heisenberg", [[1.0]], 1, Lam, ns, no, nn, 0.1, seed)
        lat, r, m, a = wl.build_state(w)
        da = Action.empty_like(a)
        with FlowContext(r, m, precision="fp64") as ctx:
            ctx.compute_dsigma(Lam, a, da)
            ref = da.copy()
            ctx.compute_dgamma(Lam, a, ref, eval_, tol, loops=1)

        a_dev = torch.from_numpy(a.buf.copy()).cuda()
        da_dev = torch.from_numpy(da.buf.copy()).cuda()
        rc = _call(lib, r, m, a, a_dev, da_dev, Lam, eval_, tol)
        assert rc == 0, lib.pffrg_noalloc_last_error().decode()
        out = da_dev.cpu().numpy()
        rel = float(np.max(np.abs(out - ref.buf)) / np.max(np.abs(ref.buf)))
        assert rel < 1e-10, f"{lattice}: no-allocation dΓ differs from pffrg_dgamma by {rel:.3e}"
        # the same call again allocates nothing: the device's free memory stays as it was
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        rc = _call(lib, r, m, a, a_dev, da_dev, Lam, eval_, tol)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert rc == 0, lib.pffrg_noalloc_last_error().decode()
        assert free1 == free0, f"{lattice}: free device memory changed by {free0 - free1} bytes"


def test_noalloc_rejects_problems_beyond_the_array(pkg):
    """Pyrochlore L = 6 with 50/15/10 meshes at eval 10 needs far more than 128 MiB of scratch."""
    import torch

    import pffrg_gb300.workloads as wl

    lib = _lib()
    w = wl.WORKLOADS["pyrochlore-L6-2l"]
    lat, r, m, a = wl.build_state(w)
    a_dev = torch.from_numpy(a.buf.copy()).cuda()
    da_dev = torch.zeros_like(a_dev)
    rc = _call(lib, r, m, a, a_dev, da_dev, 1.0, 10, (1e-8, 1e-4))
    msg = lib.pffrg_noalloc_last_error().decode()
    assert rc == LIMIT and "bytes of scratch" in msg, (rc, msg)
    assert float(da_dev.abs().max()) == 0.0  # nothing was written


def test_noalloc_reports_gauss_kronrod_overflow(pkg):
    """With negative tolerances no error estimate meets them (zero ones can: |K15 - G7| reaches 0 on
    nearly linear segments), so the boundary integrals bisect until the array's 2048 segments per
    integral run out: the call returns PFFRG_E_LIMIT before any pass runs.  The meshes are squeezed
    so that Ω[end] + ν[end] = 3 Λ: on the regular meshes the Katanin propagator vanishes at the
    integration bound and the boundary integrals are skipped (bubbles.jl:121-153)."""
    import dataclasses

    import torch

    import pffrg_gb300.workloads as wl

    lib = _lib()
    w = wl.Workload("noalloc", "square", 3, "heisenberg", [[1.0]], 1, 1.0, 11, 4, 3, 0.1, 3)
    lat, r, m, a = wl.build_state(w)
    f = 3.0 / (m.omega_s[-1] + m.nu_s[-1])
    m = dataclasses.replace(m, sigma=m.sigma * f, omega_s=m.omega_s * f, nu_s=m.nu_s * f, omega_t=m.omega_t * f,
                            nu_t=m.nu_t * f)
    a_dev = torch.from_numpy(a.buf.copy()).cuda()
    da_dev = torch.zeros_like(a_dev)
    rc = _call(lib, r, m, a, a_dev, da_dev, 1.0, 4, (-1.0, -1.0))
    msg = lib.pffrg_noalloc_last_error().decode()
    assert rc == LIMIT and "Gauss-Kronrod" in msg, (rc, msg)
    assert float(da_dev.abs().max()) == 0.0  # no pass ran
