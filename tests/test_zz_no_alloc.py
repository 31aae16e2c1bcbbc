"""The no-allocation one-loop dΓ entry point against the regular one.

pffrg_dgamma_1l_noalloc serves callers that cannot allocate device memory --
code running under CUDA graph capture, hosts whose device memory belongs to
another framework's pool, embedders with a fixed memory budget -- by keeping
all of its scratch in one static device array.  This test calls it through
the C ABI on device-resident actions, twice in a row on different states
(different lattices and mesh sizes, so stale scratch from the first call
would show in the second), and compares each result with the regular
pffrg_dgamma(loops = 1) FP64 path within the FP64 parity tolerance of the
other GPU tests (1e-10 relative in the max norm).
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


def test_noalloc_matches_dgamma(pkg):
    import torch

    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.action import Action
    from pffrg_gb300.flow import FlowContext

    lib = C.load()
    lib.pffrg_dgamma_1l_noalloc.argtypes = [ctypes.POINTER(C.LatticeView), ctypes.POINTER(C.MeshView),
                                            ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    lib.pffrg_noalloc_last_error.restype = ctypes.c_char_p
    lib.pffrg_noalloc_scratch_bytes.restype = ctypes.c_int64
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
        lv, lkeep = C.lattice_view(r)
        mv, mkeep = C.mesh_view(m)
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.pffrg_dgamma_1l_noalloc(ctypes.byref(lv), ctypes.byref(mv), a.S, Lam, a_dev.data_ptr(),
                                         da_dev.data_ptr(), eval_, tol[0], tol[1], stream)
        assert rc == 0, lib.pffrg_noalloc_last_error().decode()
        out = da_dev.cpu().numpy()
        rel = float(np.max(np.abs(out - ref.buf)) / np.max(np.abs(ref.buf)))
        assert rel < 1e-10, f"{lattice}: no-allocation dΓ differs from pffrg_dgamma by {rel:.3e}"
