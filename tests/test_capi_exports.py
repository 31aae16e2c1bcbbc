"""libpffrg_gpu.so loads on a machine without a GPU and exports every function include/*.h declares.

No compute call is made here; without a CUDA device pffrg_create must refuse
(there is no CPU fallback) with a message.
"""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(pffrg_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import importlib.util

    spec = importlib.util.spec_from_file_location("pffrg_build", ROOT / "pffrgsolver.jl_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    path = b.build()
    return ctypes.CDLL(str(path))


def test_every_declared_function_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_lists_every_export():
    import pffrg_gb300._capi as C

    assert set(C.EXPORTED) <= set(declared_functions())


def test_no_device_means_no_context(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import pffrg_gb300.workloads as wl
    import pffrg_gb300._capi as C

    lib = C.load()

    lat, r, m, a = wl.build_state(wl.WORKLOADS["square-L3-1l"], num_sigma=8, num_omega=4, num_nu=3)
    lv, keep = C.lattice_view(r)
    mv, mkeep = C.mesh_view(m)
    h = lib.pffrg_create(ctypes.byref(lv), ctypes.byref(mv), 0, 0.5, 0, 0)
    assert not h
    assert lib.pffrg_last_error(None)


def test_committed_ncu_traffic_summary_parses():
    """bench.py's roofline traffic and limiter figures come from the committed ncu summary of the
    benchmark state."""
    import importlib.util
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    spec = importlib.util.spec_from_file_location("bench_mod", root / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    prof = bench.ncu_profile_summary()
    assert prof is not None and prof["workload"] == bench.WORKLOAD and prof["precision"] == "mixed"
    assert prof["dram_bytes_per_rhs"] > 0 and prof["passes_per_rhs"] == 2
    assert 0 < prof["issue_active_pct"] <= 100 and 0 < prof["warps_active_per_sm"] <= 64
    assert isinstance(prof["limiter"], str) and prof["limiter"]


def test_setters_refuse_a_null_context():
    """The tuning and precision setters check their context before anything else (no device needed)."""
    import pffrg_gb300._capi as C

    L = C.load()
    assert L.pffrg_set_async_waves(None, 1) == 1
    assert L.pffrg_set_team_shape(None, 16, 3) == 1
    assert L.pffrg_set_fp64_handoff(None, 1e-6) == 1
    assert L.pffrg_set_chi_cluster(None, 32768, 8) == 1
    assert L.pffrg_set_chi_integrand(None, 0) == 1
    assert L.pffrg_autotune_team_shape(None, 1, 1.0, 0, 1, 10, 1e-8, 1e-4, 1e-8, 1e-4, None, None) == 1
