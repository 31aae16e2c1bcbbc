"""Build libpffrg_gpu.so for sm_103a in-tree (nvcc, translation units compiled in parallel)."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libpffrg_gpu.so"
# (source, object, defines): the pass kernels are compiled once per precision, component count and
# group of team shapes so that the longest objects build in parallel
SOURCES = [(s, s + ".o", []) for s in ["pffrg_passes.cu", "pffrg_sigma.cu", "pffrg_state.cu", "pffrg_capi.cu",
                                       "pffrg_noalloc.cu", "pffrg_mlp.cu"]]
SOURCES += [("pffrg_shapes.cu", f"pffrg_shapes_{r}_c{c}_g{g}.o",
             [f"-DPFFRG_R={r}", f"-DPFFRG_C={c}", f"-DPFFRG_GROUP={g}"])
            for r in ("double", "float") for c in (2, 6) for g in (0, 1, 2)]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [HERE.parent / "include" / "pffrg_gpu.h"]
    t = obj.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    procs = []
    objs = []
    for s, o, defs in SOURCES:
        src = CSRC / s
        obj = OUT_DIR / o
        objs.append(obj)
        if force or _stale(obj, src):
            cmd = [NVCC, *ARCH, *FLAGS, *defs, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((o, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((s, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or procs or not LIB.exists():
        cmd = [NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
