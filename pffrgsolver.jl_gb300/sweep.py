"""Coupling sweeps: many independent flows on one GPU at once.

Every instance (lattice, size, couplings) gets its own context, and so its
own CUDA stream and device scratch; the instances' flows run from a pool of
host threads, so the kernels of different instances overlap on the GPU
while each instance's host steps (the ODE control, the resampling) wait for
its own stream only.  The ctypes calls into the library release the GIL.
Results are those of ``launcher.launch`` for each instance on its own.
"""
from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from .launcher import FlowResult, launch


@dataclass
class Instance:
    name: str
    size: int
    model: str
    J: list
    symmetry: str = "su2"
    kwargs: dict = field(default_factory=dict)


def square_j1j2_sweep(n: int = 64, sizes=(3, 4, 5, 6, 8), seed: int = 2):
    """n square-lattice J1-J2 Heisenberg instances, J1 = 1, J2 ~ U[0, 1] (numpy seed), the sizes
    taken round-robin."""
    rng = np.random.default_rng(seed)
    j2 = rng.uniform(0.0, 1.0, size=n)
    return [Instance("square", sizes[k % len(sizes)], "heisenberg", [[1.0], [float(j2[k])]]) for k in range(n)]


def launch_sweep(instances, *, workers: int = 16, verbose: bool = False, **common) -> list:
    """Run every instance's flow (``launch`` with ``common`` keyword arguments, overridden by the
    instance's own); returns the FlowResults in instance order."""

    def run(inst: Instance) -> FlowResult:
        kw = dict(common)
        kw.update(inst.kwargs)
        return launch("", inst.name, inst.size, inst.model, inst.symmetry, inst.J, verbose=verbose, **kw)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, workers)) as pool:
        results = list(pool.map(run, instances))
    wall = time.perf_counter() - t0
    for r in results:
        r.sweep_seconds = wall
    return results
