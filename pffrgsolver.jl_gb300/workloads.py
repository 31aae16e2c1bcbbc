"""Seeded synthetic flow states of the benchmark configurations.

No dataset is involved: the reference's workloads are model definitions
(lattice, couplings, mesh sizes).  A state is the bare action of the model
plus seeded normal noise on every channel entry and on Σ, drawn with
``numpy.random.default_rng(seed)`` in a fixed order (component, then channel
s/t/u, then kernel q1/q2_1/q2_2/q3, each array in column-major order, then
Σ[2:end]; Σ[1] = 0).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import action as A
from . import frequency as F
from . import lattice as L


@dataclass
class Workload:
    name: str
    lattice: str
    size: int
    model: str
    J: list
    loops: int
    Lam: float
    num_sigma: int
    num_omega: int
    num_nu: int
    noise: float
    seed: int
    bare_on_t: bool = False
    symmetry: str = "su2"
    S: float = 0.5
    eval: int = 10  # subdomains per integration range (launcher_1l.jl:78 gives 10 at Λ = 1)


WORKLOADS = {
    # square L=3 Heisenberg, 1 loop, 50/15/10 frequencies, one dΓ at Λ=1, N(0, 0.1), seed 0
    "square-L3-1l": Workload("square-L3-1l", "square", 3, "heisenberg", [[1.0]], 1, 1.0, 50, 15, 10, 0.1, 0),
    # pyrochlore L=6 Heisenberg, 2 loop, same meshes, N(0, 0.05) seed 1 + bare J on Ω=0 of ch_t spin (benchmark)
    "pyrochlore-L6-2l": Workload("pyrochlore-L6-2l", "pyrochlore", 6, "heisenberg", [[1.0]], 2, 1.0, 50, 15, 10,
                                 0.05, 1, bare_on_t=True),
    # the same lattice and state on small meshes (11/4/3 positive frequencies, eval 2, 1 loop): profiling case
    "pyrochlore-L6-reduced": Workload("pyrochlore-L6-reduced", "pyrochlore", 6, "heisenberg", [[1.0]], 1, 1.0, 11, 4,
                                      3, 0.05, 1, bare_on_t=True, eval=2),
    # kagome L=8 XXZ + DM (J⊥ = 1, Jz = 0.8, Dz = 0.2), U(1)-DM, 3 loops with the Σ corrections, one
    # right-hand side at Λ=1 on N(0, 0.05) seed 5: the largest workload's meshes (60/20/15) and smaller
    # ones (30/10/8) for profiling and quick timing
    "kagome-L8-3l-u1dm": Workload("kagome-L8-3l-u1dm", "kagome", 8, "kagome-xxz-dm", [[1.0, 0.8, 0.2]], 3, 1.0, 60,
                                  20, 15, 0.05, 5, symmetry="u1-dm"),
    "kagome-L8-3l-u1dm-reduced": Workload("kagome-L8-3l-u1dm-reduced", "kagome", 8, "kagome-xxz-dm",
                                          [[1.0, 0.8, 0.2]], 3, 1.0, 30, 10, 8, 0.05, 5, symmetry="u1-dm"),
}


def normalize_couplings(J, A_rep: float = 0.0):
    """LinearAlgebra.normalize([J, [[A]]]) of launch! (Launcher.jl:647-650)."""
    flat = [x for j in J for x in j] + [A_rep]
    nrm = float(np.sqrt(sum(x * x for x in flat)))
    return [[x / nrm for x in j] for j in J], A_rep / nrm


def build_state(w: Workload, num_sigma=None, num_omega=None, num_nu=None, size=None):
    """(lattice, reduced lattice, mesh, action) of a workload; sizes may be overridden for small tests."""
    J, _ = normalize_couplings(w.J)
    lat = L.get_lattice(w.lattice, size or w.size)
    r = L.get_reduced_lattice(w.model, J, lat)
    m = F.initial_mesh(w.Lam, num_sigma or w.num_sigma, num_omega or w.num_omega, num_nu or w.num_nu, 10)
    a = A.get_action_empty(w.symmetry, r, m, S=w.S)
    A.init_action(lat, r, a)
    fill_noise(a, w.noise, w.seed)
    if w.bare_on_t:
        for k in ("q1", "q2_1", "q2_2", "q3"):
            q = getattr(a.Γ[0].ch_t, k)
            q[:, 0, ...] += a.Γ[0].bare.reshape((-1,) + (1,) * (q.ndim - 2))
    return lat, r, m, a


def fill_noise(a: A.Action, sigma: float, seed: int) -> None:
    rng = np.random.default_rng(seed)
    for v in a.Γ:
        for ch in v.channels:
            for k in ("q1", "q2_1", "q2_2", "q3"):
                q = getattr(ch, k)
                q[...] = rng.normal(0.0, sigma, q.size).reshape(q.shape, order="F")
    a.Σ[0] = 0.0
    a.Σ[1:] = rng.normal(0.0, sigma, a.Σ.size - 1)
