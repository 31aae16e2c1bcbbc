"""Action storage in the reference's memory layout (host side).

An ``Action`` holds the self energy Σ and, per vertex component, the bare
couplings and the s/t/u channels with their four asymptotic kernels
(src/Action/channel.jl:10-15, src/Action/vertex.jl:10-15,
src/Action/action_lib/action_su2.jl:8-12).  All arrays live in ONE
contiguous float64 buffer, each array in Julia column-major order with the
site index fastest, so that a Julia array maps onto a view of this buffer
one-to-one and the device copy is a single memcpy:

    Σ[Nσ] | for comp c: bare[Ns] | for ch in (s, t, u):
                                     q1[Ns,NΩ] q2_1[Ns,NΩ,Nν] q2_2[Ns,NΩ,Nν] q3[Ns,NΩ,Nν,Nν]
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SYMMETRIES = {"su2": 2, "u1-dm": 6}
CHANNELS = ("s", "t", "u")
KERNELS = ("q1", "q2_1", "q2_2", "q3")


@dataclass(frozen=True)
class Layout:
    """Offsets of every array inside the packed buffer."""

    num_sites: int
    num_sigma: int
    num_omega: int
    num_nu: int
    num_comps: int

    @property
    def k1(self) -> int:
        return self.num_sites * self.num_omega

    @property
    def k2(self) -> int:
        return self.k1 * self.num_nu

    @property
    def k3(self) -> int:
        return self.k2 * self.num_nu

    @property
    def channel_size(self) -> int:
        return self.k1 + 2 * self.k2 + self.k3

    @property
    def comp_size(self) -> int:
        return self.num_sites + 3 * self.channel_size

    @property
    def size(self) -> int:
        return self.num_sigma + self.num_comps * self.comp_size

    def bare_offset(self, comp: int) -> int:
        return self.num_sigma + comp * self.comp_size

    def kernel_offset(self, comp: int, ch: int, kernel: int) -> int:
        base = self.bare_offset(comp) + self.num_sites + ch * self.channel_size
        return base + (0, self.k1, self.k1 + self.k2, self.k1 + 2 * self.k2)[kernel]

    def kernel_shape(self, kernel: int) -> tuple:
        Ns, NO, Nn = self.num_sites, self.num_omega, self.num_nu
        return ((Ns, NO), (Ns, NO, Nn), (Ns, NO, Nn), (Ns, NO, Nn, Nn))[kernel]


class Channel:
    def __init__(self, buf: np.ndarray, lay: Layout, comp: int, ch: int):
        for k, name in enumerate(KERNELS):
            off = lay.kernel_offset(comp, ch, k)
            shape = lay.kernel_shape(k)
            n = int(np.prod(shape))
            setattr(self, name, buf[off:off + n].reshape(shape, order="F"))


class Vertex:
    def __init__(self, buf: np.ndarray, lay: Layout, comp: int):
        off = lay.bare_offset(comp)
        self.bare = buf[off:off + lay.num_sites]
        self.ch_s = Channel(buf, lay, comp, 0)
        self.ch_t = Channel(buf, lay, comp, 1)
        self.ch_u = Channel(buf, lay, comp, 2)

    @property
    def channels(self):
        return (self.ch_s, self.ch_t, self.ch_u)


class Action:
    """Σ and vertex of one flow state (Action_su2 / Action_u1_dm)."""

    def __init__(self, symmetry: str, num_sites: int, num_sigma: int, num_omega: int, num_nu: int,
                 S: float = 0.5, buf: np.ndarray | None = None):
        if symmetry not in SYMMETRIES:
            raise ValueError(f"Symmetry {symmetry} unknown. Valid arguments are su2 and u1-dm.")
        self.symmetry = symmetry
        self.S = float(S)
        self.layout = Layout(num_sites, num_sigma, num_omega, num_nu, SYMMETRIES[symmetry])
        if buf is None:
            buf = np.zeros(self.layout.size)
        if buf.dtype != np.float64 or buf.size != self.layout.size or not buf.flags.c_contiguous:
            raise ValueError("action buffer must be a contiguous float64 array of the layout size")
        self.buf = buf
        self.Σ = buf[:num_sigma]
        self.Γ = [Vertex(buf, self.layout, c) for c in range(self.layout.num_comps)]

    @classmethod
    def empty_like(cls, other: "Action") -> "Action":
        lay = other.layout
        return cls(other.symmetry, lay.num_sites, lay.num_sigma, lay.num_omega, lay.num_nu, other.S)

    def copy(self) -> "Action":
        lay = self.layout
        return Action(self.symmetry, lay.num_sites, lay.num_sigma, lay.num_omega, lay.num_nu, self.S,
                      self.buf.copy())

    # vertex part of the buffer (everything after Σ) without the bare couplings
    def gamma_mask(self) -> np.ndarray:
        lay = self.layout
        m = np.zeros(lay.size, dtype=bool)
        for c in range(lay.num_comps):
            off = lay.bare_offset(c) + lay.num_sites
            m[off:off + 3 * lay.channel_size] = True
        return m

    def q3_mask(self) -> np.ndarray:
        lay = self.layout
        m = np.zeros(lay.size, dtype=bool)
        for c in range(lay.num_comps):
            for ch in range(3):
                off = lay.kernel_offset(c, ch, 3)
                m[off:off + lay.k3] = True
        return m

    def abs_max(self) -> float:
        """get_abs_max: maximum |q3| over all components and channels (Action.jl:346-359)."""
        return float(np.max(np.abs(self.buf[self.q3_mask()]))) if self.layout.k3 else 0.0


def get_action_empty(symmetry: str, r, m, S: float = 0.5) -> Action:
    """Zero action on the lattice ``r`` and meshes ``m`` (Action.jl:566-579)."""
    return Action(symmetry, r.num_sites, m.num_sigma, m.num_omega, m.num_nu, S)


def init_action(lat, r, a: Action) -> None:
    """Bare couplings from the lattice bonds (action_su2.jl:35-56, action_u1_dm.jl:32-61)."""
    origin = 0
    if a.symmetry == "su2":
        for i, site in enumerate(r.irreducible):
            b = lat.bond(origin, int(site))
            a.Γ[0].bare[i] = b[0, 0] / 4.0 / (2.0 * a.S)
    else:
        for i, site in enumerate(r.irreducible):
            b = lat.bond(origin, int(site))
            a.Γ[0].bare[i] = b[0, 0] / 4.0
            a.Γ[1].bare[i] = b[2, 2] / 4.0
            a.Γ[2].bare[i] = b[0, 1] / 4.0


def add_repulsion(A: float, a: Action) -> None:
    """On-site level repulsion (action_su2.jl:59-70, action_u1_dm.jl:64-76)."""
    if a.symmetry == "su2":
        a.Γ[0].bare[0] += A / 4.0 / (2.0 * a.S)
    else:
        a.Γ[0].bare[0] += A / 4.0
        a.Γ[1].bare[0] += A / 4.0
