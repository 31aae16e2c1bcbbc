"""The reference's observable (``*_obs``) and checkpoint (``*_cp``) files.

Same HDF5 paths, shapes and types as src/Observable/disk.jl,
src/Action/disk.jl, src/Action/checkpoint_lib/checkpoint_{su2,u1_dm}.jl and
src/Lattice/disk.jl, so files move between this package and PFFRGSolver.jl
in both directions.  Cutoffs in group names are Julia's ``string(Λ)``.
Written with the package's own HDF5 module (no libhdf5 needed).
"""
from __future__ import annotations

import numpy as np

from . import action as A
from . import frequency as F
from . import lattice as L
from .hdf5 import File, julia_float_str

COMP_NAMES = {"su2": ("spin", "dens"), "u1-dm": ("Γxx", "Γzz", "ΓDM", "Γdd", "Γzd", "Γdz")}
CHI_LABELS = {"su2": ("diag",), "u1-dm": ("xx", "zz", "xy")}


def _key(Lam: float) -> str:
    return julia_float_str(Lam)


def _nearest(f: File, group: str, Lam: float, verbose: bool = True) -> str:
    keys = f.keys(group)
    cut = np.array([float(k) for k in keys])
    k = keys[int(np.argmin(np.abs(cut - Lam)))]
    if verbose:
        print(f"Λ was adjusted to {k}.")
    return k


# ---- lattice (Lattice/disk.jl:2-47) ----
def save_lattice(f: File, r: L.ReducedLattice, euclidean: bool) -> None:
    f["reduced_lattice/name"] = r.name
    f["reduced_lattice/size"] = int(r.size)
    f["reduced_lattice/model"] = r.model
    f["reduced_lattice/euclidean"] = bool(euclidean)
    for i, j in enumerate(r.J, start=1):
        f[f"reduced_lattice/J/{i}"] = np.asarray(j, dtype=np.float64)


def read_lattice(f: File):
    name = f.read("reduced_lattice/name")
    size = int(f.read("reduced_lattice/size"))
    model = f.read("reduced_lattice/model")
    euclidean = bool(f.read("reduced_lattice/euclidean"))
    J = [list(np.atleast_1d(f.read(f"reduced_lattice/J/{i}"))) for i in range(1, len(f.keys("reduced_lattice/J")) + 1)]
    lat = L.get_lattice(name, size, euclidean=euclidean)
    r = L.get_reduced_lattice(model, J, lat)
    return lat, r


# ---- self energy (Action/disk.jl:56-104) ----
def save_self(f: File, Lam: float, m: F.Mesh, a: A.Action) -> None:
    f[f"σ/{_key(Lam)}"] = np.asarray(m.sigma, dtype=np.float64)
    f[f"Σ/{_key(Lam)}"] = np.array(a.Σ, dtype=np.float64)


def read_self(f: File, Lam: float):
    k = _nearest(f, "σ", Lam)
    return f.read(f"σ/{k}"), f.read(f"Σ/{k}")


# ---- correlations (Observable/disk.jl:2-160) ----
def save_chi(f: File, Lam: float, symmetry: str, m: F.Mesh, chi) -> None:
    if "symmetry" not in f:
        f["symmetry"] = symmetry
    k = _key(Lam)
    f[f"χ/{k}/mesh"] = np.asarray(m.chi, dtype=np.float64)
    mats = [chi] if symmetry == "su2" and isinstance(chi, np.ndarray) else list(chi)
    for label, c in zip(CHI_LABELS[symmetry], mats):
        f[f"χ/{k}/{label}"] = np.asfortranarray(c, dtype=np.float64)


def read_chi_labels(f: File) -> list:
    ref = f.keys("χ")[0]
    return [k for k in f.keys(f"χ/{ref}") if k != "mesh"]


def read_chi(f: File, Lam: float, label: str, verbose: bool = True):
    k = _nearest(f, "χ", Lam, verbose)
    return f.read(f"χ/{k}/mesh"), f.read(f"χ/{k}/{label}")


def read_chi_all(f: File, Lam: float, verbose: bool = True):
    k = _nearest(f, "χ", Lam, verbose)
    return f.read(f"χ/{k}/mesh"), [f.read(f"χ/{k}/{label}") for label in read_chi_labels(f)]


def read_chi_flow_at_site(f: File, site: int, label: str):
    """(cutoffs descending, static χ at irreducible site `site`, 1-based)."""
    cut = sorted((float(k) for k in f.keys("χ")), reverse=True)
    vals = np.array([f.read(f"χ/{_key(c)}/{label}")[site - 1, 0] for c in cut])
    return np.array(cut), vals


# ---- checkpoints (checkpoint_su2.jl, checkpoint_u1_dm.jl, Action/disk.jl:2-53, 106-140) ----
def _save_vertex(f: File, label: str, a: A.Action, c: int) -> None:
    f[label + "/bare"] = np.array(a.Γ[c].bare)
    for name, ch in zip(("ch_s", "ch_t", "ch_u"), a.Γ[c].channels):
        for q in ("q1", "q2_1", "q2_2", "q3"):
            f[f"{label}/{name}/{q}"] = np.asfortranarray(getattr(ch, q))


def checkpoint(f: File, Lam: float, dLam: float, m: F.Mesh, a: A.Action) -> None:
    k = _key(Lam)
    f[f"dΛ/{k}"] = float(dLam)
    f[f"σ/{k}"] = np.asarray(m.sigma, dtype=np.float64)
    f[f"Ωs/{k}"] = np.asarray(m.omega_s, dtype=np.float64)
    f[f"νs/{k}"] = np.asarray(m.nu_s, dtype=np.float64)
    f[f"Ωt/{k}"] = np.asarray(m.omega_t, dtype=np.float64)
    f[f"νt/{k}"] = np.asarray(m.nu_t, dtype=np.float64)
    f[f"χ/{k}"] = np.asarray(m.chi, dtype=np.float64)
    if a.symmetry == "su2" and "S" not in f:
        f["S"] = float(a.S)
    if "symmetry" not in f:
        f["symmetry"] = a.symmetry
    f[f"a/{k}/Σ"] = np.array(a.Σ)
    for c, name in enumerate(COMP_NAMES[a.symmetry]):
        _save_vertex(f, f"a/{k}/Γ/{name}", a, c)


def read_checkpoint(f: File, Lam: float):
    """(Λ, dΛ, mesh, action) of the checkpoint nearest to Λ (read_checkpoint, Action.jl:588-601)."""
    symmetry = f.read("symmetry")
    k = _nearest(f, "σ", Lam)
    dLam = float(f.read(f"dΛ/{k}"))
    sig, Os, ns, Ot, nt, chi = (np.asarray(f.read(f"{g}/{k}"), dtype=np.float64)
                                for g in ("σ", "Ωs", "νs", "Ωt", "νt", "χ"))
    m = F.Mesh(len(sig), len(Os), len(ns), len(chi), sig, Os, ns, Ot, nt, chi)
    S = float(f.read("S")) if symmetry == "su2" else 0.5
    bare = f.read(f"a/{k}/Γ/{COMP_NAMES[symmetry][0]}/bare")
    a = A.Action(symmetry, len(bare), len(sig), len(Os), len(ns), S)
    a.Σ[:] = f.read(f"a/{k}/Σ")
    for c, name in enumerate(COMP_NAMES[symmetry]):
        a.Γ[c].bare[:] = f.read(f"a/{k}/Γ/{name}/bare")
        for chname, ch in zip(("ch_s", "ch_t", "ch_u"), a.Γ[c].channels):
            for q in ("q1", "q2_1", "q2_2", "q3"):
                getattr(ch, q)[...] = f.read(f"a/{k}/Γ/{name}/{chname}/{q}")
    return float(k), dLam, m, a
