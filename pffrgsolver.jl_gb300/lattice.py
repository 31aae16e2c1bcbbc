"""Lattice graphs, spin models and their symmetry reduction (host-side set-up).

This module builds the tables that the flow right-hand side consumes:
irreducible sites, their multiplicities (``mult``), the site-exchange map
(``exchange``) and the overlap tables of the t-channel site sum
(``overlap``).  It restates the reference's Lattice layer:

* unit cells               -- src/Lattice/unitcell_lib/*.jl
* sites by bond distance   -- src/Lattice/site.jl:29-157 (``get_sites``)
* bond metric              -- src/Lattice/site.jl:159-207 (``get_metric``)
* n-th neighbours          -- src/Lattice/site.jl:235-271 (``get_nbs``)
* test sites               -- src/Lattice/site.jl:290-327 (``get_test_sites``)
* lattice                  -- src/Lattice/build.jl:34-84 (``get_lattice``)
* Heisenberg model         -- src/Lattice/model_lib/model_heisenberg.jl:13-56
* symmetry reduction       -- src/Lattice/reduced.jl:46-758

Site ordering, the choice of representatives and the row order of the
overlap tables follow the reference so that the vertex arrays use the same
site index as the Julia code (the drop-in layout).  Indices inside this
module are 0-based; the exported tables (``exchange``, ``overlap``) are
1-based exactly as the reference stores them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_S3 = math.sqrt(3.0)
_S2 = math.sqrt(2.0)


def _uc(basis, vectors, bonds):
    return (
        [np.array(b, dtype=np.float64) for b in basis],
        [np.array(v, dtype=np.float64) for v in vectors],
        [[tuple(int(x) for x in bd) for bd in bl] for bl in bonds],
    )


# Unit cells: (basis positions, Bravais vectors, bonds per basis site as
# (n1, n2, n3, delta_basis)).  src/Lattice/unitcell_lib/*.jl
UNITCELLS = {
    "square": _uc(
        [(0.0, 0.0, 0.0)],
        [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 0.0)],
        [[(1, 0, 0, 0), (-1, 0, 0, 0), (0, 1, 0, 0), (0, -1, 0, 0)]],
    ),
    "honeycomb": _uc(
        [(0.0, 0.0, 0.0), (1.0, 0.0, 0.0)],
        [(1.5, _S3 / 2.0, 0.0), (1.5, -_S3 / 2.0, 0.0), (0.0, 0.0, 0.0)],
        [[(0, -1, 0, 1), (-1, 0, 0, 1), (0, 0, 0, 1)],
         [(0, 1, 0, -1), (1, 0, 0, -1), (0, 0, 0, -1)]],
    ),
    "kagome": _uc(
        [(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.5, 0.5 * _S3, 0.0)],
        [(2.0, 0.0, 0.0), (1.0, _S3, 0.0), (0.0, 0.0, 0.0)],
        [[(0, 0, 0, 1), (0, 0, 0, 2), (-1, 0, 0, 1), (0, -1, 0, 2)],
         [(0, 0, 0, -1), (1, 0, 0, -1), (0, 0, 0, 1), (1, -1, 0, 1)],
         [(0, 0, 0, -2), (0, 0, 0, -1), (0, 1, 0, -2), (-1, 1, 0, -1)]],
    ),
    "triangular": _uc(
        [(0.0, 0.0, 0.0)],
        [(_S3 / 2.0, -0.5, 0.0), (_S3 / 2.0, 0.5, 0.0), (0.0, 0.0, 0.0)],
        [[(1, 0, 0, 0), (-1, 0, 0, 0), (0, 1, 0, 0), (0, -1, 0, 0), (1, -1, 0, 0), (-1, 1, 0, 0)]],
    ),
    "cubic": _uc(
        [(0.0, 0.0, 0.0)],
        [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)],
        [[(1, 0, 0, 0), (-1, 0, 0, 0), (0, 1, 0, 0), (0, -1, 0, 0), (0, 0, 1, 0), (0, 0, -1, 0)]],
    ),
    "fcc": _uc(
        [(0.0, 0.0, 0.0)],
        [(0.0, 1.0 / _S2, 1.0 / _S2), (1.0 / _S2, 0.0, 1.0 / _S2), (1.0 / _S2, 1.0 / _S2, 0.0)],
        [[(1, 0, 0, 0), (-1, 0, 0, 0), (0, 1, -1, 0), (0, -1, 1, 0), (0, 1, 0, 0), (0, -1, 0, 0),
          (1, 0, -1, 0), (-1, 0, 1, 0), (0, 0, 1, 0), (0, 0, -1, 0), (1, -1, 0, 0), (-1, 1, 0, 0)]],
    ),
    "bcc": _uc(
        [(0.0, 0.0, 0.0)],
        [(0.5, 0.5, -0.5), (-0.5, 0.5, 0.5), (0.5, -0.5, 0.5)],
        [[(-1, 0, 0, 0), (1, 0, 0, 0), (0, -1, 0, 0), (0, 1, 0, 0), (0, 0, -1, 0), (0, 0, 1, 0),
          (1, 1, 1, 0), (-1, -1, -1, 0)]],
    ),
    "hyperhoneycomb": _uc(
        [(0.0, 0.0, 0.0), (1.0, 1.0, 0.0), (1.0, 2.0, 1.0), (0.0, -1.0, 1.0)],
        [(-1.0, 1.0, -2.0), (-1.0, 1.0, 2.0), (2.0, 4.0, 0.0)],
        [[(0, 0, 0, 1), (0, 0, 0, 3), (1, 0, 0, 3)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (0, -1, 0, 1)],
         [(0, 0, 0, -1), (0, 1, 0, -1), (0, 0, 1, 1)],
         [(0, 0, 0, -3), (-1, 0, 0, -3), (0, 0, -1, -1)]],
    ),
    "hyperkagome": _uc(
        [(0.0, 0.0, 0.0),
         (-1.0 / _S2, 1.0 / _S2, 0.0),
         (0.0, 1.0 / _S2, 1.0 / _S2),
         (0.0, 2.0 / _S2, 2.0 / _S2),
         (-1.0 / _S2, 2.0 / _S2, 3.0 / _S2),
         (-2.0 / _S2, 1.0 / _S2, 3.0 / _S2),
         (-2.0 / _S2, 0.0, 2.0 / _S2),
         (-3.0 / _S2, 0.0, 3.0 / _S2),
         (-1.0 / _S2, 3.0 / _S2, 2.0 / _S2),
         (-2.0 / _S2, 3.0 / _S2, 1.0 / _S2),
         (-3.0 / _S2, 3.0 / _S2, 0.0),
         (-3.0 / _S2, 2.0 / _S2, 1.0 / _S2)],
        [(2.0 * _S2, 0.0, 0.0), (0.0, 2.0 * _S2, 0.0), (0.0, 0.0, 2.0 * _S2)],
        [[(0, 0, 0, 1), (0, 0, 0, 2), (1, 0, -1, 7), (1, -1, 0, 10)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (0, 0, -1, 3), (0, 0, -1, 4)],
         [(0, 0, 0, -1), (0, 0, 0, -2), (0, 0, 0, 1), (1, 0, 0, 9)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (0, 0, 0, 5), (1, 0, 0, 8)],
         [(0, 0, 0, -1), (0, 0, 0, 4), (0, 0, 0, 1), (0, 0, 1, -3)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (0, 0, 0, 2), (0, 0, 1, -4)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (0, -1, 0, 2), (0, -1, 0, 3)],
         [(0, 0, 0, -2), (0, 0, 0, -1), (-1, 0, 1, -7), (0, -1, 1, 3)],
         [(0, 0, 0, -5), (0, 0, 0, -4), (0, 1, 0, -2), (0, 0, 0, 1)],
         [(0, 1, 0, -3), (0, 0, 0, -1), (0, 0, 0, 1), (0, 0, 0, 2)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (-1, 1, 0, -10), (0, 1, -1, -3)],
         [(0, 0, 0, -2), (0, 0, 0, -1), (-1, 0, 0, -9), (-1, 0, 0, -8)]],
    ),
    "pyrochlore": _uc(
        [(0.0, 0.0, 0.0), (0.0, 0.25, 0.25), (0.25, 0.0, 0.25), (0.25, 0.25, 0.0)],
        [(0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)],
        [[(0, 0, 0, 1), (0, 0, 0, 2), (0, 0, 0, 3), (-1, 0, 0, 1), (0, -1, 0, 2), (0, 0, -1, 3)],
         [(0, 0, 0, -1), (0, 0, 0, 1), (0, 0, 0, 2), (1, 0, 0, -1), (1, -1, 0, 1), (1, 0, -1, 2)],
         [(0, 0, 0, -2), (0, 0, 0, -1), (0, 0, 0, 1), (0, 1, 0, -2), (-1, 1, 0, -1), (0, 1, -1, 1)],
         [(0, 0, 0, -3), (0, 0, 0, -2), (0, 0, 0, -1), (0, 0, 1, -3), (-1, 0, 1, -2), (0, -1, 1, -1)]],
    ),
    "diamond": _uc(
        [(0.0, 0.0, 0.0), (1.0 / _S3, 1.0 / _S3, 1.0 / _S3)],
        [(0.0, 2.0 / _S3, 2.0 / _S3), (2.0 / _S3, 0.0, 2.0 / _S3), (2.0 / _S3, 2.0 / _S3, 0.0)],
        [[(0, 0, 0, 1), (-1, 0, 0, 1), (0, -1, 0, 1), (0, 0, -1, 1)],
         [(0, 0, 0, -1), (1, 0, 0, -1), (0, 1, 0, -1), (0, 0, 1, -1)]],
    ),
}


def get_vec(t, uc) -> np.ndarray:
    """Cartesian position of site t = (n1, n2, n3, b), b 1-based (site.jl:14-27).

    The sum is formed component by component in the reference's order.
    """
    basis, vectors, _ = uc
    b = basis[t[3] - 1]
    out = np.empty(3)
    for k in range(3):
        out[k] = t[0] * vectors[0][k] + t[1] * vectors[1][k] + t[2] * vectors[2][k] + b[k]
    return out


def _add(t, bond):
    return (t[0] + bond[0], t[1] + bond[1], t[2] + bond[2], t[3] + bond[3])


def _neighbours(t, uc):
    return [_add(t, bd) for bd in uc[2][t[3] - 1]]


def get_sites(size: int, uc, euclidean: bool = False) -> list:
    """Sites in breadth-first order out to bond distance ``size`` (site.jl:29-157)."""
    origin = (0, 0, 0, 1)
    ints = [origin]
    seen = {origin}
    if not euclidean:
        current = [origin]
        for _ in range(size):
            new = []
            for t in current:
                for n in _neighbours(t, uc):
                    if n not in seen:
                        seen.add(n)
                        new.append(n)
                        ints.append(n)
            current = new
        return ints
    # Euclidean build: grow by bond steps while sites stay inside the sphere
    # of radius size * nearest-neighbour distance, following re-entrant paths
    # that leave and re-enter the sphere (site.jl:41-126).
    nn = float(np.linalg.norm(get_vec(_add(origin, uc[2][0][0]), uc)))
    radius = size * nn
    current = [origin]
    touched = [origin]
    while True:
        new, out = [], []
        touched_set = set(touched)
        for t in current:
            for n in _neighbours(t, uc):
                if n in touched_set or n in seen:
                    continue
                if np.linalg.norm(get_vec(n, uc)) <= radius:
                    new.append(n)
                    ints.append(n)
                    seen.add(n)
                else:
                    out.append(n)
        if not out:
            touched, current = current, new
            if not new:
                break
            continue
        cur_set = set(current)
        re = []
        for t in out:
            for n in _neighbours(t, uc):
                if n in cur_set or n in seen:
                    continue
                if np.linalg.norm(get_vec(n, uc)) <= radius:
                    re.append(t)
                    break
        if re:
            touched, current = current, new + re
        elif new:
            touched, current = current, new
        else:
            break
    return ints


def get_metric(t1, t2, uc) -> int:
    """Minimal number of bonds connecting two sites (site.jl:159-207)."""
    if t1 == t2:
        return 0
    seen = {t2}
    current = [t2]
    metric = 0
    while True:
        metric += 1
        new = []
        for t in current:
            for n in _neighbours(t, uc):
                if n not in seen:
                    seen.add(n)
                    new.append(n)
        if t1 in seen:
            return metric
        current = new


def get_test_sites(uc, euclidean: bool = False):
    """Basis sites plus their bonded neighbours (site.jl:290-327)."""
    basis, _, bonds = uc
    tests = []
    vecs = []

    def add(t, v):
        for w in vecs:
            if np.linalg.norm(w - v) <= 1e-8:
                return
        tests.append(t)
        vecs.append(v)

    for i in range(len(basis)):
        t = (0, 0, 0, i + 1)
        add(t, basis[i].copy())
        for bd in bonds[i]:
            n = _add(t, bd)
            add(n, get_vec(n, uc))
    if euclidean:
        metric = max(float(np.linalg.norm(v)) for v in vecs)
    else:
        metric = max(get_metric(tests[0], t, uc) for t in tests)
    return tests, vecs, metric


class _SiteIndex:
    """Coordinate -> site index lookup with the reference's 1e-8 tolerance."""

    def __init__(self, vecs: np.ndarray):
        self.vecs = vecs
        self.table = {}
        for i, v in enumerate(vecs):
            self.table.setdefault(self._key(v), i)

    @staticmethod
    def _key(v):
        return (round(v[0] * 1e5), round(v[1] * 1e5), round(v[2] * 1e5))

    def find(self, v) -> int:
        k = self._key(v)
        for d0 in (0, -1, 1):
            for d1 in (0, -1, 1):
                for d2 in (0, -1, 1):
                    i = self.table.get((k[0] + d0, k[1] + d1, k[2] + d2))
                    if i is not None and np.linalg.norm(self.vecs[i] - v) <= 1e-8:
                        return i
        return -1

    def find_many(self, V: np.ndarray) -> np.ndarray:
        keys = np.rint(V * 1e5).astype(np.int64)
        out = np.full(len(V), -1, dtype=np.int64)
        for n in range(len(V)):
            i = self.table.get((int(keys[n, 0]), int(keys[n, 1]), int(keys[n, 2])))
            if i is not None and np.linalg.norm(self.vecs[i] - V[n]) <= 1e-8:
                out[n] = i
            else:
                out[n] = self.find(V[n])
        return out


@dataclass
class Lattice:
    """Lattice graph (build.jl:13-20); bonds are a sparse map (i, j) -> 3x3 matrix."""

    name: str
    size: int
    uc: tuple
    test_sites: list
    test_vecs: list
    sites: list
    vecs: np.ndarray
    bonds: dict = field(default_factory=dict)
    euclidean: bool = False

    def __post_init__(self):
        self.index = _SiteIndex(self.vecs)

    def bond(self, i: int, j: int) -> np.ndarray:
        b = self.bonds.get((i, j))
        return b if b is not None else _ZERO_BOND

    def add_bond(self, J: float, i: int, j: int, mu: int, nu: int) -> None:
        b = self.bonds.get((i, j))
        if b is None:
            b = np.zeros((3, 3))
            self.bonds[(i, j)] = b
        b[mu, nu] += J


_ZERO_BOND = np.zeros((3, 3))


def _bonds_equal(b1, b2) -> bool:
    return float(np.linalg.norm(b1 - b2)) <= 1e-8


def get_lattice(name: str, size: int, verbose: bool = False, euclidean: bool = False) -> Lattice:
    """Lattice of all sites within ``size`` bonds of the origin (build.jl:34-84)."""
    if name not in UNITCELLS:
        raise ValueError(f"Unitcell {name} unknown.")
    uc = UNITCELLS[name]
    tests, tvecs, metric = get_test_sites(uc, euclidean)
    if euclidean:
        nn = float(np.linalg.norm(get_vec(_add(tests[0], uc[2][0][0]), uc)))
        if metric > size * nn:
            raise ValueError("Lattice is too small to perform symmetry reduction.")
    elif metric > size:
        raise ValueError("Lattice is too small to perform symmetry reduction.")
    ints = get_sites(size, uc, euclidean)
    vecs = np.array([get_vec(t, uc) for t in ints])
    lat = Lattice(name, size, uc, tests, tvecs, ints, vecs, euclidean=euclidean)
    if verbose:
        print(f"Done. Lattice has {len(ints)} sites.")
    return lat


def get_nbs(n: int, i: int, vecs: np.ndarray) -> np.ndarray:
    """Indices of the n-th nearest neighbours (Euclidean) of site i (site.jl:235-271)."""
    d = np.linalg.norm(vecs - vecs[i], axis=1)
    uniq = []
    for x in d:
        if not any(abs(u - x) <= 1e-8 for u in uniq):
            uniq.append(float(x))
    uniq.sort()
    if len(uniq) < n + 1:
        raise ValueError("Could not find neighbors in list.")
    dn = uniq[n]
    return np.nonzero(np.abs(dn - d) <= 1e-8)[0]


def _distinct_distances(d: np.ndarray) -> list:
    s = np.sort(d)
    out = [float(s[0])]
    for x in s[1:]:
        if abs(x - out[-1]) > 1e-8:
            out.append(float(x))
    return out


def _nbs_fast(n: int, i: int, vecs: np.ndarray) -> np.ndarray:
    d = np.linalg.norm(vecs - vecs[i], axis=1)
    uniq = _distinct_distances(d)
    if len(uniq) < n + 1:
        raise ValueError("Could not find neighbors in list.")
    dn = uniq[n]
    return np.nonzero(np.abs(dn - d) <= 1e-8)[0]


def init_model_heisenberg(J, lat: Lattice) -> None:
    """Heisenberg couplings to the n-th Euclidean neighbours (model_heisenberg.jl:13-56)."""
    for i in range(len(lat.sites)):
        for n, Jn in enumerate(J, start=1):
            nbs = _nbs_fast(n, i, lat.vecs)
            if len(Jn) == 1:
                for j in nbs:
                    for mu in range(3):
                        lat.add_bond(Jn[0], i, int(j), mu, mu)
            else:
                dist = [get_metric(lat.sites[int(j)], lat.sites[i], lat.uc) for j in nbs]
                kinds = sorted(set(dist))
                if len(Jn) != len(kinds):
                    raise ValueError(
                        f"{lat.name} has {len(kinds)} inequivalent {n}-th nearest neighbors, "
                        f"but {len(Jn)} couplings were supplied.")
                for k, kind in enumerate(kinds):
                    for j, dj in zip(nbs, dist):
                        if dj == kind:
                            for mu in range(3):
                                lat.add_bond(Jn[k], i, int(j), mu, mu)


def _grow_test_sites(lat: Lattice, metric: int) -> None:
    """Enlarge the symmetry test set to bond distance ``metric`` (build.jl:87-150)."""
    current = max(get_metric(lat.test_sites[0], t, lat.uc) for t in lat.test_sites)
    if current >= metric:
        return
    for t in get_sites(metric, lat.uc, False):
        v = get_vec(t, lat.uc)
        if not any(np.linalg.norm(w - v) <= 1e-8 for w in lat.test_vecs):
            lat.test_sites.append(t)
            lat.test_vecs.append(v)


def init_model_triangular_dm_c3(J, lat: Lattice) -> None:
    """XXZ + out-of-plane DM couplings on the triangular lattice (model_triangular_dm_c3.jl:14-73)."""
    if lat.name != "triangular":
        raise ValueError("Model requires triangular lattice.")
    if len(J) > 3:
        raise ValueError("Model initialization only works up to third-nearest neighbors.")
    for n, Jn in enumerate(J, start=1):
        if len(Jn) != 3:
            raise ValueError(f"Jxx, Jzz and Jxy all need to be specified for J[{n}].")
    max_nbs = _nbs_fast(len(J), 0, lat.vecs)
    metric = max(get_metric(lat.sites[0], lat.sites[int(i)], lat.uc) for i in max_nbs)
    _grow_test_sites(lat, metric)
    ref_vecs = []
    for i in range(len(lat.sites)):
        for n, Jn in enumerate(J, start=1):
            nbs = _nbs_fast(n, i, lat.vecs)
            Jxx, Jzz, Jxy = Jn
            if len(ref_vecs) < n:
                ref_vecs.append(lat.vecs[int(nbs[0])] - lat.vecs[i])
            ref = ref_vecs[n - 1]
            for j in nbs:
                j = int(j)
                vec = lat.vecs[j] - lat.vecs[i]
                p = round(float(np.dot(ref, vec) / (np.linalg.norm(ref) * np.linalg.norm(vec))), 8)
                p = min(1.0, max(-1.0, p))
                if math.fmod(math.acos(p), 2.0 * math.pi / 3.0) < 1e-8:
                    lat.add_bond(+Jxy, i, j, 0, 1)
                    lat.add_bond(-Jxy, i, j, 1, 0)
                else:
                    lat.add_bond(-Jxy, i, j, 0, 1)
                    lat.add_bond(+Jxy, i, j, 1, 0)
                lat.add_bond(Jxx, i, j, 0, 0)
                lat.add_bond(Jxx, i, j, 1, 1)
                lat.add_bond(Jzz, i, j, 2, 2)


def init_model_kagome_xxz_dm(J, lat: Lattice) -> None:
    """Nearest-neighbour XXZ + out-of-plane DM model on the kagome lattice, J = [[J⊥, Jz, Dz]].

    Not a model of the reference: it extends its bond-matrix convention
    (model_triangular_dm_c3.jl:14-73: exchange[1,1] = exchange[2,2] = J⊥,
    exchange[3,3] = Jz, exchange[1,2] = +D, exchange[2,1] = -D) with the usual
    kagome DM pattern: D_ij = +Dz ẑ when i -> j runs counterclockwise around the
    triangle that contains the bond, -Dz ẑ otherwise.
    """
    if lat.name != "kagome":
        raise ValueError("Model requires kagome lattice.")
    if len(J) != 1 or len(J[0]) != 3:
        raise ValueError("Model takes nearest-neighbour couplings [[Jperp, Jz, Dz]] only.")
    Jp, Jz, Dz = (float(x) for x in J[0])
    max_nbs = _nbs_fast(1, 0, lat.vecs)
    metric = max(get_metric(lat.sites[0], lat.sites[int(i)], lat.uc) for i in max_nbs)
    _grow_test_sites(lat, metric)
    nbs = [set(int(j) for j in _nbs_fast(1, i, lat.vecs)) for i in range(len(lat.sites))]
    for i in range(len(lat.sites)):
        for j in sorted(nbs[i]):
            # the third corner of the bond's triangle: the common nearest neighbour of i and j
            common = nbs[i] & nbs[j]
            if len(common) == 1:
                k = next(iter(common))
                a = lat.vecs[j] - lat.vecs[i]
                b = lat.vecs[k] - lat.vecs[i]
                ccw = a[0] * b[1] - a[1] * b[0] > 0.0
                d = Dz if ccw else -Dz
                lat.add_bond(+d, i, j, 0, 1)
                lat.add_bond(-d, i, j, 1, 0)
            lat.add_bond(Jp, i, j, 0, 0)
            lat.add_bond(Jp, i, j, 1, 1)
            lat.add_bond(Jz, i, j, 2, 2)


MODELS = {
    "heisenberg": init_model_heisenberg,
    "triangular-dm-c3": init_model_triangular_dm_c3,
    "kagome-xxz-dm": init_model_kagome_xxz_dm,
}


def init_model(name: str, J, lat: Lattice) -> None:
    """Dispatch to a model initialiser (build.jl:184-203)."""
    if name not in MODELS:
        raise ValueError(f"Model {name} unknown.")
    MODELS[name](J, lat)


# ---------------------------------------------------------------------------
# symmetry reduction (reduced.jl)
# ---------------------------------------------------------------------------

def _get_rotation(vec, ref) -> np.ndarray:
    """Rodrigues rotation of vec onto ref (reduced.jl:48-76)."""
    a = vec / np.linalg.norm(vec)
    b = ref / np.linalg.norm(ref)
    n = np.cross(a, b)
    s = float(np.linalg.norm(n))
    c = float(np.dot(a, b))
    if s < 1e-8:
        return -np.eye(3) if c < 0.0 else np.eye(3)
    n = n / s
    K = np.array([[0.0, -n[2], n[1]], [n[2], 0.0, -n[0]], [-n[1], n[0], 0.0]])
    return np.eye(3) + s * K + (1.0 - c) * (K @ K)


def _get_rotation_for_axis(vec, ref, axis) -> np.ndarray:
    """Rotation of vec onto ref about ``axis``, zeros on failure (reduced.jl:79-124)."""
    a = vec / np.linalg.norm(vec)
    b = ref / np.linalg.norm(ref)
    ax = axis / np.linalg.norm(axis)
    ovec = vec - np.dot(vec, ax) * ax
    ovec = ovec / np.linalg.norm(ovec)
    oref = ref - np.dot(ref, ax) * ax
    oref = oref / np.linalg.norm(oref)
    s = float(np.linalg.norm(np.cross(ovec, oref)))
    c = float(np.dot(ovec, oref))
    x, y, z = ax
    mat = np.array([
        [x * x + (1.0 - x * x) * c, x * y * (1.0 - c) - z * s, x * z * (1.0 - c) + y * s],
        [x * y * (1.0 - c) + z * s, y * y + (1.0 - y * y) * c, y * z * (1.0 - c) - x * s],
        [x * z * (1.0 - c) - y * s, y * z * (1.0 - c) + x * s, z * z + (1.0 - z * z) * c],
    ])
    if np.linalg.norm(mat @ a - b) > 1e-8:
        if np.linalg.norm(mat.T @ a - b) < 1e-8:
            return mat.T.copy()
        return np.zeros((3, 3))
    return mat


def _rotate(v1, v2, r1, r2) -> np.ndarray:
    mat = _get_rotation(v1, r1)
    return _get_rotation_for_axis(mat @ v2, r2, r1) @ mat


def _in_list(mat, mats) -> bool:
    return any(np.max(np.abs(m - mat)) <= 1e-8 for m in mats)


def _valid_origin_trafo(mat, lat: Lattice) -> bool:
    for t, v in zip(lat.test_sites, lat.test_vecs):
        k = lat.index.find(mat @ v)
        if k < 0:
            return False
        ti = lat.index.find(v)
        if not _bonds_equal(lat.bond(0, ti), lat.bond(0, k)):
            return False
    return True


def get_trafos_orig(lat: Lattice) -> list:
    """Point-group operations fixing the origin (reduced.jl:132-263)."""
    trafos = []
    con = lat.uc[2][0]
    ref = lat.sites[0]
    nv = [get_vec(_add(ref, c), lat.uc) for c in con]
    pairs = []
    for i1 in range(len(con)):
        for i2 in range(len(con)):
            if i1 == i2 or np.linalg.norm(np.cross(nv[i1], nv[i2])) <= 1e-8:
                continue
            pairs.append((i1, i2))
    for i1, i2 in pairs:
        for j1, j2 in pairs:
            mat = _rotate(nv[i1], nv[i2], nv[j1], nv[j2])
            if np.max(np.abs(mat)) > 1e-8:
                if not _in_list(mat, trafos) and _valid_origin_trafo(mat, lat):
                    trafos.append(mat)
                if not _in_list(-mat, trafos) and _valid_origin_trafo(-mat, lat):
                    trafos.append(-mat)
    return trafos


def get_reduced(lat: Lattice, trafos: list) -> np.ndarray:
    """Representative (smallest original index) of every site's orbit (reduced.jl:266-305)."""
    N = len(lat.sites)
    reduced = np.arange(N, dtype=np.int64)
    for i in range(1, N):
        if reduced[i] < i:
            continue
        vi = lat.vecs[i]
        b0i = lat.bond(0, i)
        for mat in trafos:
            mv = mat @ vi
            if np.linalg.norm(mv - vi) > 1e-8:
                k = lat.index.find(mv)
                if k < 0:
                    raise AssertionError("Validity on test set could not be generalized.")
                if _bonds_equal(b0i, lat.bond(0, k)):
                    reduced[k] = i
    return reduced


def get_trafos_uc(lat: Lattice) -> list:
    """Maps of every basis site onto the origin (reduced.jl:314-470).

    As in the reference, a later valid transformation overwrites an earlier
    one for the same basis site.
    """
    uc = lat.uc
    nb = len(uc[0])
    trafos = [None] * (nb - 1)
    ref = lat.sites[0]
    con = uc[2][0]
    rv = [get_vec(_add(ref, c), uc) for c in con]
    ridx = [lat.index.find(v) for v in rv]
    for b in range(2, nb + 1):
        bt = (0, 0, 0, b)
        bvec = get_vec(bt, uc)
        bi = lat.index.find(bvec)
        cb = uc[2][b - 1]
        bv = [get_vec(_add(bt, c), uc) for c in cb]
        bidx = [lat.index.find(v) for v in bv]
        in_range = []
        for t, v in zip(lat.test_sites, lat.test_vecs):
            if get_metric(t, bt, uc) <= lat.size:
                in_range.append((v, lat.index.find(v)))
        for b1 in range(len(cb)):
            for b2 in range(len(cb)):
                if b1 == b2 or np.linalg.norm(np.cross(bv[b1] - bvec, bv[b2] - bvec)) <= 1e-8:
                    continue
                bond_b1 = lat.bond(bi, bidx[b1])
                bond_b2 = lat.bond(bi, bidx[b2])
                for r1 in range(len(con)):
                    # a valid transformation ends the scan over r2 (the
                    # reference's ``break`` leaves the innermost loop only)
                    for r2 in range(len(con)):
                        if r1 == r2 or np.linalg.norm(np.cross(rv[r1], rv[r2])) <= 1e-8:
                            continue
                        if not (_bonds_equal(bond_b1, lat.bond(0, ridx[r1]))
                                and _bonds_equal(bond_b2, lat.bond(0, ridx[r2]))):
                            continue
                        found = False
                        for inverted in (False, True):
                            sg = -1.0 if inverted else 1.0
                            mat = _rotate(sg * (bv[b1] - bvec), sg * (bv[b2] - bvec), rv[r1], rv[r2])
                            if np.max(np.abs(mat)) <= 1e-8:
                                continue
                            valid = True
                            for v, ti in in_range:
                                mv = mat @ (sg * (v - bvec))
                                k = lat.index.find(mv)
                                if k < 0 or not _bonds_equal(lat.bond(bi, ti), lat.bond(0, k)):
                                    valid = False
                                    break
                            if valid:
                                trafos[b - 2] = (mat, inverted)
                                found = True
                                break
                        if found:
                            break
    return trafos


def get_mappings(lat: Lattice, reduced: np.ndarray, trafos_uc: list) -> np.ndarray:
    """Representative of every pair (i, j), -1 outside the lattice (reduced.jl:491-564)."""
    N = len(lat.sites)
    mat = np.full((N, N), -1, dtype=np.int64)
    np.fill_diagonal(mat, 0)
    uc = lat.uc
    basis = uc[0]
    for i in range(N):
        n1, n2, n3, b = lat.sites[i]
        shift = get_vec((n1, n2, n3, 1), uc)
        V = lat.vecs
        if b != 1:
            R, inv = trafos_uc[b - 2]
            if inv:
                M = (shift[None, :] - V + basis[b - 1][None, :]) @ R.T
            else:
                M = (V - shift[None, :] - basis[b - 1][None, :]) @ R.T
        else:
            M = V - shift[None, :]
        idx = lat.index.find_many(M)
        row = np.where(idx >= 0, reduced[np.maximum(idx, 0)], -1)
        row[i] = 0
        mat[i] = row
    return mat


@dataclass
class ReducedLattice:
    """Irreducible sites and the tables of the flow (reduced.jl:13-24).

    ``exchange`` and the overlap rows are 1-based, ``overlap[i]`` is an
    (rows, 3) array of (site a, site b, multiplicity).
    """

    name: str
    size: int
    model: str
    J: list
    sites: list
    vecs: np.ndarray
    overlap: list
    mult: np.ndarray
    exchange: np.ndarray
    project: np.ndarray
    irreducible: np.ndarray

    @property
    def num_sites(self) -> int:
        return len(self.sites)

    def overlap_csr(self):
        """Flattened overlap: (offsets[Ns+1], rows[R,3]) with 1-based site indices."""
        offs = np.zeros(len(self.overlap) + 1, dtype=np.int64)
        for i, t in enumerate(self.overlap):
            offs[i + 1] = offs[i] + len(t)
        rows = np.concatenate(self.overlap).astype(np.int64) if self.overlap else np.zeros((0, 3), np.int64)
        return offs, np.ascontiguousarray(rows)


def get_reduced_lattice(model: str, J, lat: Lattice, verbose: bool = False) -> ReducedLattice:
    """Symmetry-reduced representation of a lattice with a model (reduced.jl:716-758)."""
    init_model(model, J, lat)
    trafos = get_trafos_orig(lat)
    reduced = get_reduced(lat, trafos)
    irreducible = []
    seen = set()
    for x in reduced:
        if int(x) not in seen:
            seen.add(int(x))
            irreducible.append(int(x))
    irreducible = np.array(irreducible, dtype=np.int64)
    pos = {int(x): k for k, x in enumerate(irreducible)}
    trafos_uc = get_trafos_uc(lat)
    mappings = get_mappings(lat, reduced, trafos_uc)
    N = len(lat.sites)
    overlap = []
    for ir in irreducible:
        cols = np.nonzero(mappings[ir] >= 0)[0]
        order, counts = [], {}
        for j in cols:
            p = (int(reduced[j]), int(mappings[j, ir]))
            if p not in counts:
                counts[p] = 0
                order.append(p)
            counts[p] += 1
        table = np.zeros((len(order), 3), dtype=np.int64)
        for k, p in enumerate(order):
            table[k, 0] = pos[p[0]] + 1
            table[k, 1] = pos[p[1]] + 1
            table[k, 2] = counts[p]
        overlap.append(table)
    mult = np.array([int(np.count_nonzero(reduced == ir)) for ir in irreducible], dtype=np.int64)
    exchange = np.array([pos[int(mappings[ir, 0])] + 1 for ir in irreducible], dtype=np.int64)
    project = np.zeros((N, N), dtype=np.int64)
    lut = np.zeros(N, dtype=np.int64)
    for k, x in enumerate(irreducible):
        lut[x] = k + 1
    valid = mappings >= 0
    project[valid] = lut[mappings[valid]]
    sites = [lat.sites[int(i)] for i in irreducible]
    vecs = lat.vecs[irreducible]
    if verbose:
        print(f"Done. Reduced lattice has {len(sites)} sites.")
    return ReducedLattice(lat.name, lat.size, model, [list(map(float, j)) for j in J], sites, vecs,
                          overlap, mult, exchange, project, irreducible)
