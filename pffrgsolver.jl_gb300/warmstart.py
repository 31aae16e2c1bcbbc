"""Learned parquet warm start (no counterpart in the reference).

A small network, trained on the GPU by the library's own kernels
(``pffrg_mlp_*``, csrc/pffrg_mlp.cu), maps a model's normalised couplings to
the leading principal-component coordinates of its converged parquet vertex
(Σ and every channel q at the cutoff of the parquet start); a fixed affine
decoder turns them back into a vertex.  ``launcher.launch(..., warm_start=w)``
starts the parquet iteration of src/Launcher/parquet.jl from that vertex
instead of the bare couplings; the iteration itself, unchanged, decides
convergence, so a poor prediction costs iterations but never changes the
converged result.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi

_fp = ctypes.POINTER(ctypes.c_float)


def _lib():
    L = _capi.load()
    if not getattr(L, "_mlp_typed", False):
        vp = ctypes.c_void_p
        L.pffrg_mlp_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_uint]
        L.pffrg_mlp_create.restype = vp
        L.pffrg_mlp_destroy.argtypes = [vp]
        L.pffrg_mlp_last_error.argtypes = [vp]
        L.pffrg_mlp_last_error.restype = ctypes.c_char_p
        L.pffrg_mlp_num_params.argtypes = [vp]
        L.pffrg_mlp_num_params.restype = ctypes.c_int64
        L.pffrg_mlp_get_params.argtypes = [vp, _fp]
        L.pffrg_mlp_set_params.argtypes = [vp, _fp]
        L.pffrg_mlp_forward.argtypes = [vp, _fp, ctypes.c_int, _fp]
        L.pffrg_mlp_gradient.argtypes = [vp, _fp, _fp, ctypes.c_int, _fp, _fp]
        L.pffrg_mlp_train.argtypes = [vp, _fp, _fp, ctypes.c_int, ctypes.c_int, ctypes.c_float, _fp]
        L.pffrg_mlp_set_decoder.argtypes = [vp, _fp, _fp, ctypes.c_int, ctypes.c_int64]
        L.pffrg_mlp_predict.argtypes = [vp, _fp, _fp]
        L._mlp_typed = True
    return L


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


class MLP:
    """Dense network on the GPU: tanh hidden layers, linear output."""

    def __init__(self, sizes, seed: int = 0):
        self.lib = _lib()
        self.sizes = [int(s) for s in sizes]
        arr = (ctypes.c_int * len(self.sizes))(*self.sizes)
        self.h = self.lib.pffrg_mlp_create(len(self.sizes) - 1, arr, seed)
        if not self.h:
            raise _capi.PffrgError("pffrg_mlp_create failed")

    def _check(self, rc, what):
        if rc != 0:
            raise _capi.PffrgError(f"{what}: {self.lib.pffrg_mlp_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.pffrg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(self.lib.pffrg_mlp_num_params(self.h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, dtype=np.float32)
        self._check(self.lib.pffrg_mlp_get_params(self.h, p.ctypes.data_as(_fp)), "get_params")
        return p

    def set_params(self, p) -> None:
        p = _f32(p)
        self._check(self.lib.pffrg_mlp_set_params(self.h, p.ctypes.data_as(_fp)), "set_params")

    def forward(self, X) -> np.ndarray:
        X = _f32(X)
        Y = np.zeros((X.shape[0], self.sizes[-1]), dtype=np.float32)
        self._check(self.lib.pffrg_mlp_forward(self.h, X.ctypes.data_as(_fp), X.shape[0], Y.ctypes.data_as(_fp)),
                    "forward")
        return Y

    def gradient(self, X, T):
        X, T = _f32(X), _f32(T)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        self._check(self.lib.pffrg_mlp_gradient(self.h, X.ctypes.data_as(_fp), T.ctypes.data_as(_fp), X.shape[0],
                                                g.ctypes.data_as(_fp), loss.ctypes.data_as(_fp)), "gradient")
        return float(loss[0]), g

    def train(self, X, T, epochs: int, lr: float) -> float:
        X, T = _f32(X), _f32(T)
        loss = np.zeros(1, dtype=np.float32)
        self._check(self.lib.pffrg_mlp_train(self.h, X.ctypes.data_as(_fp), T.ctypes.data_as(_fp), X.shape[0],
                                             int(epochs), float(lr), loss.ctypes.data_as(_fp)), "train")
        return float(loss[0])

    def set_decoder(self, basis, mean) -> None:
        basis, mean = _f32(basis), _f32(mean)
        self._check(self.lib.pffrg_mlp_set_decoder(self.h, basis.ctypes.data_as(_fp), mean.ctypes.data_as(_fp),
                                                   basis.shape[0], basis.shape[1]), "set_decoder")
        self._dec_d = basis.shape[1]

    def predict(self, x) -> np.ndarray:
        x = _f32(x)
        out = np.zeros(self._dec_d, dtype=np.float32)
        self._check(self.lib.pffrg_mlp_predict(self.h, x.ctypes.data_as(_fp), out.ctypes.data_as(_fp)), "predict")
        return out


def coupling_features(J) -> np.ndarray:
    """The normalised couplings (launch!'s normalisation, Launcher.jl:647-650), flattened."""
    flat = np.array([float(x) for j in J for x in j])
    n = np.linalg.norm(flat)
    return flat / n if n > 0 else flat


def vertex_mask(a) -> np.ndarray:
    """Entries of an action the warm start predicts: Σ and every channel (not the bare couplings)."""
    m = a.gamma_mask().copy()
    m[:a.layout.num_sigma] = True
    return m


def _poly2(x) -> np.ndarray:
    """1, x_i and x_i x_j (i <= j) of each row of x: the terms of the least-squares part."""
    x = np.atleast_2d(x)
    n = x.shape[1]
    cols = [np.ones(len(x))] + [x[:, i] for i in range(n)] + [x[:, i] * x[:, j] for i in range(n) for j in range(i, n)]
    return np.stack(cols, axis=1)


class ParquetWarmStart:
    """Principal components of converged parquet vertices and a model from the couplings to their
    coordinates: a least-squares part quadratic in the couplings plus the network for the rest (a
    residual head), so the network learns only what the quadratic part misses."""

    def __init__(self, k: int = 16, hidden=(64, 64), seed: int = 0):
        self.k, self.hidden, self.seed = k, tuple(hidden), seed
        self.net = None

    def fit(self, features, vertices, epochs: int = 4000, lr: float = 3e-3) -> float:
        X = np.asarray(features, dtype=np.float64)
        V = np.asarray(vertices, dtype=np.float64)
        self.x_mean, self.x_std = X.mean(axis=0), X.std(axis=0) + 1e-12
        Xn = (X - self.x_mean) / self.x_std
        self.mean = V.mean(axis=0)
        U, S, Vt = np.linalg.svd(V - self.mean, full_matrices=False)
        k = min(self.k, Vt.shape[0])
        self.basis = Vt[:k]                             # [k, D], orthonormal rows
        Z = (V - self.mean) @ self.basis.T              # principal coordinates
        # quadratic part of the coordinates (least squares), the network fits the remainder
        Xa = _poly2(Xn)
        self.lin, *_ = np.linalg.lstsq(Xa, Z, rcond=None)
        Zr = Z - Xa @ self.lin
        self.z_scale = Zr.std(axis=0) + 1e-12
        sizes = [X.shape[1], *self.hidden, k]
        self.net = MLP(sizes, self.seed)
        loss = self.net.train(Xn, Zr / self.z_scale, epochs, lr)
        # the decoder undoes the coordinate scaling: vertex = mean + (z / scale) (scale basis)
        self.net.set_decoder(self.basis * self.z_scale[:, None], self.mean)
        return loss

    def predict(self, feature, part: str = "full") -> np.ndarray:
        """The predicted vertex; ``part`` selects what predicts it, for ablations: "full" (the
        least-squares part plus the network), "lsq" (the least-squares part alone) or "mean" (the
        mean of the training vertices)."""
        x = (np.asarray(feature, dtype=np.float64) - self.x_mean) / self.x_std
        if part == "mean":
            return self.mean.copy()
        z_lin = (_poly2(x) @ self.lin)[0]
        if part == "lsq":
            return self.mean + z_lin @ self.basis
        if part != "full":
            raise ValueError(f"unknown part {part!r}")
        return self.net.predict(x).astype(np.float64) + z_lin @ self.basis
