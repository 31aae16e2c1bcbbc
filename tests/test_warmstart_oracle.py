"""The CPU restatement of the warm-start network against finite differences (CPU only)."""
import numpy as np


def test_mlp_oracle_gradient_matches_finite_differences(O):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import mlp_oracle as M

    rng = np.random.default_rng(0)
    sizes = [3, 7, 5, 4]
    n = sum(a * b + b for a, b in zip(sizes[:-1], sizes[1:]))
    p = rng.normal(scale=0.5, size=n)
    X, T = rng.normal(size=(6, 3)), rng.normal(size=(6, 4))
    loss, g = M.loss_and_grad(p, sizes, X, T)
    h = 1e-6
    fd = np.array([(M.loss_and_grad(p + h * e, sizes, X, T)[0] - M.loss_and_grad(p - h * e, sizes, X, T)[0]) / (2 * h)
                   for e in np.eye(n)])
    assert np.allclose(g, fd, rtol=1e-6, atol=1e-9)
    assert loss == np.mean((M.forward(p, sizes, X)[-1] - T) ** 2)


def test_quadratic_part_reproduces_a_quadratic_map(pkg):
    """The least-squares part of the warm start: coordinates that are a quadratic function of the
    couplings are reproduced exactly, so the network only sees what is beyond second order."""
    from pffrg_gb300.warmstart import _poly2

    rng = np.random.default_rng(4)
    X = rng.normal(size=(40, 3))
    P = _poly2(X)
    assert P.shape == (40, 10)
    assert np.allclose(P[:, 0], 1.0) and np.allclose(P[:, 1:4], X) and np.allclose(P[:, 4], X[:, 0] ** 2)
    coef = rng.normal(size=(10, 5))
    Z = P @ coef
    fit, *_ = np.linalg.lstsq(P, Z, rcond=None)
    assert np.allclose(P @ fit, Z, atol=1e-10)
    assert np.allclose(_poly2(X[0]), P[:1])
