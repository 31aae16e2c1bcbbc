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
