"""The learned parquet warm start on the GPU: kernels against the CPU oracle, and what the trained
network gains over the bare-coupling start (the parquet iteration stays the judge)."""
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))


def test_mlp_kernels_match_oracle(pkg):
    import mlp_oracle as M
    from pffrg_gb300.warmstart import MLP

    rng = np.random.default_rng(1)
    sizes = [3, 24, 16, 5]
    net = MLP(sizes, seed=3)
    p = net.get_params().astype(np.float64)
    X, T = rng.normal(size=(40, 3)), rng.normal(size=(40, 5))
    loss, g = net.gradient(X, T)
    loss_ref, g_ref = M.loss_and_grad(p, sizes, X.astype(np.float32).astype(np.float64),
                                      T.astype(np.float32).astype(np.float64))
    assert loss == pytest.approx(loss_ref, rel=1e-5)
    assert np.max(np.abs(g - g_ref)) <= 1e-5 * np.max(np.abs(g_ref))  # FP32 kernels against FP64
    Y = net.forward(X)
    assert np.allclose(Y, M.forward(p, sizes, X)[-1], rtol=1e-5, atol=1e-6)
    l1 = net.train(X, T, 200, 1e-2)
    assert l1 < 0.5 * loss
    # the decoder behind the network
    basis, mean = rng.normal(size=(5, 1000)), rng.normal(size=1000)
    net.set_decoder(basis, mean)
    x = rng.normal(size=3)
    z = M.forward(net.get_params().astype(np.float64), sizes, x[None, :].astype(np.float32))[-1][0]
    assert np.allclose(net.predict(x), mean + z @ basis, rtol=1e-4, atol=1e-4)


def test_warm_start_saves_parquet_iterations(pkg):
    """Honeycomb J1-J2-J3 Heisenberg on small meshes: a network fitted to converged parquet vertices at
    training couplings starts held-out couplings closer to their fixed point than the bare couplings;
    both starts converge to the same vertex."""
    from pffrg_gb300.launcher import launch
    from pffrg_gb300.warmstart import ParquetWarmStart, coupling_features, vertex_mask

    kw = dict(num_sigma=10, num_omega=4, num_nu=3, num_chi=4, initial=5.0, final=5.0, parquet=True,
              parquet_tol=(1e-8, 1e-8), precision="fp64")
    rng = np.random.default_rng(3)
    J = [[[1.0], [float(a)], [float(b)]] for a, b in rng.uniform(0.0, 0.5, size=(20, 2))]
    train, test = J[:16], J[16:]
    feats, verts = [], []
    for j in train:
        res = launch("", "honeycomb", 3, "heisenberg", "su2", j, **kw)
        feats.append(coupling_features(j))
        verts.append(res.action.buf[vertex_mask(res.action)].copy())
    ws = ParquetWarmStart(k=8, hidden=(32, 32))
    ws.fit(feats, verts, epochs=3000, lr=3e-3)
    bare, warm = [], []
    for j in test:
        r0 = launch("", "honeycomb", 3, "heisenberg", "su2", j, **kw)
        r1 = launch("", "honeycomb", 3, "heisenberg", "su2", j, warm_start=ws, **kw)
        bare.append(r0.parquet_iterations)
        warm.append(r1.parquet_iterations)
        m = vertex_mask(r0.action)
        d = np.max(np.abs(r0.action.buf[m] - r1.action.buf[m])) / np.max(np.abs(r0.action.buf[m]))
        assert d < 1e-5
    print(f"parquet iterations: bare start {bare}, learned start {warm}")
    assert np.mean(warm) < np.mean(bare)
