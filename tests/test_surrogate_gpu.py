"""Tensor-core surrogate network: the tcgen05 product against numpy, the forward and backward pass
against the NumPy restatement (oracle/mlp_ref.py, same BF16 roundings, float64 elsewhere), and
training that lowers the loss."""
import numpy as np
import pytest

from arbo_gpu_fit_gb300.surrogate import MLP, tc_gemm
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 160, 192), (200, 48, 16), (384, 512, 512)])
def test_tc_gemm_matches_numpy(gpu, M, N, K):
    rng = np.random.default_rng(M + N + K)
    a = rng.standard_normal((M, K)).astype(np.float32)
    b = rng.standard_normal((N, K)).astype(np.float32)
    c, _ = tc_gemm(a, b)
    want = mlp_ref.bf16(a) @ mlp_ref.bf16(b).T
    err = np.abs(c - want).max() / np.abs(want).max()
    assert err < 1e-5, err


def test_gradients_match_restatement(gpu):
    rng = np.random.default_rng(4)
    net = MLP(6, 64, 2, 40, max_batch=64, seed=3)
    x = rng.uniform(-1, 1, (48, 6)).astype(np.float32)
    t = rng.standard_normal((48, 40)).astype(np.float32)
    loss = net.gradients(x, t)
    ws, bs = [], []
    for l in range(net.layers):
        w, b, _, _ = net.layer(l)
        ws.append(w)
        bs.append(b)
    want_loss, dws, dbs, _ = mlp_ref.forward_backward(x, t, ws, bs, net.dims, 40)
    assert loss == pytest.approx(want_loss, rel=1e-4)
    for l in range(net.layers):
        _, _, dw, db = net.layer(l)
        rel_w = np.linalg.norm(dw - dws[l]) / np.linalg.norm(dws[l])
        rel_b = np.linalg.norm(db - dbs[l]) / np.linalg.norm(dbs[l])
        assert rel_w < 2e-3 and rel_b < 2e-3, (l, rel_w, rel_b)


def test_forward_matches_restatement(gpu):
    rng = np.random.default_rng(5)
    net = MLP(6, 128, 3, 96, max_batch=128, seed=9)
    x = rng.uniform(-1, 1, (80, 6)).astype(np.float32)
    ws = [net.layer(l)[0] for l in range(net.layers)]
    bs = [net.layer(l)[1] for l in range(net.layers)]
    y = net.forward(x)
    _, _, _, want = mlp_ref.forward_backward(x, np.zeros((80, 96), np.float32), ws, bs, net.dims, 96)
    assert np.abs(y - want[:, :96]).max() < 1e-3 * max(1.0, np.abs(want).max())


def test_training_lowers_loss(gpu):
    rng = np.random.default_rng(6)
    x = rng.uniform(-1, 1, (1024, 6)).astype(np.float32)
    proj = rng.standard_normal((6, 48)).astype(np.float32)
    t = np.sin(x @ proj).astype(np.float32)
    net = MLP(6, 256, 3, 48, max_batch=256, seed=2)
    first = net.gradients(x[:256], t[:256])
    for ep in range(60):
        for i in range(0, 1024, 256):
            net.train_step(x[i:i + 256], t[i:i + 256], 2e-3)
    last = net.gradients(x[:256], t[:256])
    assert last < 0.1 * first, (first, last)


def test_surrogate_pipeline_on_simulator_runs(gpu):
    # Training data from batched simulator runs, a small network fitted to it, and the
    # surrogate likelihood of observed data: the path delayed acceptance uses.
    from arbo_gpu_fit_gb300 import configs, mcmc
    from arbo_gpu_fit_gb300.surrogate import Surrogate, training_set

    w = configs.scaled(800, 2400, 3, 120, seed=4, sigma=0.3, bitingRate=0.9, nInitialInf=30.0, mInitialInf=90.0)
    theta, inc = training_set(w, 48, 4, seed=1, batch_size=16)
    assert theta.shape == (48, 6) and inc.shape == (48, 4, 4) and inc.sum() > 0
    sur = Surrogate(4, 4, hidden=64, hidden_layers=2, seed=2, max_batch=64)
    losses = sur.fit(theta, inc, epochs=80, batch=16, lr=3e-3)
    assert losses[-1] < 0.5 * losses[0]
    obs = mcmc.synthetic_data(w, theta[0], months=4, seed=2)
    ll = sur.loglik(theta[:5], obs)
    assert ll.shape == (5,) and np.all(np.isfinite(ll))
