"""Warm-start network: the tensor-core forward pass and the hand-written backward pass
against the FP64 restatement in oracle/mlp_oracle.py (same BF16 roundings), and Adam
training on a synthetic regression."""
import numpy as np
import pytest

import mlp_oracle
from splishsplash_gb300 import native

pytestmark = pytest.mark.gpu


def random_params(rng, scale=0.3):
    p = np.zeros(mlp_oracle.N_PARAMS, np.float32)
    p[:] = rng.normal(0, scale, size=p.size)
    # the padding stays zero, as the device keeps it
    W1 = p[mlp_oracle.OFF_W1:mlp_oracle.OFF_B1].reshape(64, 16)
    W1[:, 10:] = 0
    W3 = p[mlp_oracle.OFF_W3:mlp_oracle.OFF_B3].reshape(8, 64)
    W3[2:] = 0
    p[mlp_oracle.OFF_B3 + 2:] = 0
    return p


def test_forward_matches_oracle():
    rng = np.random.default_rng(0)
    net = native.Mlp(seed=3)
    p = random_params(rng)
    net.set_params(p)
    X = rng.normal(0, 1, size=(1000, 10)).astype(np.float32)   # not a multiple of 16 rows
    Y = net.forward(X)
    Yr, _ = mlp_oracle.forward(p, X)
    err = np.abs(Y - Yr)
    assert np.mean(err) < 2e-3 * np.mean(np.abs(Yr))
    assert np.max(err) < 3e-2 * np.max(np.abs(Yr))
    net.close()


def test_gradients_match_oracle():
    rng = np.random.default_rng(1)
    net = native.Mlp(seed=4)
    p = random_params(rng)
    net.set_params(p)
    X = rng.normal(0, 1, size=(777, 10)).astype(np.float32)
    T = rng.normal(0, 1, size=(777, 2)).astype(np.float32)
    M = (rng.uniform(size=(777, 2)) > 0.3).astype(np.float32)
    loss, g = net.loss_grad(X, T, M)
    loss_r, g_r = mlp_oracle.loss_grad(p, X, T, M)
    assert loss == pytest.approx(loss_r, rel=1e-2)
    for a, b in ((mlp_oracle.OFF_W1, mlp_oracle.OFF_B1), (mlp_oracle.OFF_B1, mlp_oracle.OFF_W2),
                 (mlp_oracle.OFF_W2, mlp_oracle.OFF_B2), (mlp_oracle.OFF_B2, mlp_oracle.OFF_W3),
                 (mlp_oracle.OFF_W3, mlp_oracle.OFF_B3), (mlp_oracle.OFF_B3, mlp_oracle.N_PARAMS)):
        rel = np.linalg.norm(g[a:b] - g_r[a:b]) / max(np.linalg.norm(g_r[a:b]), 1e-12)
        assert rel < 2e-2, (a, b, rel)
    net.close()


def test_adam_training_fits_a_smooth_target():
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, size=(20000, 10)).astype(np.float32)
    T = np.stack([np.sin(2 * X[:, 0]) + 0.5 * X[:, 1] * X[:, 2], np.tanh(X[:, 3] - X[:, 4])], 1).astype(np.float32)
    net = native.Mlp(seed=5)
    losses = net.train(X, T, epochs=30, batch=1024, lr=1e-3)
    assert losses[-1] < 0.1 * losses[0]
    Y = net.forward(X[:2000])
    assert np.mean((Y - T[:2000]) ** 2) < 0.02
    net.close()
