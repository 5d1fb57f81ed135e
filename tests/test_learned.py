"""Learned warm start inside the DFSPH step: the fallback rule and the gain of a trained
network over the classic warm start (both iterate to the same tolerances)."""
import numpy as np
import pytest

from splishsplash_gb300 import learned, native, scenes
from splishsplash_gb300.dfsph import TimeStepDFSPH

pytestmark = pytest.mark.gpu


def test_features_are_collected_and_finite():
    sc = scenes.small_block(counts=(10, 10, 10))
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_feature_output(True)
    for _ in range(5):
        ts.step()
    X = ts.ctx.download("features", np.float32)
    assert X.shape == (sc.n, 10) and np.isfinite(X).all()
    # the neighbour means lie inside the range of the raw features
    for k in range(5):
        assert X[:, 5 + k].min() >= X[:, k].min() - 1e-5 and X[:, 5 + k].max() <= X[:, k].max() + 1e-5
    ts.close()


def test_fallback_keeps_classic_warm_start_when_prediction_is_worse():
    """An untrained network with large outputs: the predicted warm start may be used only in
    solves where its initial residual is lower, and the solves still reach their tolerance."""
    rng = np.random.default_rng(0)
    net = native.Mlp(seed=11)
    p = net.params()
    p *= 20.0
    net.set_params(p + rng.normal(0, 0.5, size=p.size).astype(np.float32) * (p != 0))
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 1.0, 0.8))
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_warmstart_mlp(net)
    for _ in range(40):
        st = ts.step()
        for k in range(2):
            if st["learned_used"] & (1 << k):
                assert st["ws_residual_learned"][k] < st["ws_residual_classic"][k]
        assert st["avg_density_err"] <= 0.01 * 0.01 * 1000 + 1e-9 or st["iterations"] == 100
    ts.close()
    net.close()


def test_trained_network_gain_over_classic_warm_start():
    ens = scenes.ensemble(num_scenes=8, seed=77, n_min=4000, n_max=12000)
    X, Y = learned.collect(ens[:6], steps=60, warmup=10, stride=3, frac=0.5)
    net, losses = learned.train(X, Y, epochs=25)
    assert losses[-1] < losses[0]
    res = learned.evaluate(ens[6], net, steps=120)
    print("learned warm start gain:", res["gain"], res["plain"], res["learned"])
    # the network must not cost iterations: with the residual fallback it is used only when it helps
    assert res["learned"]["solver_iterations_total"] <= 1.05 * res["plain"]["solver_iterations_total"]
    assert res["learned"]["final_avg_density_error_percent"] <= 0.01 + 1e-9
    net.close()
