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
    for k in (0, 1, 2, 4):
        assert X[:, 5 + k].min() >= X[:, k].min() - 1e-5 and X[:, 5 + k].max() <= X[:, k].max() + 1e-5
    # feature 3: previous kappa relative to its neighbourhood mean; its mean column is the
    # weighted fraction of the neighbourhood that carried pressure
    assert (X[:, 3] >= 0).all() and (X[:, 8] >= 0).all() and (X[:, 8] <= 1 + 1e-6).all()
    ts.close()


def _constant_network(m_v, m_p):
    """All weights zero, output biases = the multipliers: the network outputs (m_v, m_p)."""
    net = native.Mlp(seed=3)
    p = np.zeros(net.n_params, np.float32)
    p[5760] = m_v   # b3[0]
    p[5761] = m_p   # b3[1]
    net.set_params(p)
    net.set_output_scale(1.0, 1.0)
    return net


def test_multiplier_one_half_reproduces_the_classic_warm_start():
    """A network that outputs the classic factor 0.5 gives the classic warm start: the fused
    selection (first Jacobi iteration of both candidates) must then match the plain solver."""
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 1.0, 0.8))
    runs = []
    for net in (None, _constant_network(0.5, 0.5)):
        ts = TimeStepDFSPH(sc)
        if net is not None:
            ts.ctx.set_warmstart_mlp(net)
            ts.ctx.set_warmstart_gate(1, 2)   # gate within the iterations the plain solver runs anyway
        st = [ts.step() for _ in range(30)]
        runs.append((st, ts.getFluidModel().getFieldBuffer("position"), ts.getFluidModel().getFieldBuffer("velocity")))
        ts.close()
    (s0, x0, v0), (s1, x1, v1) = runs
    assert all(b["learned_used"] == 0 for b in s1)   # equal residuals: the classic candidate is kept
    same = np.mean([a["iterations"] == b["iterations"] and a["iterations_v"] == b["iterations_v"] for a, b in zip(s0, s1)])
    assert same >= 0.9
    np.testing.assert_allclose(x1, x0, rtol=0, atol=1e-5)
    np.testing.assert_allclose(v1, v0, rtol=0, atol=1e-3)


def test_full_previous_kappa_cuts_pressure_iterations_on_a_settling_column():
    """Multiplier 1 (the full previous kappa instead of half of it) on a column at rest: the
    converged kappa barely changes between steps, so the predicted warm start wins the
    residual check and the pressure solve needs fewer iterations at the same tolerance."""
    sc = scenes.small_block(counts=(14, 24, 14), box=(0.9, 1.5, 0.9), corner=(0.1, 0.05, 0.1))
    out = []
    for net in (None, _constant_network(0.5, 1.0)):
        ts = TimeStepDFSPH(sc)
        if net is not None:
            ts.ctx.set_warmstart_mlp(net)
        st = [ts.step() for _ in range(150)]
        out.append(st[50:])
        ts.close()
    plain = sum(s["iterations"] for s in out[0])
    learned = sum(s["iterations"] for s in out[1])
    used = np.mean([(s["learned_used"] & 2) > 0 for s in out[1]])
    print("pressure iterations plain", plain, "multiplier 1", learned, "used", used)
    assert used > 0.5
    assert learned < plain
    for s in out[1]:
        assert s["avg_density_err"] <= 0.01 * 0.01 * 1000 + 1e-9 or s["iterations"] == 100


@pytest.mark.parametrize("gate", [0, 1])
def test_fallback_keeps_classic_warm_start_when_prediction_is_worse(gate):
    """An untrained network with large outputs (multipliers up to the limit 4): the predicted
    warm start may be used only in solves where its initial residual is lower, and the solves
    still reach their tolerance."""
    rng = np.random.default_rng(0)
    net = native.Mlp(seed=11)
    p = net.params()
    p *= 20.0
    net.set_params(p + rng.normal(0, 0.5, size=p.size).astype(np.float32) * (p != 0))
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 1.0, 0.8))
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_warmstart_mlp(net)
    ts.ctx.set_warmstart_gate(gate, gate)
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
    X, T, W = learned.collect(ens[:6], steps=60, warmup=10, stride=3, frac=0.5)
    assert X.shape[0] == T.shape[0] == W.shape[0] and (W >= 0).all() and (T >= 0).all()
    net, losses = learned.train(X, T, W, epochs=25)
    assert losses[-1] < losses[0]
    res = learned.evaluate(ens[6], net, steps=120, strict=False)
    print("learned warm start gain:", res["gain"], res["plain"], res["learned"])
    # the network must not cost iterations: with the residual fallback it is used only when it helps
    assert res["learned"]["solver_iterations_total"] <= 1.05 * res["plain"]["solver_iterations_total"]
    assert res["learned"]["final_avg_density_error_percent"] <= 0.01 + 1e-9
    net.close()
