"""Neighbourhood staging of the solver passes (FP32, one lane per particle).

The staged pressure-acceleration and Jacobi passes copy their block's neighbourhood into
shared memory and walk 16-bit local lists that the list build writes in the order of the
fluid lists.  Their sums are therefore bitwise those of the unstaged passes: the tests compare
whole trajectories bit for bit, single scene (graph and host loops) and batch, and check that
the dense blocks of a scene are staged and that the autotuner times the staged candidate.
"""
import numpy as np
import pytest

from splishsplash_gb300 import scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "p / rho^2", "p_v / rho^2", "density")


def run(sc, mode, steps, use_graph=True, precision="fp32"):
    ts = TimeStepDFSPH(sc, use_graph=use_graph, precision=precision)
    ts.ctx.set_lanes_per_particle(1)
    ts.ctx.set_neighbor_staging(mode)
    stats = [ts.step() for _ in range(steps)]
    m = ts.getFluidModel()
    out = {f: m.getFieldBuffer(f) for f in FIELDS}
    info = ts.ctx.neighbor_staging()
    ts.close()
    return out, [(s["iterations"], s["iterations_v"], s["visco_iterations"]) for s in stats], info


@pytest.mark.parametrize("use_graph", [True, False])
def test_staged_passes_are_bitwise_the_unstaged_ones(use_graph):
    sc = scenes.small_block(counts=(16, 20, 16), box=(1.2, 1.4, 1.2), viscosity=True,
                            velocity=(0.4, 0.0, -0.3)).as_float32()
    a, ia, info_a = run(sc, 2, 30, use_graph)
    b, ib, info_b = run(sc, 1, 30, use_graph)
    assert info_a[0] and not info_b[0]
    assert info_a[1] > 0.9, info_a          # dense block: nearly every block staged
    assert ia == ib
    for f in FIELDS:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_staged_batch_matches_unstaged_separate_contexts():
    scs = [scenes.small_block(counts=(10, 12, 10), box=(0.8, 1.0, 0.8), seed=s, viscosity=True).as_float32()
           for s in (3, 4)]
    scs[1].params = scs[0].params
    batch = BatchedTimeStepDFSPH(scs)
    batch.ctx.set_lanes_per_particle(1)
    batch.ctx.set_neighbor_staging(2)
    for _ in range(12):
        batch.step()
    assert batch.ctx.neighbor_staging()[0]
    pos = batch.getFieldBuffer("position")
    batch.close()
    for k, sc in enumerate(scs):
        out, _, _ = run(sc, 1, 12)
        np.testing.assert_array_equal(pos[k], out["position"])


def test_autotuner_times_the_staged_candidate():
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 1.0, 0.8)).as_float32()
    ts = TimeStepDFSPH(sc)
    ts.step()
    active, frac, trial = ts.ctx.neighbor_staging()
    lanes, trials = ts.ctx.lanes_per_particle()
    assert trial > 0.0 and all(t > 0.0 for t in trials)
    assert active == (trial < min(trials))      # the fastest candidate wins, ties to the unstaged one
    if active:
        assert lanes == 1
    ts.close()


def test_fp64_context_ignores_staging():
    sc = scenes.small_block(counts=(8, 8, 8)).as_float32()
    a, ia, info = run(sc, 2, 5, precision="fp64")
    b, ib, _ = run(sc, 1, 5, precision="fp64")
    assert not info[0]
    assert ia == ib
    np.testing.assert_array_equal(a["position"], b["position"])
