"""Edge cases and error paths of the C ABI on the GPU: a single particle, a fluid without
boundary and an empty fluid; ragged batches; neighbour-list capacity, grid limits, out-of-order
calls and invalid inputs, each reported as its status code with the context still usable."""
import numpy as np
import pytest

import oracle
from splishsplash_gb300 import native, scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

from test_gpu_parity import relv

pytestmark = pytest.mark.gpu

ERR = {v: k for k, v in native.ERR_NAMES.items()}


def code_of(fn):
    with pytest.raises(native.SphgbError) as e:
        fn()
    return native.ERR_NAMES[e.value.code]


def context(sc, **kw):
    ctx = native.Context(precision="fp32", **kw)
    ctx.set_params(sc.params)
    return ctx


def test_step_before_upload_and_of_an_empty_fluid():
    sc = scenes.small_block(counts=(4, 4, 4)).as_float32()
    ctx = context(sc)
    assert code_of(ctx.step) == "STATE"
    ctx.upload_boundary(sc.xb)
    ctx.upload_fluid(np.zeros((0, 3)), np.zeros((0, 3)))
    assert code_of(ctx.step) == "STATE"
    ctx.upload_fluid(sc.x, sc.v)          # usable again after the error
    assert ctx.step()["time"] > 0.0
    ctx.close()


def test_invalid_uploads_are_rejected():
    sc = scenes.small_block(counts=(4, 4, 4)).as_float32()
    ctx = context(sc)
    x = sc.x.copy()
    x[3, 1] = np.nan
    assert code_of(lambda: ctx.upload_fluid(x, sc.v)) == "NONFINITE"
    xb = sc.xb.copy()
    xb[0, 0] = np.inf
    assert code_of(lambda: ctx.upload_boundary(xb)) == "NONFINITE"
    ids = np.arange(sc.n, dtype=np.uint32)
    ids[1] = ids[0]                        # not a permutation
    assert code_of(lambda: ctx.upload_fluid(sc.x, sc.v, ids)) == "ARGUMENT"
    ctx.close()


def test_neighbor_capacity_overflow_is_reported():
    sc = scenes.small_block(counts=(10, 10, 10)).as_float32()
    ctx = context(sc, max_fluid_neighbors=8)
    ctx.upload_boundary(sc.xb)
    ctx.upload_fluid(sc.x, sc.v)
    assert code_of(ctx.step) == "CAPACITY"
    ctx.close()


def test_scene_beyond_the_grid_limit_is_reported():
    sc = scenes.small_block(counts=(4, 4, 4)).as_float32()
    sc.params.particleRadius = 0.0002     # 2 m box / 0.0008 m cells > 1024 cells per axis
    xb = np.array([[0.0, 0.0, 0.0], [2.0, 2.0, 2.0]])
    ctx = context(sc)
    ctx.upload_boundary(xb)
    ctx.upload_fluid(sc.x, sc.v)
    assert code_of(ctx.step) == "GRID"
    ctx.close()


def test_batch_rejects_an_empty_scene():
    a = scenes.small_block(counts=(6, 6, 6)).as_float32()
    ctx = context(a)
    assert code_of(lambda: ctx.upload_scenes([a.x, np.zeros((0, 3))], [a.v, np.zeros((0, 3))],
                                             [a.xb, a.xb])) == "ARGUMENT"
    ctx.close()


@pytest.mark.parametrize("case", ["single particle", "no boundary"])
def test_degenerate_scenes_match_the_oracle(case):
    sc = scenes.small_block(counts=(8, 8, 8)).as_float32()
    if case == "single particle":
        sc.x, sc.v = sc.x[:1].copy(), sc.v[:1].copy()
    else:
        sc.xb = np.zeros((0, 3))
    ts = TimeStepDFSPH(sc, use_graph=False)
    sim = oracle.OracleSim(sc)
    for _ in range(5):
        st = ts.step()
        sim.step()
        assert st["iterations"] == sim.stats()["iterations"]
        assert st["iterations_v"] == sim.stats()["iterations_v"]
    m = ts.getFluidModel()
    assert relv(m.getFieldBuffer("velocity"), sim.v, 1e-3) < 1e-4
    assert np.max(np.abs(m.getFieldBuffer("position") - sim.x)) < 1e-6
    ts.close()


def test_ragged_batch_with_a_scene_without_boundary():
    a = scenes.small_block(counts=(9, 7, 5), seed=21).as_float32()
    b = scenes.small_block(counts=(3, 3, 3), seed=22).as_float32()
    b.xb = np.zeros((0, 3))
    b.params = a.params
    batch = BatchedTimeStepDFSPH([a, b])
    batch.ctx.set_lanes_per_particle(1)
    for _ in range(8):
        batch.step()
    pos = batch.getFieldBuffer("position")
    batch.close()
    for k, sc in enumerate((a, b)):
        ts = TimeStepDFSPH(sc)
        ts.ctx.set_lanes_per_particle(1)
        for _ in range(8):
            ts.step()
        np.testing.assert_array_equal(pos[k], ts.getFluidModel().getFieldBuffer("position"))
        ts.close()
