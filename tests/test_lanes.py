"""Lanes per particle of the neighbour passes: every variant (1, 2, 4 lanes, with the matching
fluid-list layout) gives the same neighbour sets and the same step within FP32 summation-order
tolerance, and the autotuner's trial steps leave no trace in the simulation."""
import numpy as np
import pytest

from splishsplash_gb300 import scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

pytestmark = pytest.mark.gpu


def _run(sc, lanes, steps, viscosity_fields=False):
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_lanes_per_particle(lanes)
    st = [ts.step() for _ in range(steps)]
    m = ts.getFluidModel()
    out = {f: m.getFieldBuffer(f) for f in ("position", "velocity", "density", "factor", "p / rho^2", "p_v / rho^2")}
    nbr = ts.ctx.neighbors(0)
    assert ts.ctx.lanes_per_particle()[0] == lanes
    ts.close()
    return st, out, nbr


@pytest.mark.parametrize("viscosity", [False, True])
def test_lane_variants_agree(viscosity):
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 1.0, 0.8), viscosity=viscosity)
    ref_st, ref, ref_nbr = _run(sc, 1, 3)
    for lanes in (2, 4):
        st, out, nbr = _run(sc, lanes, 3)
        off0, idx0 = ref_nbr
        off1, idx1 = nbr
        np.testing.assert_array_equal(off0, off1)
        for i in range(sc.n):
            np.testing.assert_array_equal(np.sort(idx0[off0[i]:off0[i + 1]]), np.sort(idx1[off1[i]:off1[i + 1]]))
        np.testing.assert_allclose(out["density"], ref["density"], rtol=2e-6)
        np.testing.assert_allclose(out["velocity"], ref["velocity"], rtol=0, atol=1e-5)
        np.testing.assert_allclose(out["position"], ref["position"], rtol=0, atol=1e-7)
        assert [s["iterations"] for s in st] == [s["iterations"] for s in ref_st]


def test_autotune_trials_are_undone():
    sc = scenes.small_block(counts=(14, 14, 14), box=(0.9, 1.0, 0.9), velocity=(0.5, 0.0, 0.0))
    a = TimeStepDFSPH(sc)
    sa = [a.step() for _ in range(10)]
    lanes, trial_ms = a.ctx.lanes_per_particle()
    assert lanes in (1, 2, 4) and all(t > 0 for t in trial_ms)
    threads, nt_ms = a.ctx.solver_block_threads()
    assert threads in (128, 256, 512) and all(t > 0 for t in nt_ms)
    b = TimeStepDFSPH(sc)
    b.ctx.set_lanes_per_particle(lanes)
    b.ctx.set_solver_block_threads(threads)
    sb = [b.step() for _ in range(10)]
    for f in ("position", "velocity", "p / rho^2"):
        np.testing.assert_array_equal(a.getFluidModel().getFieldBuffer(f), b.getFluidModel().getFieldBuffer(f))
    for x, y in zip(sa, sb):
        assert x["iterations"] == y["iterations"] and x["time"] == y["time"] and x["dt_used"] == y["dt_used"]
    a.close()
    b.close()


def test_batch_lane_variants_agree():
    ens = scenes.ensemble(num_scenes=5, seed=9, n_min=2000, n_max=5000)
    res = []
    for lanes in (1, 4):
        b = BatchedTimeStepDFSPH(ens)
        b.ctx.set_lanes_per_particle(lanes)
        for _ in range(3):
            b.step()
        res.append((b.scene_stats(), b.ctx.download("density")))
        b.close()
    assert [s["iterations"] for s in res[0][0]] == [s["iterations"] for s in res[1][0]]
    np.testing.assert_allclose(res[0][1], res[1][1], rtol=2e-6)


@pytest.mark.parametrize("batch", [False, True])
def test_solver_block_sizes_agree(batch):
    """The one-lane solver passes at 128, 256 and 512 threads per block (512: one scene) compute
    every particle's sums in the same order.  The FP64 error sums add the block partials in
    another grouping, and each block size is its own compiled instance of the passes, whose
    floating-point contractions may differ in the last bit.  One scene: the same iteration
    counts and step sizes, positions to 1e-9 m, velocities to 1e-6 m/s, kappa to 1e-5.  A batch
    takes one decision per scene and iteration, and one of them may fall on the other side of
    its tolerance under the other grouping (the batch's largest counts and step sizes stay
    equal): positions to 1e-6 m, velocities to 1e-4 m/s, kappa to 1e-3."""
    if batch:
        sc = scenes.ensemble(num_scenes=4, seed=3, n_min=2000, n_max=6000)
        make = lambda: BatchedTimeStepDFSPH(sc)
        sizes = (128, 256)
    else:
        sc = scenes.small_block(counts=(14, 14, 14), box=(0.9, 1.0, 0.9), velocity=(0.5, 0.0, 0.0))
        make = lambda: TimeStepDFSPH(sc)
        sizes = (128, 256, 512)
    runs = []
    for nt in sizes:
        t = make()
        t.ctx.set_lanes_per_particle(1)
        t.ctx.set_neighbor_staging(1)
        t.ctx.set_solver_block_threads(nt)
        st = [t.step() for _ in range(8)]
        assert t.ctx.solver_block_threads()[0] == nt
        runs.append(([(s["iterations"], s["iterations_v"], s["dt_used"]) for s in st],
                     t.ctx.download("position"), t.ctx.download("velocity"), t.ctx.download("p / rho^2")))
        t.close()
    tol = (1e-6, 1e-4, 1e-3) if batch else (1e-9, 1e-6, 1e-5)
    for r in runs[1:]:
        assert r[0] == runs[0][0]
        np.testing.assert_allclose(r[1], runs[0][1], rtol=0, atol=tol[0])
        np.testing.assert_allclose(r[2], runs[0][2], rtol=0, atol=tol[1])
        np.testing.assert_allclose(r[3], runs[0][3], rtol=tol[2], atol=tol[2] * float(np.max(np.abs(runs[0][3]))))


def test_solver_block_threads_are_checked():
    """Sizes other than 0, 128, 256 and 512 are refused, and 512 on a batch (its blocks would span
    two scenes' tiles); the refusals leave the context usable."""
    from splishsplash_gb300 import native
    ts = TimeStepDFSPH(scenes.small_block(counts=(6, 6, 6)))
    with pytest.raises(native.SphgbError):
        ts.ctx.set_solver_block_threads(100)
    ts.ctx.set_solver_block_threads(512)
    ts.step()
    assert ts.ctx.solver_block_threads()[0] in (256, 512)
    ts.close()
    b = BatchedTimeStepDFSPH(scenes.ensemble(num_scenes=2, seed=4, n_min=2000, n_max=3000))
    with pytest.raises(native.SphgbError):
        b.ctx.set_solver_block_threads(512)
    b.ctx.set_solver_block_threads(128)
    b.step()
    b.close()
