"""Batched scenes: many independent scenes in one context advance exactly like the same
scenes in separate contexts (per-scene grids, CFL step sizes, solver iteration counts and
convergence), in graph and host-loop mode, with and without Weiler2018 viscosity."""
import dataclasses

import numpy as np
import pytest

from splishsplash_gb300 import scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

pytestmark = pytest.mark.gpu

FIELDS = ["position", "velocity", "density", "p / rho^2", "p_v / rho^2", "factor"]


def _batch(viscosity=False):
    sc = [scenes.small_block(counts=(10, 10, 10), seed=1, velocity=(6.0, 0.0, 0.0), viscosity=viscosity),
          scenes.small_block(counts=(7, 12, 9), seed=2, box=(1.0, 1.2, 0.9), velocity=(-3.0, 2.0, 4.0),
                             viscosity=viscosity),
          scenes.small_block(counts=(5, 5, 5), seed=3, box=(0.6, 0.6, 0.6), viscosity=viscosity)]
    # the batch shares the first scene's parameter block
    for s in sc[1:]:
        s.params = dataclasses.replace(sc[0].params)
    return sc


def _run_single(sc, steps, use_graph=True, lanes=1):
    ts = TimeStepDFSPH(sc, use_graph=use_graph)
    ts.ctx.set_lanes_per_particle(lanes)   # same summation order as the batch
    stats = [ts.step() for _ in range(steps)]
    out = {f: ts.getFluidModel().getFieldBuffer(f, np.float64) for f in FIELDS}
    ts.close()
    return stats, out


@pytest.mark.parametrize("viscosity,lanes", [(False, 1), (True, 1), (False, 4), (True, 2)])
def test_batch_matches_separate_contexts_bitwise(viscosity, lanes):
    sc = _batch(viscosity)
    steps = 12
    b = BatchedTimeStepDFSPH(sc, use_graph=True)
    b.ctx.set_lanes_per_particle(lanes)
    for _ in range(steps):
        agg = b.step()
    per = b.scene_stats()
    fields = {f: b.getFieldBuffer(f, np.float64) for f in FIELDS}
    b.close()
    iters = []
    for k, s in enumerate(sc):
        stats, ref = _run_single(s, steps, lanes=lanes)
        st = stats[-1]
        for key in ("iterations", "iterations_v", "visco_iterations", "dt_used", "dt_next", "time",
                    "avg_density_err", "avg_density_err_v", "max_fluid_neighbors", "max_boundary_neighbors"):
            assert per[k][key] == st[key], (k, key, per[k][key], st[key])
        for f in FIELDS:
            np.testing.assert_array_equal(fields[f][k], ref[f], err_msg=f"scene {k} field {f}")
        iters.append(st["iterations"])
    assert agg["iterations"] == max(iters)
    # the scenes move at different speeds, so their CFL step sizes differ
    assert len({p["dt_used"] for p in per}) == len(sc)


def test_batch_host_loops_match_graph():
    sc = _batch()
    out = []
    for g in (True, False):
        b = BatchedTimeStepDFSPH(sc, use_graph=g)
        b.ctx.set_lanes_per_particle(4)
        for _ in range(8):
            b.step()
        out.append((b.scene_stats(), b.ctx.download("position"), b.ctx.download("velocity")))
        b.close()
    assert [s["iterations"] for s in out[0][0]] == [s["iterations"] for s in out[1][0]]
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


def test_ensemble_batch_reaches_tolerance_per_scene():
    ens = scenes.ensemble(num_scenes=12, seed=5, n_min=2000, n_max=8000)
    b = BatchedTimeStepDFSPH(ens, use_graph=True)
    tol = ens[0].params.maxError * 0.01 * ens[0].params.density0
    for _ in range(25):
        agg = b.step()
        assert agg["flags"] == 0
        for p in b.scene_stats():
            assert p["avg_density_err"] <= tol + 1e-9 or p["iterations"] == ens[0].params.maxIterations
    n, nb = b.ctx.num_particles()
    assert n == sum(s.n for s in ens) and nb == sum(s.nb for s in ens)
    x = b.getFieldBuffer("position")
    for s, xs in zip(ens, x):
        assert np.isfinite(xs).all()
        assert (xs >= s.box_min - 0.05).all() and (xs <= s.box_max + 0.05).all()
    b.close()
