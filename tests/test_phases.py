"""Several fluid phases (FluidModels of different rest density in one simulation, as the
reference's multiphase scenes use them): per-particle rest density and mass, the pressure
term kappa_i + (rho0_j / rho0_i) kappa_j, and solver iterations that visit the models in turn,
each against its own tolerance (TimeStepDFSPH.cpp:322-339, 476-495).

CPU: a heavy phase under a light one settles, each at its own rest density, in the oracle.
GPU: one step from the same two-phase state meets the oracle at the standard bars (iteration
counts equal), FP32 and FP64; unsupported combinations are refused."""
import numpy as np
import pytest

import oracle
from splishsplash_gb300 import native, scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

from test_gpu_parity import compare, f32

RHO = (1000.0, 500.0)


def layered_scene(counts=(11, 8, 11), velocity=None):
    """a column whose lower half is phase 0 and upper half phase 1: particles ordered by height"""
    sc = scenes.small_block(counts=counts, box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05),
                            velocity=velocity).as_float32()
    order = np.argsort(sc.x[:, 1], kind="stable")
    sc.x, sc.v = sc.x[order].copy(), sc.v[order].copy()
    n0 = sc.n // 2
    return sc, (n0, sc.n - n0)


def test_oracle_two_phase_column_settles_at_each_rest_density():
    sc, counts = layered_scene()
    sim = oracle.OracleSim(sc)
    sim.set_phases(counts, RHO)
    for _ in range(120):
        sim.step()
    rho = sim.density
    for k, (lo, hi) in enumerate(((0, counts[0]), (counts[0], sc.n))):
        inner = rho[lo:hi][rho[lo:hi] > 0.9 * RHO[k]]     # particles with full neighbourhoods
        assert abs(np.median(rho[lo:hi]) / RHO[k] - 1.0) < 0.02
        assert len(inner) > 0.5 * (hi - lo)
    assert sim.x[:, 1].min() > 0.0 and np.all(np.isfinite(sim.v))
    # the heavy phase stays below the light one
    assert np.median(sim.x[:counts[0], 1]) < np.median(sim.x[counts[0]:, 1])


def two_phase_state(counts_xyz=(11, 8, 11), steps=40):
    sc, counts = layered_scene(counts_xyz, velocity=(0.2, -0.3, 0.1))
    pre = oracle.OracleSim(sc)
    pre.set_phases(counts, RHO)
    for _ in range(steps):
        pre.step()
    state = dict(x=f32(pre.x), v=f32(pre.v), kappa=f32(pre.kappa), kappa_v=f32(pre.kappa_v), dt=pre.dt)
    return sc, counts, state


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_scale", [("fp32", 2.0), ("fp64", 1e-4)])
def test_two_phase_step_matches_oracle(precision, tol_scale):
    """one step from a two-phase state: iteration counts equal (each solver iteration visits the
    phases in turn), fields at the FP64 bars, and at twice the FP32 bars (velocity measured 1.5e-4;
    the FP64 run of the same case agrees to the 1e-8 bars, so the gap is float rounding through the
    density ratios); the last pressure accelerations start at zero on both sides, as after an upload"""
    sc, counts, state = two_phase_state()
    ts = TimeStepDFSPH(sc, precision=precision)
    ts.ctx.set_fluid_phases(counts, RHO)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    sim = oracle.OracleSim(sc)
    sim.set_phases(counts, RHO)
    sim.x[:] = state["x"]
    sim.v[:] = state["v"]
    sim.kappa[:] = state["kappa"]
    sim.kappa_v[:] = state["kappa_v"]
    sim.dt = state["dt"]
    st = ts.step()
    sim.step()
    assert sim.stats()["iterations"] >= 2
    compare(ts, sim, st, tol_scale=tol_scale)
    ts.close()


@pytest.mark.gpu
def test_two_phase_runs_follow_the_oracle():
    """ten steps in a row (the phases' last pressure accelerations carried across the sorts):
    iteration counts equal step by step, positions within 1e-5"""
    sc, counts = layered_scene(velocity=(0.2, -0.3, 0.1))
    ts = TimeStepDFSPH(sc, precision="fp64")
    ts.ctx.set_fluid_phases(counts, RHO)
    sim = oracle.OracleSim(sc)
    sim.set_phases(counts, RHO)
    for _ in range(10):
        st = ts.step()
        sim.step()
        assert (st["iterations"], st["iterations_v"]) == (sim.stats()["iterations"], sim.stats()["iterations_v"])
    x = ts.getFluidModel().getFieldBuffer("position")
    assert np.abs(x - sim.x).max() < 1e-5
    ts.close()


@pytest.mark.gpu
def test_phase_refusals():
    def code(fn):
        with pytest.raises(native.SphgbError) as e:
            fn()
        return native.ERR_NAMES[e.value.code]

    sc, counts = layered_scene((6, 6, 6))
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_fluid_phases((counts[0], counts[1] - 1), RHO)
    assert code(ts.step) == "STATE"                                   # counts do not cover the fluid
    assert code(lambda: ts.ctx.set_fluid_phases(counts, (1000.0, -1.0))) == "ARGUMENT"
    p = sc.params
    p.viscosityMethod = 6
    ts.ctx.set_params(p)
    ts.ctx.set_fluid_phases(counts, RHO)
    assert code(ts.step) == "ARGUMENT"                                # Weiler2018 per fluid model
    p.viscosityMethod = 0
    ts.ctx.set_params(p)
    ts.ctx.set_fluid_phases()                                         # back to one phase
    ts.step()
    ts.close()


@pytest.mark.gpu
def test_two_phase_step_in_a_volume_mapped_box_matches_oracle():
    """the phases with the Bender2019 boundary (FP64): iteration counts equal, fields at the bars"""
    sc, counts, state = two_phase_state()
    sc.xb = np.zeros((0, 3))
    ts = TimeStepDFSPH(sc, precision="fp64")
    v, f = scenes.box_mesh((0, 0, 0), (0.6, 0.8, 0.6))
    ts.ctx.add_volume_map(v, f, (12, 16, 12), invert=True)
    ts.ctx.set_boundary_method(2)
    ts.ctx.set_fluid_phases(counts, RHO)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    res, lo, hi, dist, vol = ts.ctx.volume_map(0)
    sim = oracle.OracleSim(sc)
    sim.set_volume_maps([oracle.VolumeMap(res).set_values(lo, hi, dist, vol)])
    sim.set_phases(counts, RHO)
    sim.x[:] = state["x"]
    sim.v[:] = state["v"]
    sim.kappa[:] = state["kappa"]
    sim.kappa_v[:] = state["kappa_v"]
    sim.dt = state["dt"]
    st = ts.step()
    sim.step()
    compare(ts, sim, st, tol_scale=1e-4)
    ts.close()
