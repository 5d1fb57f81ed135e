"""Several fluid phases (FluidModels of different rest density in one simulation, as the
reference's multiphase scenes use them): per-particle rest density and mass, the pressure
term kappa_i + (rho0_j / rho0_i) kappa_j, and solver iterations that visit the models in turn,
each against its own tolerance (TimeStepDFSPH.cpp:322-339, 476-495).

Weiler2018 viscosity solves one system per phase over same-phase neighbours (the reference's
viscosity is a per-model force, Viscosity_Weiler2018.cpp:288-289, 891-936).

CPU: a heavy phase under a light one settles, each at its own rest density, in the oracle; two
far-apart copies of one block as two phases of equal rest density step as one phase does, Weiler
iterations doubled.
GPU: one step from the same two-phase state meets the oracle at the standard bars (iteration
counts equal), FP32 and FP64, with and without Weiler2018 viscosity; unsupported combinations are
refused."""
import numpy as np
import pytest

import oracle
from splishsplash_gb300 import native, scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

from test_gpu_parity import compare, f32

RHO = (1000.0, 500.0)


def layered_scene(counts=(11, 8, 11), velocity=None, viscosity=False):
    """a column whose lower half is phase 0 and upper half phase 1: particles ordered by height"""
    sc = scenes.small_block(counts=counts, box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05),
                            velocity=velocity, viscosity=viscosity).as_float32()
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


def test_oracle_weiler_far_apart_copies_step_as_one_phase():
    """two copies of one block, farther apart than the support radius, without walls: as two phases
    of equal rest density their Weiler systems are the one system's two halves (each reaches the
    same iteration count, the sum is twice it), and the step agrees with the one-phase step up to
    the summation order of the CG reductions"""
    sc = scenes.small_block(counts=(6, 6, 6), viscosity=True).as_float32()
    sc.params.viscosity = 0.05
    rng = np.random.default_rng(3)
    v0 = rng.normal(0.0, 0.3, sc.x.shape).astype(np.float32)
    shift = np.array([0.0, 0.0, 1.0], np.float32)      # 1.0 >> support radius
    sc.x = np.concatenate([sc.x, sc.x + shift]).astype(np.float32)
    sc.v = np.concatenate([v0, v0]).astype(np.float32)
    sc.xb = np.zeros((0, 3))
    one = oracle.OracleSim(sc)
    two = oracle.OracleSim(sc)
    two.set_phases((sc.n // 2, sc.n // 2), (1000.0, 1000.0))
    for _ in range(3):
        one.step()
        two.step()
        s1, s2 = one.stats(), two.stats()
        assert s1["visco_iterations"] > 0
        assert s2["visco_iterations"] == 2 * s1["visco_iterations"]
        assert (s2["iterations"], s2["iterations_v"]) == (s1["iterations"], s1["iterations_v"])
    assert np.abs(two.x - one.x).max() < 1e-6
    assert np.abs(two.v - one.v).max() < 1e-4


def two_phase_state(counts_xyz=(11, 8, 11), steps=40, viscosity=False):
    sc, counts = layered_scene(counts_xyz, velocity=(0.2, -0.3, 0.1), viscosity=viscosity)
    if viscosity:
        sc.params.viscosity = 0.05
        sc.params.viscosityBoundary = 0.02
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


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_scale", [("fp32", 15.0), ("fp64", 1e-4)])
def test_two_phase_weiler_step_matches_oracle(precision, tol_scale):
    """Weiler2018 with boundary viscosity on the layered column, one system per phase over
    same-phase neighbours: pressure and viscosity iteration counts equal (the viscosity's the
    phases' sum).  FP64 at the tight bars (velocity measured 2.3e-12 of the speed); FP32 at 15x
    the standard bars: the velocity of a slow particle differs by 1.5e-3 of its speed (2.6e-6
    absolute, the relative bar's floor is 1e-3) while the viscous velocity change agrees to
    1.7e-5, the rounding of an FP32 CG that the FP64 run shows is not a difference of terms"""
    sc, counts, state = two_phase_state(viscosity=True)
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
    so = sim.stats()
    assert so["visco_iterations"] > 0
    assert st["visco_iterations"] == so["visco_iterations"]
    assert st["visco_error"] == pytest.approx(so["visco_error"], rel=1e-2 if precision == "fp32" else 1e-6)
    compare(ts, sim, st, tol_scale=tol_scale)
    ts.close()


@pytest.mark.gpu
def test_two_phase_weiler_graph_and_host_loops_agree():
    """the captured step (one conditional CG loop per phase) and the host-driven loops give the
    same bits over several steps (FP64)"""
    out = []
    for graph in (True, False):
        sc, counts = layered_scene(velocity=(0.2, -0.3, 0.1), viscosity=True)
        sc.params.viscosity = 0.05
        ts = TimeStepDFSPH(sc, precision="fp64", use_graph=graph)
        ts.ctx.set_lanes_per_particle(1)   # the same summation order in both runs
        ts.ctx.set_fluid_phases(counts, RHO)
        its = [ts.step()["visco_iterations"] for _ in range(4)]
        out.append((its, ts.getFluidModel().getFieldBuffer("position").copy()))
        ts.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_scale", [("fp32", 15.0), ("fp64", 1e-4)])
def test_two_phase_weiler_with_own_coefficients_matches_oracle(precision, tol_scale):
    """each model with its own Weiler2018 nu and nu_b (a viscous heavy phase with boundary viscosity
    under a thin light one without): iteration counts equal, fields at the bars of the shared case"""
    sc, counts, state = two_phase_state(viscosity=True)
    nu, nub = (0.08, 0.005), (0.03, 0.0)
    ts = TimeStepDFSPH(sc, precision=precision)
    ts.ctx.set_fluid_phases(counts, RHO)
    ts.ctx.set_fluid_phase_viscosity(nu, nub)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    sim = oracle.OracleSim(sc)
    sim.set_phases(counts, RHO)
    sim.set_phase_viscosity(nu, nub)
    sim.x[:] = state["x"]
    sim.v[:] = state["v"]
    sim.kappa[:] = state["kappa"]
    sim.kappa_v[:] = state["kappa_v"]
    sim.dt = state["dt"]
    st = ts.step()
    sim.step()
    so = sim.stats()
    assert st["visco_iterations"] == so["visco_iterations"] > 0
    compare(ts, sim, st, tol_scale=tol_scale)
    with pytest.raises(native.SphgbError):
        ts.ctx.set_fluid_phase_viscosity((0.01, -1.0), (0.0, 0.0))
    ts.close()


def test_oracle_phase_viscosity_defaults_to_the_shared_coefficients():
    """per-model coefficients equal to the shared ones give the shared run's bits"""
    sc, counts = layered_scene((6, 6, 6), velocity=(0.2, -0.3, 0.1), viscosity=True)
    sc.params.viscosity = 0.05
    sc.params.viscosityBoundary = 0.02
    a, b = oracle.OracleSim(sc), oracle.OracleSim(sc)
    for sim in (a, b):
        sim.set_phases(counts, RHO)
    b.set_phase_viscosity((0.05, 0.05), (0.02, 0.02))
    for _ in range(3):
        a.step()
        b.step()
    assert a.stats()["visco_iterations"] > 0
    assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_scale", [("fp32", 2.0), ("fp64", 1e-4)])
def test_two_phase_xsph_with_own_coefficients_matches_oracle(precision, tol_scale):
    """each model with its own XSPH fluid and boundary coefficients, the filter over the
    neighbours of every model: iteration counts equal, fields at the bars of the shared case"""
    sc, counts, state = two_phase_state()
    xs, xsb = (0.2, 0.0), (0.05, 0.3)
    ts = TimeStepDFSPH(sc, precision=precision)
    ts.ctx.set_fluid_phases(counts, RHO)
    ts.ctx.set_fluid_phase_xsph(xs, xsb)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    sim = oracle.OracleSim(sc)
    sim.set_phases(counts, RHO)
    sim.set_phase_xsph(xs, xsb)
    sim.x[:] = state["x"]
    sim.v[:] = state["v"]
    sim.kappa[:] = state["kappa"]
    sim.kappa_v[:] = state["kappa_v"]
    sim.dt = state["dt"]
    st = ts.step()
    sim.step()
    compare(ts, sim, st, tol_scale=tol_scale)
    ts.close()


def test_oracle_phase_xsph_equal_to_the_shared_coefficients_gives_the_shared_bits():
    """per-model XSPH coefficients equal to the shared ones give the shared run's bits, and a
    different coefficient on one model changes the run"""
    sc, counts = layered_scene((6, 6, 6), velocity=(0.2, -0.3, 0.1))
    sc.params.xsph = 0.2
    sc.params.xsphBoundary = 0.1
    a, b, c = oracle.OracleSim(sc), oracle.OracleSim(sc), oracle.OracleSim(sc)
    for sim in (a, b, c):
        sim.set_phases(counts, RHO)
    b.set_phase_xsph((0.2, 0.2), (0.1, 0.1))
    c.set_phase_xsph((0.2, 0.6), (0.1, 0.1))
    for _ in range(3):
        for sim in (a, b, c):
            sim.step()
    assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v)
    assert np.abs(a.v - c.v).max() > 1e-6
