"""Forces of the fluid on dynamic boundary bodies (BoundaryModel::addForce /
getForceAndTorque / clearForceAndTorque, SPlisHSPlasH/BoundaryModel.h:38-49, 86-87).

The container of a small scene is split into three bodies: the floor (dynamic), the side
walls (dynamic) and the ceiling (static).  Checks:
  * oracle: once the fluid rests, the force per step on the container equals the fluid's
    weight (the fluid-fluid pressure terms cancel pairwise, so the boundary carries M g);
  * device against the oracle after one step from the same state, with every term on
    (both solvers' pressure, XSPH boundary, Weiler2018 boundary): FP32 within 2e-3 of the
    largest component, FP64 within 1e-8;
  * graph and host loops, repeated runs, a batch against separate contexts and the
    autotuner's undone trial steps: bitwise equal sums (fixed summation order);
  * moving a body's reference point by d changes its torque by -d x F.
"""
import numpy as np
import pytest

import oracle
from splishsplash_gb300 import native, scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

from test_gpu_parity import advanced_state, compare, gpu_from_state, oracle_from_state

CENTERS = np.array([[0.4, 0.0, 0.4], [0.4, 0.5, 0.4], [0.0, 0.0, 0.0]])
DYNAMIC = [1, 1, 0]


def container_bodies(xb, top):
    """floor (y = 0) -> 0, ceiling (y = top) -> 2, the other walls -> 1"""
    return np.where(xb[:, 1] < 1e-9, 0, np.where(xb[:, 1] > top - 1e-9, 2, 1)).astype(np.uint32)


def resting_scene():
    """A block that fills the floor of its box at the rest spacing (11 x 6 x 11 particles)."""
    return scenes.small_block(counts=(11, 6, 11), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05)).as_float32()


def all_terms_scene():
    sc = scenes.small_block(counts=(10, 10, 10), box=(0.8, 1.0, 0.8), viscosity=True).as_float32()
    sc.params.viscosityBoundary = 0.05
    sc.params.xsphBoundary = 0.1
    return sc


def weight(sc):
    return sc.n * sc.params.volume * sc.params.density0 * np.asarray(sc.params.gravitation)


def test_oracle_resting_fluid_loads_container_with_its_weight():
    sc = resting_scene()
    sim = oracle.OracleSim(sc)
    sim.set_bodies(container_bodies(sc.xb, 0.8), CENTERS, DYNAMIC)
    for _ in range(150):
        sim.step()
    sim.clear_forces()
    steps = 100
    for _ in range(steps):
        sim.step()
    total = sim.body_force.sum(0) / steps
    Mg = weight(sc)
    assert np.all(sim.body_force[2] == 0.0) and np.all(sim.body_torque[2] == 0.0)
    assert abs(total[1] - Mg[1]) < 2e-3 * abs(Mg[1]), (total, Mg)
    assert np.abs(total[[0, 2]]).max() < 1e-2 * abs(Mg[1])


def test_oracle_accumulates_until_cleared():
    sc = all_terms_scene()
    state = advanced_state(sc, 40)
    a, b = oracle_from_state(sc, state), oracle_from_state(sc, state)
    for sim in (a, b):
        sim.set_bodies(container_bodies(sc.xb, 1.0), CENTERS, DYNAMIC)
        sim.step()
    f1 = b.body_force.copy()
    b.clear_forces()
    a.step()
    b.step()
    np.testing.assert_allclose(a.body_force, f1 + b.body_force, rtol=1e-12, atol=1e-9)


# ------------------------------------------------------------------- device
def moving_box_oracle(u, steps=15):
    """a column in a box of boundary particles (one dynamic body) translating at u, the fluid
    starting at u too, with XSPH, Weiler2018 and both boundary terms, a fixed step size and a fully
    converged viscous solve (its stopping rule is relative to |b|, which depends on the frame); the
    box's particles are placed at x0 + t with velocity u before every step, as
    SimulatorBase::updateBoundaryParticles does (SimulatorBase.cpp:1620-1645)"""
    sc = scenes.small_block(counts=(8, 6, 8), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05),
                            viscosity=True).as_float32()
    sc.params.cflMethod = 0
    sc.params.xsphBoundary = 0.1
    sc.params.viscosityBoundary = 0.05
    sc.params.viscoMaxError = 1e-12
    sc.params.viscoMaxIter = 1000
    sc.v = sc.v + np.asarray(u)
    sim = oracle.OracleSim(sc, fp32_predicate=False)
    xb0 = sim.xb.copy()
    sim.set_bodies(np.zeros(sc.nb, np.uint32), np.zeros((1, 3)))
    for _ in range(steps):
        t = np.asarray(u) * sim.st.time
        sim.set_boundary_state(xb0 + t, np.broadcast_to(np.asarray(u, float), xb0.shape))
        sim.body_center[0] = t
        sim.step()
    return sim


def test_oracle_moving_particle_box_is_galilean_invariant():
    """a translating box of boundary particles carrying its fluid evolves as the box at rest: every
    Akinci2012 term uses v_i - v_b (divergence source, density advection, XSPH, Weiler2018's
    right-hand side and force), and the forces and torques on the box agree"""
    u = np.array([0.4, 0.0, -0.25])
    a, b = moving_box_oracle(np.zeros(3)), moving_box_oracle(u)
    T = b.st.time
    assert abs(T - a.st.time) < 1e-15 and b.stats()["iterations"] >= 2
    assert np.abs(b.x - u * T - a.x).max() < 1e-9
    assert np.abs(b.v - u - a.v).max() < 1e-9
    scale = np.abs(a.body_force).max()
    assert scale > 1.0
    assert np.abs(b.body_force - a.body_force).max() < 1e-9 * scale
    assert np.abs(b.body_torque - a.body_torque).max() < 1e-9 * max(1.0, np.abs(a.body_torque).max())


def device_forces(ctx):
    f, t = ctx.boundary_forces()
    return f.copy(), t.copy()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp32", 2e-3), ("fp64", 1e-8)])
def test_forces_match_oracle_with_every_term(precision, tol):
    sc = all_terms_scene()
    state = advanced_state(sc, 40)
    body = container_bodies(sc.xb, 1.0)
    sim = oracle_from_state(sc, state)
    sim.set_bodies(body, CENTERS, DYNAMIC)
    ts = gpu_from_state(sc, state, precision=precision)
    ts.ctx.set_boundary_bodies(body, CENTERS, DYNAMIC)
    st = ts.step()
    sim.step()
    assert st["iterations"] == sim.stats()["iterations"]
    f, t = device_forces(ts.ctx)
    scale_f = np.abs(sim.body_force).max()
    scale_t = np.abs(sim.body_torque).max()
    assert scale_f > 100.0
    assert np.abs(f - sim.body_force).max() < tol * scale_f, (f, sim.body_force)
    assert np.abs(t - sim.body_torque).max() < tol * scale_t, (t, sim.body_torque)
    assert np.all(f[2] == 0.0) and np.all(t[2] == 0.0)
    ts.close()


@pytest.mark.gpu
def test_resting_fluid_loads_container_with_its_weight():
    sc = resting_scene()
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_boundary_bodies(container_bodies(sc.xb, 0.8), CENTERS, DYNAMIC)
    for _ in range(150):
        ts.step()
    ts.ctx.clear_boundary_forces()
    steps = 100
    for _ in range(steps):
        ts.step()
    f, _ = device_forces(ts.ctx)
    total = f.sum(0) / steps
    Mg = weight(sc)
    assert abs(total[1] - Mg[1]) < 2e-3 * abs(Mg[1]), (total, Mg)
    assert np.abs(total[[0, 2]]).max() < 1e-2 * abs(Mg[1])
    ts.close()


def run_bodies(sc, body, steps, use_graph=True, lanes=2, centers=CENTERS):
    ts = TimeStepDFSPH(sc, use_graph=use_graph)
    if lanes:
        ts.ctx.set_lanes_per_particle(lanes)
    ts.ctx.set_boundary_bodies(body, centers, DYNAMIC)
    for _ in range(steps):
        ts.step()
    out = device_forces(ts.ctx)
    lanes_used = ts.ctx.lanes_per_particle()[0]
    ts.close()
    return out, lanes_used


@pytest.mark.gpu
def test_graph_host_and_repeat_runs_agree_bitwise():
    sc = all_terms_scene()
    body = container_bodies(sc.xb, 1.0)
    (f0, t0), _ = run_bodies(sc, body, 15, use_graph=False)
    (f1, t1), _ = run_bodies(sc, body, 15, use_graph=True)
    (f2, t2), _ = run_bodies(sc, body, 15, use_graph=True)
    for a, b in ((f0, f1), (t0, t1), (f1, f2), (t1, t2)):
        np.testing.assert_array_equal(a, b)
    assert np.abs(f1).max() > 100.0


@pytest.mark.gpu
def test_autotune_trial_steps_are_not_counted():
    sc = all_terms_scene()
    body = container_bodies(sc.xb, 1.0)
    (fa, ta), pick = run_bodies(sc, body, 3, lanes=0)
    (ff, tf), _ = run_bodies(sc, body, 3, lanes=pick)
    np.testing.assert_array_equal(fa, ff)
    np.testing.assert_array_equal(ta, tf)


@pytest.mark.gpu
def test_torque_follows_the_reference_point():
    sc = all_terms_scene()
    body = container_bodies(sc.xb, 1.0)
    d = np.array([0.3, -0.2, 0.5])
    (f0, t0), _ = run_bodies(sc, body, 5)
    (f1, t1), _ = run_bodies(sc, body, 5, centers=CENTERS + d)
    np.testing.assert_array_equal(f0, f1)
    expect = t0 - np.cross(d, f0)
    assert np.abs(t1 - expect).max() < 1e-9 * (np.abs(t0).max() + np.abs(f0).max())


@pytest.mark.gpu
def test_batch_matches_separate_contexts_bitwise():
    a = all_terms_scene()
    b = scenes.small_block(counts=(8, 12, 8), box=(0.8, 1.0, 0.8), seed=11, viscosity=True).as_float32()
    b.params = a.params
    ba, bb = container_bodies(a.xb, 1.0), container_bodies(b.xb, 1.0) + 3
    centers = np.concatenate([CENTERS, CENTERS + 0.1])
    dyn = DYNAMIC + DYNAMIC
    batch = BatchedTimeStepDFSPH([a, b])
    batch.ctx.set_lanes_per_particle(2)
    batch.ctx.set_boundary_bodies(np.concatenate([ba, bb]), centers, dyn)
    for _ in range(10):
        batch.step()
    fb, tb = device_forces(batch.ctx)
    batch.close()
    for k, (sc, body) in enumerate(((a, ba), (b, bb - 3))):
        ts = TimeStepDFSPH(sc)
        ts.ctx.set_lanes_per_particle(2)
        ts.ctx.set_boundary_bodies(body, centers[3 * k:3 * k + 3], DYNAMIC)
        for _ in range(10):
            ts.step()
        f, t = device_forces(ts.ctx)
        ts.close()
        np.testing.assert_array_equal(fb[3 * k:3 * k + 3], f)
        np.testing.assert_array_equal(tb[3 * k:3 * k + 3], t)


@pytest.mark.gpu
def test_api_errors_and_reset():
    sc = resting_scene()   # touches the floor from the first step
    ts = TimeStepDFSPH(sc)
    body = container_bodies(sc.xb, 0.8)
    with pytest.raises(RuntimeError):
        ts.ctx.set_boundary_bodies(body + 5, CENTERS, DYNAMIC)   # body index out of range
    ts.ctx.set_boundary_bodies(body, CENTERS, DYNAMIC)
    ts.step()
    f, _ = device_forces(ts.ctx)
    assert np.abs(f).max() > 0.0
    ts.ctx.clear_boundary_forces()
    f, t = device_forces(ts.ctx)
    assert np.all(f == 0.0) and np.all(t == 0.0)
    ts.ctx.set_boundary_bodies([], np.zeros((0, 3)))           # removes the bodies
    ts.step()
    f, t = device_forces(ts.ctx)
    assert f.shape == (0, 3)
    ts.close()


# ------------------------------------------------------------- moving particle bodies
@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp32", 2e-3), ("fp64", 1e-8)])
def test_moving_body_step_and_forces_match_oracle(precision, tol):
    """one step with the floor (body 0) lifted, sliding and spinning about its position, with every
    boundary term on: fields and forces against the oracle, which gets the same placed particles
    and their velocities w x (x0) + v"""
    sc = all_terms_scene()
    state = advanced_state(sc, 40)
    body = container_bodies(sc.xb, 1.0)
    t = np.array([0.0, 0.002, 0.0])
    vel, omega = np.array([0.3, 0.1, 0.0]), np.array([0.0, 0.5, 0.0])
    ts = gpu_from_state(sc, state, precision=precision)
    ts.ctx.set_boundary_bodies(body, CENTERS, DYNAMIC)
    ts.ctx.set_body_motion(0, np.eye(3), t, vel, omega)
    dt = np.float32 if precision == "fp32" else np.float64
    x0 = sc.xb.astype(dt)
    xb = np.where((body == 0)[:, None], x0 + t.astype(dt), x0).astype(np.float64)   # the device's arithmetic
    vb = np.where((body == 0)[:, None], np.cross(omega, sc.xb) + vel, 0.0)
    sim = oracle_from_state(sc, state)
    sim.set_bodies(body, CENTERS, DYNAMIC)
    sim.body_center[0] = t
    sim.set_boundary_state(xb, vb)
    st = ts.step()
    sim.step()
    np.testing.assert_array_equal(ts.ctx.download("boundary position"), xb)
    compare(ts, sim, st, tol_scale=1.0 if precision == "fp32" else 1e-4)
    f, tq = device_forces(ts.ctx)
    scale_f, scale_t = np.abs(sim.body_force).max(), np.abs(sim.body_torque).max()
    assert scale_f > 100.0
    assert np.abs(f - sim.body_force).max() < tol * scale_f, (f, sim.body_force)
    assert np.abs(tq - sim.body_torque).max() < tol * scale_t, (tq, sim.body_torque)
    ts.close()


@pytest.mark.gpu
def test_device_moving_particle_box_is_galilean_invariant():
    """the oracle's invariance check on the device (FP64): the box of boundary particles translating
    with its fluid, placed before every step, evolves as the box at rest"""
    u = np.array([0.4, 0.0, -0.25])
    out = []
    for uu in (np.zeros(3), u):
        sc = scenes.small_block(counts=(8, 6, 8), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05),
                                viscosity=True).as_float32()
        sc.params.cflMethod = 0
        sc.params.xsphBoundary = 0.1
        sc.params.viscosityBoundary = 0.05
        sc.params.viscoMaxError = 1e-12
        sc.params.viscoMaxIter = 1000
        sc.v = sc.v + uu
        ts = TimeStepDFSPH(sc, precision="fp64", use_graph=True)
        ts.ctx.set_boundary_bodies(np.zeros(sc.nb, np.uint32), np.zeros((1, 3)))
        time = 0.0
        for _ in range(15):
            ts.ctx.set_body_motion(0, None, uu * time, uu)
            st = ts.step()
            time = st["time"]
        m = ts.getFluidModel()
        out.append((m.getFieldBuffer("position"), m.getFieldBuffer("velocity"), device_forces(ts.ctx), time))
        ts.close()
    (xa, va, (fa, ta), Ta), (xb, vb, (fb, tb), Tb) = out
    assert Ta == Tb
    assert np.abs(xb - u * Tb - xa).max() < 1e-8
    assert np.abs(vb - u - va).max() < 1e-8
    assert np.abs(fb - fa).max() < 1e-8 * np.abs(fa).max()
    assert np.abs(tb - ta).max() < 1e-8 * max(1.0, np.abs(ta).max())


@pytest.mark.gpu
def test_moving_body_bounds_the_cfl_step():
    """fluid at rest, its floor moving at 1 m/s: the step size follows the boundary particles'
    speed (|v_b|^2 in the CFL maximum)"""
    sc = resting_scene()
    sc.params.cflMaxTimeStepSize = 0.1
    body = container_bodies(sc.xb, 0.8)
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_boundary_bodies(body, CENTERS, DYNAMIC)
    ts.ctx.set_body_motion(0, None, None, (1.0, 0.0, 0.0))
    st = ts.step()
    expect = sc.params.cflFactor * 0.4 * 2 * sc.params.particleRadius / 1.0
    assert st["dt_next"] == pytest.approx(expect, rel=1e-6)
    ts.close()


@pytest.mark.gpu
def test_body_motion_refusals():
    def code(fn):
        with pytest.raises(native.SphgbError) as e:
            fn()
        return native.ERR_NAMES[e.value.code]

    sc = scenes.small_block(counts=(4, 4, 4))
    ts = TimeStepDFSPH(sc)
    assert code(lambda: ts.ctx.set_body_motion(0, None, (0, 0, 0))) == "ARGUMENT"          # no bodies
    ts.ctx.set_boundary_bodies(np.zeros(sc.nb, np.uint32), np.zeros((1, 3)))
    assert code(lambda: ts.ctx.set_body_motion(1, None, (0, 0, 0))) == "ARGUMENT"          # no such body
    assert code(lambda: ts.ctx.set_body_motion(0, None, (np.inf, 0, 0))) == "NONFINITE"
    ts.close()


@pytest.mark.gpu
def test_batch_with_moving_bodies_matches_separate_contexts():
    """two scenes whose floors slide at different speeds (bodies 0 and 3, one per scene): the batch
    equals the scenes run in separate contexts bit for bit, forces included"""
    a = all_terms_scene()
    b = scenes.small_block(counts=(8, 12, 8), box=(0.8, 1.0, 0.8), seed=11, viscosity=True).as_float32()
    b.params = a.params
    ba, bb = container_bodies(a.xb, 1.0), container_bodies(b.xb, 1.0) + 3
    centers = np.concatenate([CENTERS, CENTERS + 0.1])
    dyn = DYNAMIC + DYNAMIC
    speeds = ((0.3, 0.0, 0.0), (0.0, 0.0, -0.2))
    batch = BatchedTimeStepDFSPH([a, b])
    batch.ctx.set_lanes_per_particle(1)
    batch.ctx.set_boundary_bodies(np.concatenate([ba, bb]), centers, dyn)
    for _ in range(10):
        batch.ctx.set_body_motion(0, None, None, speeds[0])
        batch.ctx.set_body_motion(3, None, None, speeds[1])
        batch.step()
    xs = batch.getFieldBuffer("position")
    fb, tb = device_forces(batch.ctx)
    batch.close()
    for k, (sc, body) in enumerate(((a, ba), (b, bb - 3))):
        ts = TimeStepDFSPH(sc)
        ts.ctx.set_lanes_per_particle(1)
        ts.ctx.set_boundary_bodies(body, centers[3 * k:3 * k + 3], DYNAMIC)
        for _ in range(10):
            ts.ctx.set_body_motion(0, None, None, speeds[k])
            ts.step()
        np.testing.assert_array_equal(xs[k], ts.getFluidModel().getFieldBuffer("position"))
        f, t = device_forces(ts.ctx)
        ts.close()
        assert np.abs(f[0]).max() > 1.0
        np.testing.assert_array_equal(fb[3 * k:3 * k + 3], f)
        np.testing.assert_array_equal(tb[3 * k:3 * k + 3], t)
