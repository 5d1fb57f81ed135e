"""Bender2019 volume-map boundaries (the reference's default boundary handling).

CPU (oracle/vmap.c): the cubic serendipity grid reproduces linear fields exactly and its shape
functions sum to one; the signed distance of a box mesh equals the analytic one; the volume
saturates near 0.8 x the support ball; a resting column stays in a volume-mapped box with the
average density error under the solver tolerance.

GPU: the map the device builds (FP64) equals the oracle's node by node; one step from the same
state matches the oracle (the parity bars of test_gpu_parity); a particle found inside a body is
moved back as the oracle moves it; a resting column behaves as in the oracle; unsupported
combinations are refused with their status codes.
"""
import numpy as np
import pytest

import oracle
from splishsplash_gb300 import native, scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

from test_gpu_parity import compare, f32, relv

BOX = (0.8, 1.0, 0.8)
RES = (10, 12, 10)


def box_sdf_inside(p, lo, hi):
    """analytic distance to the box surface, positive inside"""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    d_in = np.minimum(p - lo, hi - p).min(axis=1)
    d_out = np.linalg.norm(np.maximum(np.maximum(lo - p, p - hi), 0.0), axis=1)
    inside = np.all((p >= lo) & (p <= hi), axis=1)
    return np.where(inside, d_in, -d_out)


def container_map(support, res=RES, box=BOX):
    v, f = scenes.box_mesh((0, 0, 0), box)
    return oracle.VolumeMap(res).build(v, f, support, invert=True)


def vmap_scene(counts=(10, 10, 10), seed=7, velocity=None, viscosity=False):
    """a block in a volume-mapped box; with viscosity, Weiler2018 with boundary viscosity 0.05"""
    sc = scenes.small_block(counts=counts, box=BOX, seed=seed, velocity=velocity, viscosity=viscosity).as_float32()
    sc.xb = np.zeros((0, 3))
    if viscosity:
        sc.params.viscosityBoundary = 0.05
    return sc


# --------------------------------------------------------------------- oracle
def test_oracle_grid_interpolation_is_exact_for_linear_fields():
    m = oracle.VolumeMap((3, 4, 5), dmin=(-1.0, -2.0, 0.0), dmax=(2.0, 2.0, 3.0))
    p = m.node_positions()
    a = np.array([0.3, -1.2, 0.7])
    m.fields[0][:] = p @ a + 0.5
    m.fields[1][:] = 1.0
    rng = np.random.default_rng(0)
    for x in rng.uniform((-1, -2, 0), (2, 2, 3), size=(50, 3)):
        val, g = m.interpolate(0, x)
        assert abs(val - (x @ a + 0.5)) < 1e-12
        np.testing.assert_allclose(g, a, atol=1e-11)
        one, g1 = m.interpolate(1, x)
        assert abs(one - 1.0) < 1e-13 and np.abs(g1).max() < 1e-11
    assert m.interpolate(0, np.array([2.5, 0.0, 0.0])) is None


def test_oracle_box_map_distance_and_volume():
    h = 0.1
    m = container_map(h)
    p = m.node_positions()
    np.testing.assert_allclose(m.fields[0], box_sdf_inside(p, (0, 0, 0), BOX), atol=1e-12)
    vol = m.fields[1]
    ball = 0.8 * 4.0 / 3.0 * np.pi * h ** 3
    assert np.all(vol >= 0.0) and abs(vol.max() / ball - 1.0) < 0.05
    assert np.all(vol[m.fields[0] > 2 * h] == 0.0)
    # a node a full support radius inside the wall sees the whole ball
    deep = (m.fields[0] < -1.2 * h) & (m.fields[0] > -2.0 * h)
    np.testing.assert_allclose(vol[deep], vol.max(), rtol=1e-9)


def test_oracle_resting_column_in_a_volume_mapped_box():
    sc = scenes.small_block(counts=(11, 6, 11), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05)).as_float32()
    sc.xb = np.zeros((0, 3))
    sim = oracle.OracleSim(sc)
    sim.set_volume_maps([container_map(4 * sc.params.particleRadius, (12, 16, 12), (0.6, 0.8, 0.6))])
    for _ in range(150):
        sim.step()
        assert sim.stats()["avg_density_err"] <= 0.01 * 0.01 * 1000.0 + 1e-12
    assert sim.x.min() > 0.02 and np.all(sim.x.max(0) < np.array([0.58, 0.8, 0.58]))


def test_oracle_boundary_viscosity_of_a_map_brakes_tangential_motion():
    """one particle sliding along the floor of a volume-mapped box without gravity: the Weiler2018
    boundary term (four samples per map point) slows it and leaves the normal velocity alone up to
    a small fraction, in proportion to the boundary viscosity"""
    out = []
    for mub in (0.05, 0.1):
        sc = vmap_scene(counts=(1, 1, 1), viscosity=True)
        sc.x = np.array([[0.4, 1.5 * sc.params.particleRadius, 0.4]])
        sc.v = np.array([[1.0, 0.0, 0.0]])
        sc.params.gravitation = (0.0, 0.0, 0.0)
        sc.params.viscosity = 0.0
        sc.params.viscosityBoundary = mub
        sc.params.xsph = 0.0
        sim = oracle.OracleSim(sc)
        sim.set_volume_maps([container_map(4 * sc.params.particleRadius)])
        sim.step()
        out.append(sim.vdiff[0].copy())
    assert out[0][0] < 0.0 and out[1][0] < out[0][0]
    assert abs(out[0][1]) < 0.1 * abs(out[0][0]) and abs(out[0][2]) < 1e-6 * abs(out[0][0])


def moving_container_run(u, steps=15, precision="f64"):
    """a column in a volume-mapped box translating at velocity u (the fluid starting at u as well),
    with XSPH, Weiler2018 and both boundary terms on and a fixed step size; the box's pose and
    velocity are set before every step, as a rigid-body solver would.  The column starts 0.07
    from the walls, where the coarse map's distance is positive (a particle found inside a body is
    stopped, v = 0, which no frame change carries), and the viscous solve converges fully (its
    stopping rule is relative to |b|, which depends on the frame)."""
    sc = scenes.small_block(counts=(8, 6, 8), box=(0.6, 0.8, 0.6), corner=(0.07, 0.07, 0.07),
                            viscosity=True).as_float32()
    sc.xb = np.zeros((0, 3))
    sc.params.cflMethod = 0
    sc.params.xsphBoundary = 0.1
    sc.params.viscosityBoundary = 0.05
    sc.params.viscoMaxError = 1e-12
    sc.params.viscoMaxIter = 1000
    sc.v = sc.v + np.asarray(u)
    sim = oracle.OracleSim(sc, precision=precision, fp32_predicate=False)
    sim.set_volume_maps([container_map(4 * sc.params.particleRadius, (12, 16, 12), (0.6, 0.8, 0.6))])
    sim.set_bodies(None, np.zeros((1, 3)))
    for _ in range(steps):
        sim.set_map_motion(0, translation=np.asarray(u) * sim.st.time, velocity=u)
        sim.step()
    return sim


def test_oracle_moving_container_is_galilean_invariant():
    """a uniformly translating box carrying its fluid along evolves as the same fluid at rest in
    the box at rest: every boundary term uses v_i - v_b (divergence source, density advection,
    XSPH, Weiler2018's right-hand side and its force), and the forces and torques on the box (about
    its moving position) agree"""
    u = np.array([0.4, 0.0, -0.25])
    a, b = moving_container_run(np.zeros(3)), moving_container_run(u)
    T = b.st.time
    assert abs(T - a.st.time) < 1e-15 and b.stats()["iterations"] >= 2
    assert np.abs(b.x - u * T - a.x).max() < 1e-9
    assert np.abs(b.v - u - a.v).max() < 1e-9
    scale = np.abs(a.body_force).max()
    assert scale > 1.0
    assert np.abs(b.body_force - a.body_force).max() < 1e-9 * scale
    assert np.abs(b.body_torque - a.body_torque).max() < 1e-9 * max(1.0, np.abs(a.body_torque).max())


# --------------------------------------------------------------------- device
def device_context(sc, precision="fp32", res=RES, use_graph=False):
    ts = TimeStepDFSPH(sc, precision=precision, use_graph=use_graph)
    v, f = scenes.box_mesh((0, 0, 0), BOX)
    ts.ctx.add_volume_map(v, f, res, invert=True)
    ts.ctx.set_boundary_method(2)
    return ts


@pytest.mark.gpu
def test_device_map_matches_oracle():
    sc = vmap_scene()
    ts = device_context(sc)
    res, lo, hi, dist, vol = ts.ctx.volume_map(0)
    ref = container_map(4 * sc.params.particleRadius)
    np.testing.assert_array_equal(res, RES)
    np.testing.assert_allclose(lo, ref.m.dmin[:], atol=1e-15)
    np.testing.assert_allclose(hi, ref.m.dmax[:], atol=1e-15)
    assert np.abs(dist - ref.fields[0]).max() < 1e-12
    assert np.abs(vol - ref.fields[1]).max() < 1e-12 * max(1.0, ref.fields[1].max() * 1e3)
    ts.close()


def oracle_with_map(sc, ts, state=None):
    res, lo, hi, dist, vol = ts.ctx.volume_map(0)
    m = oracle.VolumeMap(res).set_values(lo, hi, dist, vol)
    sim = oracle.OracleSim(sc)
    sim.set_volume_maps([m])
    if state is not None:
        sim.x[:] = state["x"]
        sim.v[:] = state["v"]
        sim.kappa[:] = state["kappa"]
        sim.kappa_v[:] = state["kappa_v"]
        sim.dt = state["dt"]
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize("viscosity", [False, True])
@pytest.mark.parametrize("precision,tol_scale", [("fp32", 1.0), ("fp64", 1e-4)])
def test_step_matches_oracle(precision, tol_scale, viscosity):
    """FP64 bar 1e-4 of the FP32 one (velocity 1e-8): the map samples sum 32 products per field,
    contracted to fused multiply-adds on the device and not in the oracle, and the solver
    iterations carry those last-bit differences to about 5e-9 in the velocities.  With viscosity
    the Weiler2018 boundary term samples each map point at four tangential points; the FP32 bar is
    then 3x the standard one (measured 2.4e-4 on the velocities, the pressure solve carrying the
    samples' float rounding), while the FP64 run of the same case agrees to 4e-13."""
    if viscosity and precision == "fp32":
        tol_scale = 3.0
    sc = vmap_scene(velocity=(0.3, -0.5, 0.2), viscosity=viscosity)
    probe = device_context(sc)
    pre = oracle_with_map(sc, probe)
    probe.close()
    for _ in range(40):    # a compressed state against the walls
        pre.step()
    state = dict(x=f32(pre.x), v=f32(pre.v), kappa=f32(pre.kappa), kappa_v=f32(pre.kappa_v), dt=pre.dt)
    ts = device_context(sc, precision)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    sim = oracle_with_map(sc, ts, state)
    st = ts.step()
    sim.step()
    assert st["max_boundary_neighbors"] == 0
    assert sim.stats()["iterations"] >= 2
    compare(ts, sim, st, tol_scale=tol_scale)
    if viscosity:
        assert st["visco_iterations"] == sim.stats()["visco_iterations"]
        vd = ts.getFluidModel().getFieldBuffer("velocity difference")
        assert relv(vd, sim.vdiff, 1e-3) < (1e-3 if precision == "fp32" else 1e-9)
    ts.close()


@pytest.mark.gpu
def test_particle_inside_a_body_is_moved_back_like_the_oracle():
    sc = vmap_scene(counts=(6, 6, 6))
    sc.x = np.concatenate([sc.x, [[-0.004, 0.5, 0.4]]])    # inside the wall, far from the fluid
    sc.v = np.concatenate([sc.v, [[-1.0, 0.0, 0.0]]])
    ts = device_context(sc, "fp64")
    sim = oracle_with_map(sc, ts)
    ts.step()
    sim.step()
    x = ts.getFluidModel().getFieldBuffer("position")
    assert np.abs(x[-1] - sim.x[-1]).max() < 1e-12
    assert x[-1, 0] > -0.004                                  # moved toward the fluid side
    ts.close()


@pytest.mark.gpu
def test_resting_column_in_a_volume_mapped_box():
    sc = scenes.small_block(counts=(11, 6, 11), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05)).as_float32()
    sc.xb = np.zeros((0, 3))
    ts = TimeStepDFSPH(sc, use_graph=True)
    v, f = scenes.box_mesh((0, 0, 0), (0.6, 0.8, 0.6))
    ts.ctx.add_volume_map(v, f, (12, 16, 12), invert=True)
    ts.ctx.set_boundary_method(2)
    for _ in range(150):
        st = ts.step()
        assert st["avg_density_err"] <= 0.01 * 0.01 * 1000.0 + 1e-9
    x = ts.getFluidModel().getFieldBuffer("position")
    assert x.min() > 0.02 and np.all(x.max(0) < np.array([0.58, 0.8, 0.58]))
    ts.close()


@pytest.mark.gpu
def test_unsupported_combinations_are_refused():
    def code(fn):
        with pytest.raises(native.SphgbError) as e:
            fn()
        return native.ERR_NAMES[e.value.code]

    sc = vmap_scene(counts=(6, 6, 6))
    ts = TimeStepDFSPH(sc, use_graph=False)
    ts.ctx.set_boundary_method(2)
    assert code(ts.step) == "STATE"                           # no map
    v, f = scenes.box_mesh((0, 0, 0), BOX)
    ts.ctx.add_volume_map(v, f, RES, invert=True)
    ts.ctx.upload_boundary(scenes.small_block(counts=(2, 2, 2)).xb)
    assert code(ts.step) == "STATE"                           # boundary particles as well
    ts.ctx.upload_boundary(np.zeros((0, 3)))
    p = sc.params
    p.particleRadius = 0.02
    ts.ctx.set_params(p)
    assert code(ts.step) == "STATE"                           # map built for another radius
    p.particleRadius = sc.params.particleRadius
    ts.ctx.set_params(p)
    ts.ctx.set_volume_map_scene(0, 3)
    assert code(ts.step) == "ARGUMENT"                        # a scene that is not uploaded
    ts.close()


# ------------------------------------------------- forces on volume-map bodies
MAP_CENTER = np.array([[0.4, 0.0, 0.4]])


def column_scene():
    """a block filling the floor of a 0.6 x 0.8 x 0.6 box at the rest spacing, no XSPH (which does
    not conserve momentum exactly), so that the box carries all the fluid's momentum change"""
    sc = scenes.small_block(counts=(11, 6, 11), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05)).as_float32()
    sc.xb = np.zeros((0, 3))
    sc.params.xsph = 0.0
    return sc


def momentum_balance(sc, forces_sum, p0, p1, steps, dt):
    """sum of the per-step forces on the body against K M g - (P1 - P0) / h (fluid-fluid pressure
    terms cancel pairwise, so the boundary takes the whole change of momentum besides gravity)"""
    M = sc.n * sc.params.volume * sc.params.density0
    expect = steps * M * np.asarray(sc.params.gravitation) - (p1 - p0) / dt
    return forces_sum, expect, abs(steps * M * sc.params.gravitation[1])


def test_oracle_momentum_balance_of_a_volume_mapped_box():
    sc = column_scene()
    sim = oracle.OracleSim(sc)
    sim.set_volume_maps([container_map(4 * sc.params.particleRadius, (12, 16, 12), (0.6, 0.8, 0.6))])
    sim.set_bodies(None, MAP_CENTER)
    for _ in range(60):
        sim.step()
    m = sc.params.volume * sc.params.density0
    sim.clear_forces()
    p0 = m * sim.v.sum(0)
    steps = 40
    for _ in range(steps):
        sim.step()
        assert sim.stats()["dt_old"] == 0.005 and sim.stats()["dt"] == 0.005   # CFL at its cap
    got, expect, scale = momentum_balance(sc, sim.body_force[0], p0, m * sim.v.sum(0), steps, 0.005)
    assert np.abs(got - expect).max() < 1e-6 * scale, (got, expect)


@pytest.mark.gpu
@pytest.mark.parametrize("viscosity", [False, True])
@pytest.mark.parametrize("precision,tol", [("fp32", 2e-3), ("fp64", 1e-8)])
def test_map_body_forces_match_oracle(precision, tol, viscosity):
    """pressure, XSPH and (with viscosity) the Weiler2018 boundary force at the four samples"""
    sc = vmap_scene(velocity=(0.3, -0.5, 0.2), viscosity=viscosity)
    sc.params.xsphBoundary = 0.1
    probe = device_context(sc)
    pre = oracle_with_map(sc, probe)
    probe.close()
    for _ in range(40):
        pre.step()
    state = dict(x=f32(pre.x), v=f32(pre.v), kappa=f32(pre.kappa), kappa_v=f32(pre.kappa_v), dt=pre.dt)
    ts = device_context(sc, precision)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    ts.ctx.set_boundary_bodies(None, MAP_CENTER)
    sim = oracle_with_map(sc, ts, state)
    sim.set_bodies(None, MAP_CENTER)
    ts.step()
    sim.step()
    f, t = ts.ctx.boundary_forces()
    scale_f, scale_t = np.abs(sim.body_force).max(), np.abs(sim.body_torque).max()
    assert scale_f > 10.0
    assert np.abs(f - sim.body_force).max() < tol * scale_f, (f, sim.body_force)
    assert np.abs(t - sim.body_torque).max() < tol * scale_t, (t, sim.body_torque)
    ts.close()


@pytest.mark.gpu
def test_momentum_balance_of_a_volume_mapped_box():
    sc = column_scene()
    ts = TimeStepDFSPH(sc, use_graph=True, precision="fp64")
    v, f = scenes.box_mesh((0, 0, 0), (0.6, 0.8, 0.6))
    ts.ctx.add_volume_map(v, f, (12, 16, 12), invert=True)
    ts.ctx.set_boundary_method(2)
    ts.ctx.set_boundary_bodies(None, MAP_CENTER)
    for _ in range(60):
        ts.step()
    m = sc.params.volume * sc.params.density0
    ts.ctx.clear_boundary_forces()
    p0 = m * ts.getFluidModel().getFieldBuffer("velocity").sum(0)
    steps = 40
    for _ in range(steps):
        st = ts.step()
        assert st["dt_used"] == 0.005 and st["dt_next"] == 0.005
    p1 = m * ts.getFluidModel().getFieldBuffer("velocity").sum(0)
    got, expect, scale = momentum_balance(sc, ts.ctx.boundary_forces()[0][0], p0, p1, steps, 0.005)
    assert np.abs(got - expect).max() < 1e-6 * scale, (got, expect)
    ts.close()


# ------------------------------------------------------------- moving volume-map bodies
def rotation_y(angle):
    c, s = np.cos(angle), np.sin(angle)
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_scale,ftol", [("fp32", 1.0, 2e-3), ("fp64", 1e-4, 1e-8)])
def test_moving_map_step_and_forces_match_oracle(precision, tol_scale, ftol):
    """one step with the container turned by 0.02 rad about its centre, translating and spinning,
    with XSPH and Weiler2018 and both boundary terms: fields and the forces on the box against the
    oracle at the bars of the static case"""
    sc = vmap_scene(velocity=(0.3, -0.5, 0.2), viscosity=True)
    sc.params.xsphBoundary = 0.1
    probe = device_context(sc)
    pre = oracle_with_map(sc, probe)
    probe.close()
    for _ in range(40):
        pre.step()
    state = dict(x=f32(pre.x), v=f32(pre.v), kappa=f32(pre.kappa), kappa_v=f32(pre.kappa_v), dt=pre.dt)
    centre = 0.5 * np.asarray(BOX)
    R = rotation_y(0.02)
    t = centre - R @ centre
    vel, omega = np.array([0.2, 0.05, -0.1]), np.array([0.0, 0.8, 0.3])
    ts = device_context(sc, precision)
    m = ts.getFluidModel()
    m.setFieldBuffer("position", state["x"])
    m.setFieldBuffer("velocity", state["v"])
    m.setFieldBuffer("p / rho^2", state["kappa"])
    m.setFieldBuffer("p_v / rho^2", state["kappa_v"])
    ts.setTimeStepSize(state["dt"])
    ts.ctx.set_boundary_bodies(None, t.reshape(1, 3))
    ts.ctx.set_volume_map_motion(0, R, t, vel, omega)
    sim = oracle_with_map(sc, ts, state)
    sim.set_bodies(None, t.reshape(1, 3))
    verts = scenes.box_mesh((0, 0, 0), BOX)[0]
    max_dist = np.linalg.norm(verts - verts.mean(0), axis=1).max()   # the CFL radius the device takes from the mesh
    sim.set_map_motion(0, R, t, vel, omega, max_dist=max_dist)
    st = ts.step()
    sim.step()
    assert sim.stats()["iterations"] >= 2
    compare(ts, sim, st, tol_scale=tol_scale if precision == "fp64" else 3.0)
    f, tq = ts.ctx.boundary_forces()
    scale_f, scale_t = np.abs(sim.body_force).max(), np.abs(sim.body_torque).max()
    assert scale_f > 10.0
    assert np.abs(f - sim.body_force).max() < ftol * scale_f, (f, sim.body_force)
    assert np.abs(tq - sim.body_torque).max() < ftol * scale_t, (tq, sim.body_torque)
    ts.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_moving_body_bounds_the_cfl_step(precision):
    """fluid at rest in a box moving at 0.5 m/s and turning: the next step size follows the box's
    bound |w x (maxDist, 0, 0) + v| (taken as it is against the squared fluid speeds, as the
    reference does), on the device as in the oracle"""
    sc = vmap_scene(counts=(6, 6, 6))
    sc.params.cflMaxTimeStepSize = 0.1
    vel, omega = np.array([0.5, 0.0, 0.0]), np.array([0.0, 0.2, 0.1])
    ts = device_context(sc, precision)
    ts.ctx.set_volume_map_motion(0, None, None, vel, omega)
    sim = oracle_with_map(sc, ts)
    verts = scenes.box_mesh((0, 0, 0), BOX)[0]
    max_dist = np.linalg.norm(verts - verts.mean(0), axis=1).max()
    sim.set_map_motion(0, None, None, vel, omega, max_dist=max_dist)
    st = ts.step()
    sim.step()
    speed = np.linalg.norm(vel + np.cross(omega, [max_dist, 0.0, 0.0]))
    assert speed > (np.abs(sim.v).max() * 3) ** 2
    expect = sc.params.cflFactor * 0.4 * 2 * sc.params.particleRadius / np.sqrt(speed)
    assert sim.stats()["dt"] == pytest.approx(expect, rel=1e-12)
    assert st["dt_next"] == pytest.approx(expect, rel=1e-6)
    ts.close()


@pytest.mark.gpu
def test_device_moving_container_is_galilean_invariant():
    """the oracle's invariance check on the device (FP64): a box translating with its fluid, its
    pose and velocity set before every step, evolves as the box at rest"""
    u = np.array([0.4, 0.0, -0.25])
    out = []
    for uu in (np.zeros(3), u):
        sc = scenes.small_block(counts=(8, 6, 8), box=(0.6, 0.8, 0.6), corner=(0.07, 0.07, 0.07),
                                viscosity=True).as_float32()
        sc.xb = np.zeros((0, 3))
        sc.params.cflMethod = 0
        sc.params.xsphBoundary = 0.1
        sc.params.viscosityBoundary = 0.05
        sc.params.viscoMaxError = 1e-12
        sc.params.viscoMaxIter = 1000
        sc.v = sc.v + uu
        ts = TimeStepDFSPH(sc, precision="fp64", use_graph=True)
        v, f = scenes.box_mesh((0, 0, 0), (0.6, 0.8, 0.6))
        ts.ctx.add_volume_map(v, f, (12, 16, 12), invert=True)
        ts.ctx.set_boundary_method(2)
        ts.ctx.set_boundary_bodies(None, np.zeros((1, 3)))
        time = 0.0
        for _ in range(15):
            ts.ctx.set_volume_map_motion(0, None, uu * time, uu)
            st = ts.step()
            time = st["time"]
        m = ts.getFluidModel()
        out.append((m.getFieldBuffer("position"), m.getFieldBuffer("velocity"), ts.ctx.boundary_forces(), time))
        ts.close()
    (xa, va, (fa, ta), Ta), (xb, vb, (fb, tb), Tb) = out
    assert Ta == Tb
    assert np.abs(xb - u * Tb - xa).max() < 1e-8
    assert np.abs(vb - u - va).max() < 1e-8
    assert np.abs(fb - fa).max() < 1e-8 * np.abs(fa).max()
    assert np.abs(tb - ta).max() < 1e-8 * max(1.0, np.abs(ta).max())


@pytest.mark.gpu
def test_map_motion_refusals():
    sc = vmap_scene(counts=(4, 4, 4))
    ts = device_context(sc)
    with pytest.raises(native.SphgbError) as e:
        ts.ctx.set_volume_map_motion(1, None, (0, 0, 0))
    assert native.ERR_NAMES[e.value.code] == "ARGUMENT"
    with pytest.raises(native.SphgbError) as e:
        ts.ctx.set_volume_map_motion(0, None, (np.nan, 0, 0))
    assert native.ERR_NAMES[e.value.code] == "NONFINITE"
    ts.close()


# ------------------------------------------------------------------- batches
@pytest.mark.gpu
@pytest.mark.parametrize("moving", [False, True])
def test_batch_with_volume_maps_matches_separate_contexts(moving):
    """two scenes, each in its own volume-mapped box (the second one moving), forces on both boxes:
    the batch equals the scenes run in separate contexts bit for bit"""
    a = scenes.small_block(counts=(9, 6, 9), box=(0.6, 0.8, 0.6), corner=(0.07, 0.07, 0.07)).as_float32()
    b = scenes.small_block(counts=(8, 9, 7), box=BOX, seed=11, velocity=(0.2, 0.0, -0.1)).as_float32()
    b.params = a.params
    boxes = [(0.6, 0.8, 0.6), BOX]
    res = [(12, 16, 12), RES]
    for sc in (a, b):
        sc.xb = np.zeros((0, 3))
    motion = (None, np.array([0.05, 0.0, 0.0]), np.array([0.0, 0.2, 0.0])) if moving else None
    centers = np.array([[0.3, 0.0, 0.3], [0.4, 0.0, 0.4]])

    def setup(ctx, maps):
        ctx.set_lanes_per_particle(1)   # the summation order depends on the lanes per particle
        ctx.set_neighbor_staging(1)
        for k, scene in maps:
            v, f = scenes.box_mesh((0, 0, 0), boxes[k])
            ctx.add_volume_map(v, f, res[k], invert=True)
        for body, (k, scene) in enumerate(maps):
            ctx.set_volume_map_scene(body, scene)
        ctx.set_boundary_method(2)

    batch = BatchedTimeStepDFSPH([a, b])
    setup(batch.ctx, [(0, 0), (1, 1)])
    batch.ctx.set_boundary_bodies(None, centers)
    for _ in range(20):
        if moving:
            batch.ctx.set_volume_map_motion(1, *motion)
        batch.step()
    xs, vs = batch.getFieldBuffer("position"), batch.getFieldBuffer("velocity")
    fb, tb = batch.ctx.boundary_forces()
    batch.close()
    for k, sc in enumerate((a, b)):
        ts = TimeStepDFSPH(sc)
        setup(ts.ctx, [(k, 0)])
        ts.ctx.set_boundary_bodies(None, centers[k:k + 1])
        for _ in range(20):
            if moving and k == 1:
                ts.ctx.set_volume_map_motion(0, *motion)
            ts.step()
        m = ts.getFluidModel()
        np.testing.assert_array_equal(xs[k], m.getFieldBuffer("position"))
        np.testing.assert_array_equal(vs[k], m.getFieldBuffer("velocity"))
        f, t = ts.ctx.boundary_forces()
        assert np.abs(f).max() > 1.0
        np.testing.assert_array_equal(fb[k], f[0])
        np.testing.assert_array_equal(tb[k], t[0])
        ts.close()
