"""Pins the CPU oracle to the reference's own DFSPH time step.

The reference's SPlisHSPlasH sources (TimeStep, DFSPH, Simulation, FluidModel,
BoundaryModel_Akinci2012, XSPH, Viscosity_Weiler2018, SPHKernels, ...) are compiled by
oracle/build_ref.sh against the stand-ins of oracle/shims/ and driven through
oracle/refsim.py.  The one-step fixtures in tests/golden/ref_step_*.npz were recorded
from that build (FP64, analytic cubic spline) by tests/golden/gen_ref_steps.py.

* The FP64 oracle (oracle/sph_oracle.c) is held to the fixtures at 1e-10 with equal
  pressure, divergence and Weiler2018 CG iteration counts.  These tests need only the
  committed fixtures.
* Where the reference tree is present, the reference build itself is run: it must
  reproduce the fixtures, follow the oracle step by step over many steps, and its
  FP32 AVX build (the CPU baseline, x86-64) must run the benchmark's kind of scene.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
import ref_cases
import refsim
from splishsplash_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_TOL = 1e-10


def reference_tree():
    env = os.environ.get("SPH_REFERENCE_ROOT")
    p = env if env else os.path.join(ROOT, "..", "reference")
    return p if os.path.isfile(os.path.join(p, "SPlisHSPlasH", "TimeStep.cpp")) else None


@pytest.fixture(scope="module")
def ref_build():
    """The reference library (oracle/_ref/libref_f64.so), built on demand; skips where the
    reference tree is absent."""
    if not refsim.available("f64"):
        tree = reference_tree()
        if tree is None:
            pytest.skip("reference tree not present (set SPH_REFERENCE_ROOT)")
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True,
                       env={**os.environ, "SPH_REFERENCE_ROOT": tree}, capture_output=True)
    if not refsim.available("f64"):
        pytest.skip("reference build unavailable")
    return True


def oracle_phases(sim, ph):
    sim.set_phases(ph["counts"], ph["density0"])
    sim.set_phase_viscosity(ph["viscosity"], ph["viscosity_boundary"])
    sim.set_phase_xsph(ph["xsph"], ph["xsph_boundary"])


def oracle_step(scene, state, maps=None, phases=None):
    sim = oracle.OracleSim(ref_cases.with_state(scene, state), fp32_predicate=False)
    if maps:
        sim.set_volume_maps(maps)
    if phases:
        oracle_phases(sim, phases)
    sim.kappa[:] = state["kappa"]
    sim.kappa_v[:] = state["kappa_v"]
    sim.vdiff[:] = state["vdiff"]
    sim.dt = state["dt"]
    sim.step()
    got = dict(density=sim.density.copy(), factor=sim.factor.copy(), kappa=sim.kappa.copy(),
               kappa_v=sim.kappa_v.copy(), v=sim.v.copy(), x=sim.x.copy(), vdiff=sim.vdiff.copy())
    return got, sim.stats()


@pytest.mark.parametrize("case", ref_cases.CASES)
def test_oracle_matches_reference_step(case):
    scene, state, ref = ref_cases.load_case(case)
    got, st = oracle_step(scene, state, ref_cases.case_maps(case, scene.params.supportRadius),
                          ref_cases.case_phases(case))
    assert (st["iterations"], st["iterations_v"], st["visco_iterations"]) == \
        (ref["iterations"], ref["iterations_v"], ref["visco_iterations"])
    err = ref_cases.field_errors(got, ref)
    for k, e in err.items():
        bound = ORACLE_TOL * (np.max(np.abs(ref["x"])) if k == "x" else 1.0)
        assert e <= bound, (case, k, e)
    assert st["dt"] == pytest.approx(ref["dt_next"], rel=1e-12)


def test_oracle_follows_reference_run_with_adapted_step_size():
    """25 steps of a compressed block with the iteration-adapted CFL step size (cflMethod 2):
    the oracle takes the reference's iteration counts and step sizes in every step (the step
    size shrinks after steps of more than 10 pressure iterations and grows after fewer than 5)
    and ends on its fields."""
    scene, its, dts, ref = ref_cases.load_run("cfl_iter")
    sim = oracle.OracleSim(scene, fp32_predicate=False)
    for k in range(len(its)):
        sim.step()
        st = sim.stats()
        assert (st["iterations"], st["iterations_v"], st["visco_iterations"]) == tuple(its[k]), k
        assert st["dt"] == pytest.approx(dts[k][1], rel=1e-12), k
    got = dict(density=sim.density, factor=sim.factor, kappa=sim.kappa, kappa_v=sim.kappa_v, v=sim.v, x=sim.x)
    for k, e in ref_cases.field_errors(got, ref).items():
        assert e <= ORACLE_TOL * (np.max(np.abs(ref["x"])) if k == "x" else 1.0), (k, e)
    assert its[:, 0].max() > 10 and its[:, 0].min() < 5 and len({round(d, 9) for d in dts[:, 1]}) > 10


def test_fixtures_exercise_the_solvers():
    its = {c: ref_cases.load_case(c)[2] for c in ref_cases.CASES}
    assert max(o["iterations"] for o in its.values()) >= 10            # pressure solve
    assert max(o["iterations_v"] for o in its.values()) >= 5           # divergence solve
    assert max(o["visco_iterations"] for o in its.values()) >= 5       # Weiler2018 CG


@pytest.mark.parametrize("case", ref_cases.CASES)
def test_reference_build_reproduces_fixture(ref_build, case):
    scene, state, ref = ref_cases.load_case(case)
    visc = scene.params.viscosityMethod == 6
    maps = ref_cases.case_maps(case, scene.params.supportRadius)
    with refsim.RefSim(ref_cases.with_state(scene, state), volume_maps=maps, phases=ref_cases.case_phases(case)) as r:
        r.set("p / rho^2", state["kappa"])
        r.set("p_v / rho^2", state["kappa_v"])
        if visc:
            r.set("velocity difference", state["vdiff"])
        r.set_time_step(state["dt"])
        s = r.step()
        got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                   kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"))
    assert (s["iterations"], s["iterations_v"], s["visco_iterations"]) == \
        (ref["iterations"], ref["iterations_v"], ref["visco_iterations"])
    for k, e in ref_cases.field_errors(got, ref).items():
        assert e <= 1e-13 * (np.max(np.abs(ref["x"])) if k == "x" else 1.0), (case, k, e)


def test_oracle_follows_reference_over_steps(ref_build):
    """40 steps of a viscous shear column: oracle and reference agree after every step."""
    sc = scenes.small_block(counts=(8, 14, 8), box=(0.5, 1.0, 0.5), viscosity=True)
    sc.v[:, 0] = sc.x[:, 1] - sc.x[:, 1].mean()
    sc.params.viscosity = 0.5
    sc = sc.as_float32()
    o = oracle.OracleSim(sc, fp32_predicate=False)
    with refsim.RefSim(sc) as r:
        np.testing.assert_allclose(r.boundary_volume(), o.Vb, rtol=1e-13)
        for k in range(40):
            sr = r.step()
            o.step()
            so = o.stats()
            assert (sr["iterations"], sr["iterations_v"], sr["visco_iterations"]) == \
                (so["iterations"], so["iterations_v"], so["visco_iterations"]), k
            assert sr["dt"] == pytest.approx(so["dt"], rel=1e-12)
            got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                       kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"),
                       vdiff=r.get("velocity difference"))
            ref = dict(density=o.density, factor=o.factor, kappa=o.kappa, kappa_v=o.kappa_v, v=o.v, x=o.x,
                       vdiff=o.vdiff)
            for name, e in ref_cases.field_errors(got, ref).items():
                assert e <= ORACLE_TOL, (k, name, e)


def test_oracle_follows_reference_in_a_volume_mapped_box(ref_build):
    """Bender2019: 30 steps of the fixture's viscous block in a volume-mapped box.  The map is
    the oracle's (oracle/vmap.c); the reference evaluates it through its own Bender2019 code
    (TimeStep::computeVolumeAndBoundaryX, the Bender2019 branches of the DFSPH step, XSPH and
    Weiler2018's four-sample boundary term); both agree after every step."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_ref_steps", os.path.join(ROOT, "tests", "golden",
                                                                                 "gen_ref_steps.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    sc = gen.vmap_box().as_float32()
    maps = [gen.box_volume_map(sc.params.supportRadius)]
    o = oracle.OracleSim(sc, fp32_predicate=False)
    o.set_volume_maps(maps)
    cg = 0
    with refsim.RefSim(sc, volume_maps=maps) as r:
        for k in range(30):
            sr = r.step()
            o.step()
            so = o.stats()
            cg += sr["visco_iterations"]
            assert (sr["iterations"], sr["iterations_v"], sr["visco_iterations"]) == \
                (so["iterations"], so["iterations_v"], so["visco_iterations"]), k
            assert sr["dt"] == pytest.approx(so["dt"], rel=1e-12)
            got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                       kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"),
                       vdiff=r.get("velocity difference"))
            ref = dict(density=o.density, factor=o.factor, kappa=o.kappa, kappa_v=o.kappa_v, v=o.v, x=o.x,
                       vdiff=o.vdiff)
            for name, e in ref_cases.field_errors(got, ref).items():
                assert e <= ORACLE_TOL, (k, name, e)
    assert cg > 0


def test_oracle_follows_reference_with_two_fluid_models(ref_build):
    """20 steps of the fixture's two-model column (rest densities 1000 and 500, per-model
    Weiler2018 and XSPH coefficients): the reference runs two FluidModels, the oracle two phases;
    iteration counts equal and fields at 1e-10 after every step."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_ref_steps", os.path.join(ROOT, "tests", "golden",
                                                                                 "gen_ref_steps.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    sc, ph = gen.phases_visc()
    sc = sc.as_float32()
    o = oracle.OracleSim(sc, fp32_predicate=False)
    oracle_phases(o, ph)
    cg = 0
    with refsim.RefSim(sc, phases=ph) as r:
        for k in range(20):
            sr = r.step()
            o.step()
            so = o.stats()
            cg += sr["visco_iterations"]
            assert (sr["iterations"], sr["iterations_v"], sr["visco_iterations"]) == \
                (so["iterations"], so["iterations_v"], so["visco_iterations"]), k
            assert sr["dt"] == pytest.approx(so["dt"], rel=1e-12)
            got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                       kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"),
                       vdiff=r.get("velocity difference"))
            ref = dict(density=o.density, factor=o.factor, kappa=o.kappa, kappa_v=o.kappa_v, v=o.v, x=o.x,
                       vdiff=o.vdiff)
            for name, e in ref_cases.field_errors(got, ref).items():
                assert e <= ORACLE_TOL, (k, name, e)
    assert cg > 0


def test_body_forces_follow_the_reference(ref_build):
    """BoundaryModel::addForce on dynamic Akinci2012 bodies: the container split into a dynamic
    floor, dynamic side walls and a static ceiling (tests/test_bodies.py's all-terms scene: both
    solvers' pressure, XSPH boundary and Weiler2018 boundary terms).  The reference holds one
    BoundaryModel_Akinci2012 per body, the dynamic ones on a rigid body that nothing moves.  Over
    40 steps the boundary volumes, the force and torque on every body in every step, the fields
    and the iteration counts agree with the oracle at 1e-10."""
    from test_bodies import CENTERS, DYNAMIC, all_terms_scene, container_bodies
    sc = all_terms_scene()
    sc.v[:, 0] = 0.5 * (sc.x[:, 1] - sc.x[:, 1].mean())   # shear: the viscosity solve iterates
    body = container_bodies(sc.xb, 1.0)
    o = oracle.OracleSim(sc, fp32_predicate=False)
    o.set_bodies(body, CENTERS, DYNAMIC)
    cg = 0
    with refsim.RefSim(sc, bodies=dict(body=body, center=CENTERS, dynamic=DYNAMIC)) as r:
        np.testing.assert_allclose(r.boundary_volume(), o.Vb, rtol=1e-13)
        for k in range(40):
            r.clear_body_forces()
            o.clear_forces()
            sr = r.step()
            o.step()
            so = o.stats()
            cg += sr["visco_iterations"]
            assert (sr["iterations"], sr["iterations_v"], sr["visco_iterations"]) == \
                (so["iterations"], so["iterations_v"], so["visco_iterations"]), k
            fr, tr = r.body_forces()
            scale_f = max(float(np.abs(o.body_force).max()), 1e-30)
            scale_t = max(float(np.abs(o.body_torque).max()), 1e-30)
            assert float(np.abs(fr - o.body_force).max()) <= ORACLE_TOL * scale_f, k
            assert float(np.abs(tr - o.body_torque).max()) <= ORACLE_TOL * scale_t, k
            assert not np.any(o.body_force[2]) and not np.any(fr[2])   # the static ceiling
            got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                       kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"))
            ref = dict(density=o.density, factor=o.factor, kappa=o.kappa, kappa_v=o.kappa_v, v=o.v, x=o.x)
            for name, e in ref_cases.field_errors(got, ref).items():
                assert e <= ORACLE_TOL, (k, name, e)
    assert cg > 0 and float(np.abs(o.body_force[0]).max()) > 0


def test_moving_body_follows_the_reference(ref_build):
    """A moving Akinci2012 body: the floor of the all-terms scene slides at 4.6 m/s (fast enough for
    its particles to set the CFL step) and spins about its position.  Before every step the
    reference's rigid body gets its pose and velocity and the driver places the floor's particles
    as the simulator does (x = R x0 + t, v = w x (x - t) + v); the oracle gets the same particles
    and velocities.  Over 15 steps the step sizes, iteration counts, fields, and the force and
    torque on every body agree at 1e-10."""
    from test_bodies import CENTERS, DYNAMIC, all_terms_scene, container_bodies
    sc = all_terms_scene()
    sc.v[:, 0] = 0.5 * (sc.x[:, 1] - sc.x[:, 1].mean())
    body = container_bodies(sc.xb, 1.0)
    u, w = np.array([4.5, 0.0, -1.0]), np.array([0.0, 0.8, 0.0])
    o = oracle.OracleSim(sc, fp32_predicate=False)
    o.set_bodies(body, CENTERS, DYNAMIC)
    x0, floor = o.xb.copy(), (body == 0)[:, None]
    capped = False
    with refsim.RefSim(sc, bodies=dict(body=body, center=CENTERS, dynamic=DYNAMIC)) as r:
        for k in range(15):
            t = u * o.st.time
            r.set_body_motion(0, np.eye(3), t, u, w)
            xb = np.where(floor, x0 + t, x0)
            o.set_boundary_state(xb, np.where(floor, np.cross(w, xb - t) + u, 0.0))
            o.body_center[0] = t
            r.clear_body_forces()
            o.clear_forces()
            sr = r.step()
            o.step()
            so = o.stats()
            capped = capped or sr["dt"] < sc.params.cflMaxTimeStepSize
            assert (sr["iterations"], sr["iterations_v"], sr["visco_iterations"]) == \
                (so["iterations"], so["iterations_v"], so["visco_iterations"]), k
            assert sr["dt"] == pytest.approx(so["dt"], rel=1e-12), k
            fr, tr = r.body_forces()
            assert float(np.abs(fr - o.body_force).max()) <= ORACLE_TOL * float(np.abs(o.body_force).max()), k
            assert float(np.abs(tr - o.body_torque).max()) <= ORACLE_TOL * float(np.abs(o.body_torque).max()), k
            got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                       kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"))
            ref = dict(density=o.density, factor=o.factor, kappa=o.kappa, kappa_v=o.kappa_v, v=o.v, x=o.x)
            for name, e in ref_cases.field_errors(got, ref).items():
                assert e <= ORACLE_TOL, (k, name, e)
    assert capped   # the moving particles set the CFL step


def test_moving_volume_map_follows_the_reference(ref_build):
    """A moving Bender2019 body: the volume-mapped box of the vmap_box fixture translates at
    (2, 0, 0.5) m/s and turns about the vertical axis.  Before every step the reference's rigid
    body gets the pose and velocity, and its CFL bound as the simulator's updateVMVelocity sets it;
    the oracle's map gets the same.  Over 15 steps iteration counts and fields agree at 1e-10."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_ref_steps", os.path.join(ROOT, "tests", "golden",
                                                                                 "gen_ref_steps.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    sc = gen.vmap_box().as_float32()
    maps = [gen.box_volume_map(sc.params.supportRadius)]
    u, w, max_dist = np.array([2.0, 0.0, 0.5]), np.array([0.0, 0.6, 0.0]), 0.7
    o = oracle.OracleSim(sc, fp32_predicate=False)
    o.set_volume_maps(maps)
    with refsim.RefSim(sc, volume_maps=maps) as r:
        for k in range(15):
            time = o.st.time
            c, s_ = np.cos(w[1] * time), np.sin(w[1] * time)
            R = np.array([[c, 0.0, s_], [0.0, 1.0, 0.0], [-s_, 0.0, c]])
            r.set_map_motion(0, R, u * time, u, w, max_dist)
            o.set_map_motion(0, R, u * time, u, w, max_dist)
            sr = r.step()
            o.step()
            so = o.stats()
            assert (sr["iterations"], sr["iterations_v"], sr["visco_iterations"]) == \
                (so["iterations"], so["iterations_v"], so["visco_iterations"]), k
            assert sr["dt"] == pytest.approx(so["dt"], rel=1e-12), k
            got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                       kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"))
            ref = dict(density=o.density, factor=o.factor, kappa=o.kappa, kappa_v=o.kappa_v, v=o.v, x=o.x)
            for name, e in ref_cases.field_errors(got, ref).items():
                assert e <= ORACLE_TOL, (k, name, e)


def test_reference_neighbor_counts_match_oracle(ref_build):
    sc = scenes.small_block(counts=(10, 8, 10), box=(0.8, 0.8, 0.8)).as_float32()
    with refsim.RefSim(sc) as r:
        r.step()
        nf, nb = r.neighbor_counts()
    h = sc.params.supportRadius
    off_f, _ = oracle.neighbors(sc.x, sc.x, h, True, fp32=False)
    off_b, _ = oracle.neighbors(sc.x, sc.xb, h, False, fp32=False)
    np.testing.assert_array_equal(nf, np.diff(off_f))
    np.testing.assert_array_equal(nb, np.diff(off_b))


def test_reference_fp32_avx_build_runs(ref_build):
    """The reference's FP32 AVX build with precomputeValues (the CPU baseline) runs a few
    steps of a dam break and stays close to the FP64 oracle (its fluid sums use
    CubicKernel_AVX, its boundary volumes the lookup-table kernel)."""
    if not refsim.available("f32"):
        pytest.skip("FP32 AVX build is x86-64 only")
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 0.8, 0.8)).as_float32()
    o = oracle.OracleSim(sc, fp32_predicate=False)
    with refsim.RefSim(sc, precision="f32", analytic_kernel=False) as r:
        for _ in range(5):
            r.step()
            o.step()
        rho = r.get("density")
    assert ref_cases.rel_scalar(rho, o.density, 1.0) < 1e-3
