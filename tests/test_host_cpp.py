"""The C++ host layer (splishsplash_gb300/host): the reference's TimeStep / FluidModel /
Akinci2012 / Weiler2018 plugin interface over the C ABI.  The driver runs a scene through the
C++ classes; on the GPU its results must equal the Python mirror's bit for bit (same library,
same inputs, same lanes per particle)."""
import dataclasses
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from splishsplash_gb300 import build, scenes
from splishsplash_gb300.dfsph import TimeStepDFSPH


def _write_scene(path, sc, steps, lanes, visc, body=None, position=None, vmap=None, motion=None, phases=None):
    with open(path, "wb") as f:
        f.write(struct.pack("<8I", sc.n, sc.nb, steps, lanes, 1 if visc else 0, 0 if body is None else 1,
                            0 if vmap is None else 1, 0 if phases is None else phases[0]))
        f.write(struct.pack("<d", sc.params.particleRadius))
        if phases is not None:   # the second model's rest density and own nu, nu_b, xsph, xsph_b (-1: shared)
            f.write(struct.pack("<5d", phases[1], *phases[2]))
        for a in (sc.x, sc.v, sc.xb):
            f.write(np.ascontiguousarray(a, "<f8").tobytes())
        if body is not None:
            f.write(np.ascontiguousarray(body, "<u4").tobytes())
            f.write(np.ascontiguousarray(position, "<f8").tobytes())
            f.write(np.ascontiguousarray(motion, "<f8").tobytes())
        if vmap is not None:
            verts, faces, res = vmap
            f.write(struct.pack("<6I", len(verts), len(faces), *[int(r) for r in res], 1))
            f.write(np.ascontiguousarray(verts, "<f8").tobytes())
            f.write(np.ascontiguousarray(faces, "<u4").tobytes())


def _read_out(path, n, nb, steps):
    raw = open(path, "rb").read()
    per = []
    off = 0
    for _ in range(steps):
        it = struct.unpack_from("<3I", raw, off)
        t = struct.unpack_from("<d", raw, off + 12)[0]
        per.append((it, t))
        off += 20
    a = np.frombuffer(raw, "<f8", offset=off)
    x = a[:3 * n].reshape(n, 3)
    v = a[3 * n:6 * n].reshape(n, 3)
    rho = a[6 * n:7 * n]
    kp = a[7 * n:8 * n]
    vb = a[8 * n:8 * n + nb]
    force = a[8 * n + nb:8 * n + nb + 3]
    torque = a[8 * n + nb + 3:8 * n + nb + 6]
    return per, x, v, rho, kp, vb, force, torque


def test_host_layer_is_built_and_fails_cleanly_without_a_device():
    build.build()
    assert os.path.exists(build.HOST_LIB) and os.path.exists(build.HOST_DEMO)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present: covered by the GPU test")
    sc = scenes.small_block(counts=(4, 4, 4))
    with tempfile.TemporaryDirectory() as d:
        _write_scene(os.path.join(d, "s.bin"), sc, 1, 0, False)
        r = subprocess.run([build.HOST_DEMO, os.path.join(d, "s.bin"), os.path.join(d, "o.bin")],
                           capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "sphgb_create failed" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("visc,bodies,vmap,phases", [(False, False, False, False), (True, False, False, False),
                                                     (True, True, False, False), (True, False, True, False),
                                                     (True, True, True, False), (False, False, False, True),
                                                     (True, False, False, "own")])
def test_cpp_host_layer_matches_python_mirror(visc, bodies, vmap, phases):
    """with a volume map and bodies the container is a dynamic body with a velocity and an angular
    velocity (pose held): the C++ layer hands them to the device before every step"""
    sc = scenes.small_block(counts=(10, 12, 10), box=(0.8, 1.0, 0.8), viscosity=visc,
                            velocity=(0.3, 0.0, -0.2)).as_float32()
    # the C++ layer holds every real parameter in Real (float), like the reference's FP32 build
    f32 = lambda a: float(np.float32(a))
    p = sc.params
    for name in ("particleRadius", "density0", "cflFactor", "cflMinTimeStepSize", "cflMaxTimeStepSize", "maxError",
                 "maxErrorV", "xsph", "xsphBoundary", "viscosity", "viscosityBoundary", "timeStepSize"):
        setattr(p, name, f32(getattr(p, name)))
    p.gravitation = tuple(f32(g) for g in p.gravitation)
    p.viscoMaxError = f32(1e-3)
    steps, lanes = 12, 1
    body = position = motion = None
    if bodies and vmap:
        body = np.zeros(0, np.uint32)
        position = np.zeros(3)
        motion = np.array([0.125, 0.0, -0.0625, 0.0, 0.25, 0.0])   # exact in float
    elif bodies:
        # the floor is a dynamic body (boundary model 0) sliding along x, the other walls are static
        # (model 1)
        body = np.where(sc.xb[:, 1] < 1e-9, 0, 1).astype(np.uint32)
        position = np.array([0.375, 0.0, 0.4375], np.float64)   # exact in float (the C++ layer holds Real)
        motion = np.array([0.125, 0.0, 0.0, 0.0, 0.0, 0.0])
    mesh = None
    if vmap:
        # the container as a Bender2019 volume map instead of boundary particles
        sc = dataclasses.replace(sc, xb=np.zeros((0, 3)))
        verts, faces = scenes.box_mesh((0, 0, 0), (0.75, 1.0, 0.75))   # exact in float (the C++ Real)
        mesh = (verts, faces, (8, 10, 8))
    ph = None
    if phases:
        # a second fluid model of half the rest density above the first one (TimeStepDFSPH_GB300::addFluidModel)
        order = np.argsort(sc.x[:, 1], kind="stable")
        sc = dataclasses.replace(sc, x=sc.x[order].copy(), v=sc.v[order].copy())
        # "own": the second model with its own Weiler and XSPH coefficients
        ph = (sc.n // 2, 500.0, (0.05, 0.02, 0.1, 0.05) if phases == "own" else (-1.0, -1.0, -1.0, -1.0))
    with tempfile.TemporaryDirectory() as d:
        _write_scene(os.path.join(d, "s.bin"), sc, steps, lanes, visc, body, position, mesh, motion, ph)
        r = subprocess.run([build.HOST_DEMO, os.path.join(d, "s.bin"), os.path.join(d, "o.bin")],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        assert r.stdout.startswith("DFSPH:")
        per, x, v, rho, kp, vb, force, torque = _read_out(os.path.join(d, "o.bin"), sc.n, sc.nb, steps)
    if bodies and not vmap:
        # the C++ layer uploads the boundary models in order: body 0's particles first, in body
        # coordinates (placed at x0 + position every step)
        order = np.concatenate([np.flatnonzero(body == 0), np.flatnonzero(body != 0)])
        xb = sc.xb[order].copy()
        xb[body[order] == 0] -= position
        sc = dataclasses.replace(sc, xb=xb)
    ts = TimeStepDFSPH(sc)
    ts.ctx.set_lanes_per_particle(lanes)
    if phases:
        ts.ctx.set_fluid_phases((ph[0], sc.n - ph[0]), (sc.params.density0, ph[1]))
        if phases == "own":
            p = sc.params
            ts.ctx.set_fluid_phase_viscosity((p.viscosity, ph[2][0]), (p.viscosityBoundary, ph[2][1]))
            ts.ctx.set_fluid_phase_xsph((p.xsph, ph[2][2]), (p.xsphBoundary, ph[2][3]))
    if vmap:
        ts.ctx.add_volume_map(mesh[0], mesh[1], mesh[2], invert=True)
        ts.ctx.set_boundary_method(2)
    if bodies and vmap:
        ts.ctx.set_boundary_bodies(None, position.reshape(1, 3))
    elif bodies:
        ts.ctx.set_boundary_bodies(np.sort(body), np.stack([position, np.zeros(3)]), [1, 0])
    for k in range(steps):
        if bodies and vmap:
            ts.ctx.set_volume_map_motion(0, np.eye(3), position, motion[:3], motion[3:])
        elif bodies:
            ts.ctx.set_body_motion(0, np.eye(3), position, motion[:3], motion[3:])
        st = ts.step()
        assert per[k][0] == (st["iterations"], st["iterations_v"], st["visco_iterations"] if visc else 0)
        assert per[k][1] == pytest.approx(st["time"], rel=1e-6)
    m = ts.getFluidModel()
    # the C++ layer stores Real = float: compare in float32
    np.testing.assert_array_equal(x.astype(np.float32), m.getFieldBuffer("position", np.float32))
    np.testing.assert_array_equal(v.astype(np.float32), m.getFieldBuffer("velocity", np.float32))
    np.testing.assert_array_equal(rho.astype(np.float32), m.getFieldBuffer("density", np.float32))
    np.testing.assert_array_equal(kp.astype(np.float32), m.getFieldBuffer("p / rho^2", np.float32))
    np.testing.assert_array_equal(vb.astype(np.float32), ts.ctx.download("boundary volume", np.float32))
    if bodies and vmap:
        f, t = ts.ctx.boundary_forces()
        assert np.abs(f[0]).max() > 0.1
        np.testing.assert_array_equal(force.astype(np.float32), f[0].astype(np.float32))
        np.testing.assert_array_equal(torque.astype(np.float32), t[0].astype(np.float32))
    elif bodies:
        f, t = ts.ctx.boundary_forces()
        assert np.abs(f[0]).max() > 0.1 and np.all(f[1] == 0.0)   # the block reaches the floor
        np.testing.assert_array_equal(force.astype(np.float32), f[0].astype(np.float32))
        np.testing.assert_array_equal(torque.astype(np.float32), t[0].astype(np.float32))
    else:
        assert np.all(force == 0.0) and np.all(torque == 0.0)
    ts.close()
