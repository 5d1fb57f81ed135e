"""The reference's particle state files (SimulatorBase::writeFluidParticlesState /
readFluidParticlesState, Simulator/SimulatorBase.cpp:2062-2192), written and read by the device.

The state of a fluid model is one partio BGEO file of the fields the reference marks storeData
(FluidModel.cpp:61-66, TimeStepDFSPH.cpp:51-52, Viscosity_Weiler2018.cpp:33).  The fixtures
tests/golden/{reference,device}_state_column.{bgeo,npz} were written by
tests/golden/gen_state_files.py: the reference's FP64 build through partio (vendored in its
tree, extern/partio), and the device through sphgb_save_particle_state on a GB300; each holds
one step taken from the file as stored.

* GPU: the device's file has the reference's attributes and values; the device loads its own
  file and the reference's file and continues: from the reference's file, one step matches the
  reference's step from the same file (iteration counts equal, density 1e-5, velocity 5e-4,
  kappa 1e-3 of the largest);
* CPU (reference tree present): partio, built from the reference's tree, reads the device's
  file with the stored values; the reference's build reads the device's file into its own
  Simulation and its step from it matches the device's step from the same file.
"""
import ctypes
import dataclasses
import json
import os

import numpy as np
import pytest

import ref_cases
import refbuild
import refsim
from splishsplash_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ATTRS = ["id", "state", "object_id", "velocity", "p / rho^2", "p_v / rho^2", "velocity difference"]
# FP32 device against the FP64 reference, one viscous step (nu = 0.2, tens of iterations)
BARS = dict(density=1e-5, factor=1e-4, v=5e-4, kappa=1e-3, kappa_v=1e-3, vdiff=1e-3)


def fixture(side):
    g = np.load(os.path.join(GOLDEN, f"{side}_state_column.npz"))
    params = scenes.SPHParams(**{k: (tuple(v) if isinstance(v, list) else v)
                                 for k, v in json.loads(str(g["params"])).items()})
    x = g["stored_x"].astype(np.float64)
    scene = scenes.Scene(f"{side}_state_column", x, g["stored_v"].astype(np.float64), g["xb"].astype(np.float64),
                         params, np.asarray(g["box_min"]), np.asarray(g["box_max"]))
    return scene, g


def next_step(g):
    return {k[5:]: g[k] for k in g.files if k.startswith("next_")}


def check_step(got, st, g):
    assert (st["iterations"], st["iterations_v"], st["visco_iterations"]) == \
        (int(g["iterations"]), int(g["iterations_v"]), int(g["visco_iterations"]))
    err = ref_cases.field_errors(got, next_step(g))
    for k, bar in BARS.items():
        if k in err:
            assert err[k] <= bar, (k, err[k])
    assert st["dt_next" if "dt_next" in st else "dt"] == pytest.approx(float(g["dt_next"]), rel=1e-5)


# ------------------------------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_device_state_file_layout(tmp_path):
    from test_io import read_bgeo
    from splishsplash_gb300.dfsph import TimeStepDFSPH
    sc = scenes.small_block(counts=(8, 10, 8), box=(0.6, 0.8, 0.6), viscosity=True, velocity=(0.2, 0, 0)).as_float32()
    ts = TimeStepDFSPH(sc)
    try:
        for _ in range(5):
            ts.step()
        path = str(tmp_path / "state.bgeo")
        ts.ctx.save_particle_state(path)
        b = read_bgeo(path)
        assert b["_compressed"]
        assert list(b["_types"]) == ATTRS
        assert [b["_types"][a][1] for a in ATTRS] == [1, 1, 1, 5, 0, 0, 5]   # partio INT / VECTOR / FLOAT
        m = ts.getFluidModel()
        np.testing.assert_array_equal(b["id"], np.arange(sc.n))
        assert (b["state"] == 0).all() and (b["object_id"] == 0).all()
        np.testing.assert_array_equal(b["position"], m.getFieldBuffer("position").astype(np.float32))
        for name in ("velocity", "p / rho^2", "p_v / rho^2", "velocity difference"):
            np.testing.assert_array_equal(b[name], m.getFieldBuffer(name).astype(np.float32))
    finally:
        ts.close()


@pytest.mark.gpu
def test_device_loads_its_own_state_file(tmp_path):
    from splishsplash_gb300.dfsph import TimeStepDFSPH
    sc = scenes.small_block(counts=(8, 10, 8), box=(0.6, 0.8, 0.6), viscosity=True, velocity=(0.2, 0, 0)).as_float32()
    a = TimeStepDFSPH(sc)
    b = TimeStepDFSPH(sc)
    try:
        for _ in range(8):
            st = a.step()
        path = str(tmp_path / "state.bgeo")
        a.ctx.save_particle_state(path, level=0)
        b.ctx.load_particle_state(path)
        b.setTimeStepSize(a.getTimeStepSize())
        b.ctx.set_time(st["time"])
        for name in ("position", "velocity", "p / rho^2", "p_v / rho^2", "velocity difference"):
            np.testing.assert_array_equal(b.getFluidModel().getFieldBuffer(name),
                                          a.getFluidModel().getFieldBuffer(name).astype(np.float32))
        sa, sb = a.step(), b.step()
        assert (sa["iterations"], sa["iterations_v"]) == (sb["iterations"], sb["iterations_v"])
        va, vb = a.getFluidModel().getFieldBuffer("velocity"), b.getFluidModel().getFieldBuffer("velocity")
        assert ref_cases.rel_vec(vb, va, 1e-3) < 1e-4
    finally:
        a.close()
        b.close()


@pytest.mark.gpu
def test_reference_state_file_continues_on_device():
    from splishsplash_gb300.dfsph import TimeStepDFSPH
    scene, g = fixture("reference")
    ts = TimeStepDFSPH(scene, use_graph=False)
    try:
        ts.ctx.load_particle_state(os.path.join(GOLDEN, "reference_state_column.bgeo"))
        ts.setTimeStepSize(float(g["dt"]))
        ts.ctx.set_time(float(g["time"]))
        m = ts.getFluidModel()
        for name, key in (("velocity", "v"), ("p / rho^2", "kappa"), ("p_v / rho^2", "kappa_v"),
                          ("velocity difference", "vdiff")):
            np.testing.assert_array_equal(m.getFieldBuffer(name), g[f"stored_{key}"].astype(np.float64))
        st = ts.step()
        got = dict(density=m.getFieldBuffer("density"), factor=m.getFieldBuffer("factor"),
                   kappa=m.getFieldBuffer("p / rho^2"), kappa_v=m.getFieldBuffer("p_v / rho^2"),
                   v=m.getFieldBuffer("velocity"), x=m.getFieldBuffer("position"),
                   vdiff=m.getFieldBuffer("velocity difference"))
        check_step(got, st, g)
    finally:
        ts.close()


@pytest.mark.gpu
def test_state_file_rejects_mismatched_scene(tmp_path):
    from splishsplash_gb300 import native
    from splishsplash_gb300.dfsph import TimeStepDFSPH
    scene, g = fixture("reference")
    small = scenes.small_block(counts=(6, 6, 6), viscosity=True).as_float32()
    ts = TimeStepDFSPH(small)
    try:
        with pytest.raises(native.SphgbError):
            ts.ctx.load_particle_state(os.path.join(GOLDEN, "reference_state_column.bgeo"))
        with pytest.raises(native.SphgbError):
            ts.ctx.load_particle_state(str(tmp_path / "missing.bgeo"))
    finally:
        ts.close()


# ------------------------------------------------------------------------- CPU, reference tree
@pytest.fixture(scope="module")
def state_lib():
    tree = refbuild.reference_tree()
    if tree is None:
        pytest.skip("reference tree not present (set SPH_REFERENCE_ROOT)")
    lib = refbuild.state_library(tree)
    L = refsim.lib("f64", lib)
    L.state_read.argtypes = [ctypes.c_char_p]
    L.bgeo_describe.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.bgeo_column.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    return lib, L


def test_partio_reads_the_device_state_file(state_lib):
    _, L = state_lib
    path = os.path.join(GOLDEN, "device_state_column.bgeo").encode()
    _, g = fixture("device")
    buf = ctypes.create_string_buffer(4096)
    n = ctypes.c_int()
    assert L.bgeo_describe(path, buf, 4096, ctypes.byref(n)) > 0
    kinds = dict(line.split(":") for line in buf.value.decode().strip().split("\n"))
    assert kinds == {"position": "V3", "id": "I1", "state": "I1", "object_id": "I1", "velocity": "V3",
                     "p / rho^2": "F1", "p_v / rho^2": "F1", "velocity difference": "V3"}
    npts = n.value
    assert npts == g["stored_x"].shape[0]

    def column(name, comps):
        out = np.zeros(npts * comps)
        assert L.bgeo_column(path, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size) == out.size
        return out.reshape(npts, comps) if comps > 1 else out

    ids = column("id", 1).astype(np.int64)
    np.testing.assert_array_equal(np.sort(ids), np.arange(npts))
    for name, key, comps in (("position", "x", 3), ("velocity", "v", 3), ("p / rho^2", "kappa", 1),
                             ("p_v / rho^2", "kappa_v", 1), ("velocity difference", "vdiff", 3)):
        vals = column(name, comps)
        np.testing.assert_array_equal(vals[np.argsort(ids)], g[f"stored_{key}"].astype(np.float64))


def test_reference_continues_from_the_device_state_file(state_lib):
    lib, L = state_lib
    scene, g = fixture("device")
    with refsim.RefSim(scene, library=lib) as r:
        assert L.state_read(os.path.join(GOLDEN, "device_state_column.bgeo").encode()) >= 7
        r.set_time_step(float(g["dt"]))
        s = r.step()
        got = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                   kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"),
                   vdiff=r.get("velocity difference"))
    check_step(got, s, g)
