"""The reference-side plugin (splishsplash_gb300/plugin/) compiled against the reference's
own headers and run inside the reference's own Simulation.

* TimeStepDFSPH_GB300, Viscosity_Weiler2018_GB300 and SimulationGB300 are compiled with the
  reference's SPlisHSPlasH headers (and the stand-ins of oracle/shims/ for its absent external
  projects), and linked with the reference's library objects (oracle/build_ref.sh).
* Linked against the real libsphgb300.so, every C-ABI symbol the plugin calls resolves
  (link check; running it needs a GPU and the reference tree, which a GPU host here lacks).
* Linked against tests/plugin/fake_sphgb300.cpp, a CPU stand-in of the same C ABI over the FP64
  oracle, the plugin drives the reference's Simulation through TimeStep::step(): the scene,
  parameters, warm starts, velocity differences, step sizes and time pass through the plugin's
  upload and download, and ten steps of the dam break of config 0 and of a viscous block match
  the reference's own TimeStepDFSPH step by step (iteration counts equal, fields to 1e-10).
These tests need the reference tree (SPH_REFERENCE_ROOT) and skip without it.
"""
import ctypes
import os

import numpy as np
import pytest

import ref_cases
import refbuild
import refsim
from splishsplash_gb300 import scenes


@pytest.fixture(scope="module")
def tree():
    t = refbuild.reference_tree()
    if t is None:
        pytest.skip("reference tree not present (set SPH_REFERENCE_ROOT)")
    return t


@pytest.fixture(scope="module")
def fake_lib(tree):
    return refbuild.plugin_fake_abi(tree)


def test_plugin_links_against_the_c_abi(tree):
    """Every sphgb_* symbol the plugin calls is exported by the real libsphgb300.so."""
    from splishsplash_gb300 import build as b
    if not os.path.exists(b.LIB):
        pytest.skip("libsphgb300.so not built")
    assert os.path.exists(refbuild.link_plugin_against(tree, os.path.dirname(b.LIB)))


def plugin_run(lib_path, scene, steps):
    L = refsim.lib("f64", lib_path)
    L.plugin_use_gb300_simulation.restype = ctypes.c_int
    L.plugin_install.restype = ctypes.c_int
    L.plugin_destroy.restype = None
    assert L.plugin_use_gb300_simulation() == 0
    r = refsim.RefSim(scene, library=lib_path)
    try:
        assert L.plugin_install() == 0
        return [r.step() for _ in range(steps)], fields(r, scene)
    finally:
        L.plugin_destroy()
        refsim.RefSim._alive = False


def reference_run(scene, steps):
    with refsim.RefSim(scene) as r:
        return [r.step() for _ in range(steps)], fields(r, scene)


def fields(r, scene):
    f = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
             kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"))
    if scene.params.viscosityMethod == 6:
        f["vdiff"] = r.get("velocity difference")
    return f


def viscous_block():
    sc = scenes.small_block(counts=(8, 12, 8), box=(0.5, 0.9, 0.5), viscosity=True)
    sc.v[:, 0] = sc.x[:, 1] - sc.x[:, 1].mean()
    sc.params.viscosity = 0.5
    return sc.as_float32()


@pytest.mark.parametrize("name", ["dambreak_8k", "viscous_block"])
def test_plugin_steps_match_reference_time_step(fake_lib, name):
    scene = scenes.dambreak_8k().as_float32() if name == "dambreak_8k" else viscous_block()
    steps = 10
    st_p, f_p = plugin_run(fake_lib, scene, steps)
    st_r, f_r = reference_run(scene, steps)
    for k, (a, b) in enumerate(zip(st_p, st_r)):
        assert (a["iterations"], a["iterations_v"], a["visco_iterations"]) == \
            (b["iterations"], b["iterations_v"], b["visco_iterations"]), k
        assert a["dt"] == pytest.approx(b["dt"], rel=1e-12)
        assert a["time"] == pytest.approx(b["time"], rel=1e-12)
    err = ref_cases.field_errors(f_p, f_r)
    for k, e in err.items():
        assert e <= 1e-10 * (np.max(np.abs(f_r["x"])) if k == "x" else 1.0), (name, k, e)
    if name == "viscous_block":
        assert max(s["visco_iterations"] for s in st_r) > 0


def _state_calls(lib_path):
    L = refsim.lib("f64", lib_path)
    for name in ("sim_state_write", "sim_state_read", "state_write", "state_read"):
        getattr(L, name).argtypes = [ctypes.c_char_p]
        getattr(L, name).restype = ctypes.c_int
    return L


def _load_and_step(L, lib_path, scene, bin_path, bgeo_path, steps, plugin):
    """A fresh Simulation loads the state files as SimulatorBase::loadState does (the .bin's
    library section, then the particle file) and takes `steps` steps."""
    if plugin:
        assert L.plugin_use_gb300_simulation() == 0
    r = refsim.RefSim(scene, library=lib_path)
    try:
        if plugin:
            assert L.plugin_install() == 0
        assert L.sim_state_read(bin_path) == 0
        assert L.state_read(bgeo_path) >= 6
        st = [r.step() for _ in range(steps)]
        return st, fields(r, scene)
    finally:
        if plugin:
            L.plugin_destroy()
            refsim.RefSim._alive = False
        else:
            r.close()


def test_plugin_state_files_round_trip(fake_lib, tmp_path):
    """The reference's state files with the plugin installed.  The simulator's saveState writes the
    library's section of the .bin (TimeManager and Simulation state) and the particle file from
    the host objects, which the plugin keeps current after every step; its loadState restores
    them and the plugin's TimeStep::loadState makes the next step upload them.  So: (1) the files
    written after 6 steps through the plugin equal those of the reference's own TimeStepDFSPH
    (the .bin byte for byte but for its floating-point time and step size, 1e-12; the particle
    file's float32 values within one rounding); (2) from the reference's files, 4 steps through
    the plugin match 4 steps of the reference's own time step at the 1e-10 bars."""
    L = _state_calls(fake_lib)
    L.plugin_use_gb300_simulation.restype = ctypes.c_int
    L.plugin_install.restype = ctypes.c_int
    L.plugin_destroy.restype = None
    scene = viscous_block()
    files = {}
    for side in ("reference", "plugin"):
        b, g = str(tmp_path / f"{side}.bin").encode(), str(tmp_path / f"{side}.bgeo").encode()
        if side == "plugin":
            assert L.plugin_use_gb300_simulation() == 0
        r = refsim.RefSim(scene, library=fake_lib)
        try:
            if side == "plugin":
                assert L.plugin_install() == 0
            for _ in range(6):
                r.step()
            assert L.sim_state_write(b) == 0
            assert L.state_write(g) == 8   # the storeData fields, position included
        finally:
            if side == "plugin":
                L.plugin_destroy()
                refsim.RefSim._alive = False
            else:
                r.close()
        files[side] = (b, g)
    rb, pb = open(files["reference"][0], "rb").read(), open(files["plugin"][0], "rb").read()
    # Real time, Real h, Real W_zero, uint n, n x ParticleState, emitter counts, per boundary model
    # (bool sorted, uint point set)
    assert len(rb) == len(pb) == 3 * 8 + 4 + 4 * scene.n + 8 + 5 * 1
    t_r, h_r, w_r = np.frombuffer(rb[:24], np.float64)
    t_p, h_p, w_p = np.frombuffer(pb[:24], np.float64)
    assert (t_p, h_p, w_p) == (pytest.approx(t_r, rel=1e-12), pytest.approx(h_r, rel=1e-12), w_r)
    assert rb[24:] == pb[24:]
    assert np.frombuffer(rb[24:28], np.uint32)[0] == scene.n
    st_r, f_r = _load_and_step(L, fake_lib, scene, *files["reference"], 4, plugin=False)
    st_p, f_p = _load_and_step(L, fake_lib, scene, *files["reference"], 4, plugin=True)
    for a, b in zip(st_p, st_r):
        assert (a["iterations"], a["iterations_v"], a["visco_iterations"]) == \
            (b["iterations"], b["iterations_v"], b["visco_iterations"])
        assert a["time"] == pytest.approx(b["time"], rel=1e-12)
    assert st_r[0]["time"] == pytest.approx(t_r + h_r, rel=1e-12)
    err = ref_cases.field_errors(f_p, f_r)
    for k, e in err.items():
        assert e <= 1e-10 * (np.max(np.abs(f_r["x"])) if k == "x" else 1.0), (k, e)
