"""One-step fixtures recorded from the reference's own DFSPH time step (tests/golden/
ref_step_*.npz, made by tests/golden/gen_ref_steps.py), and the bars they are held to."""
import dataclasses
import json
import os

import numpy as np

from splishsplash_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("block12", "column_visc", "dambreak8k_step203", "vmap_box", "phases_visc", "caps_cfl_iter", "fixed_dt_nodiv")


def load_case(name):
    """(scene, state, reference outputs) of a fixture; state arrays are float32 values."""
    g = np.load(os.path.join(GOLDEN, f"ref_step_{name}.npz"))
    params = scenes.SPHParams(**{k: (tuple(v) if isinstance(v, list) else v)
                                 for k, v in json.loads(str(g["params"])).items()})
    x = g["x"].astype(np.float64)
    scene = scenes.Scene(f"ref_{name}", x, g["v"].astype(np.float64), g["xb"].astype(np.float64), params,
                         np.asarray(g["box_min"]), np.asarray(g["box_max"]))
    state = dict(x=x, v=g["v"].astype(np.float64), kappa=g["kappa"].astype(np.float64),
                 kappa_v=g["kappa_v"].astype(np.float64), vdiff=g["vdiff"].astype(np.float64), dt=float(g["dt"]))
    out = {k[4:]: (g[k] if g[k].ndim else g[k].item()) for k in g.files if k.startswith("out_")}
    return scene, state, out


def load_run(name):
    """(scene, per-step iteration counts [steps, 3], per-step (dt used, dt next) [steps, 2], final
    reference fields) of a run fixture (tests/golden/ref_run_<name>.npz): the reference's steps
    from the scene's float32 initial state."""
    g = np.load(os.path.join(GOLDEN, f"ref_run_{name}.npz"))
    params = scenes.SPHParams(**{k: (tuple(v) if isinstance(v, list) else v)
                                 for k, v in json.loads(str(g["params"])).items()})
    scene = scenes.Scene(f"ref_run_{name}", g["x"].astype(np.float64), g["v"].astype(np.float64),
                         g["xb"].astype(np.float64), params, np.asarray(g["box_min"]), np.asarray(g["box_max"]))
    out = {k[4:]: g[k] for k in g.files if k.startswith("out_")}
    return scene, g["iterations"], g["dt"], out


def vmap_spec(name):
    """(cells per axis, box) of a fixture whose boundary is a Bender2019 volume map of a box
    container, or None for boundary particles"""
    g = np.load(os.path.join(GOLDEN, f"ref_step_{name}.npz"))
    if "vmap_res" not in g.files:
        return None
    return tuple(int(r) for r in g["vmap_res"]), tuple(float(b) for b in g["vmap_box"])


def case_maps(name, support):
    """The oracle's volume maps of a fixture (oracle/vmap.c, from the box mesh), or None"""
    spec = vmap_spec(name)
    if spec is None:
        return None
    import oracle
    v, f = scenes.box_mesh((0, 0, 0), spec[1])
    return [oracle.VolumeMap(spec[0]).build(v, f, support, invert=True)]


def case_phases(name):
    """The fluid models of a fixture (counts, density0 and per-model viscosity and XSPH
    coefficients, as refsim.RefSim takes them), or None for one model"""
    g = np.load(os.path.join(GOLDEN, f"ref_step_{name}.npz"))
    if "phase_counts" not in g.files:
        return None
    out = {k[6:]: g[k] for k in g.files if k.startswith("phase_")}
    out["counts"] = tuple(int(c) for c in out["counts"])
    return out


def rel_scalar(a, b, floor):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def rel_vec(a, b, floor):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = np.linalg.norm(a - b, axis=-1)
    return float(np.max(d / np.maximum(np.linalg.norm(b, axis=-1), floor)))


def field_errors(got, ref):
    """Max relative error per field against the reference's step, with the floors of the
    comparison protocol: rho0 1e-6 for density, the median |alpha| for alpha, 1e-3 of the
    largest |kappa| for kappa and kappa_v, 1e-3 m/s for velocity."""
    e = {
        "density": rel_scalar(got["density"], ref["density"], 1e-3),
        "factor": rel_scalar(got["factor"], ref["factor"], float(np.median(np.abs(ref["factor"])))),
        "v": rel_vec(got["v"], ref["v"], 1e-3),
        "x": float(np.max(np.abs(np.asarray(got["x"]) - ref["x"]))),
    }
    for k in ("kappa", "kappa_v"):
        m = float(np.max(np.abs(ref[k])))
        e[k] = float(np.max(np.abs(np.asarray(got[k]) - ref[k]))) / m if m > 0 else 0.0
    if "vdiff" in ref and "vdiff" in got:
        e["vdiff"] = rel_vec(got["vdiff"], ref["vdiff"], 1e-3)
    return e


def with_state(scene, state):
    return dataclasses.replace(scene, x=state["x"], v=state["v"])
