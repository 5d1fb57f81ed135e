"""Generate one-step fixtures from the reference's own DFSPH time step.

The reference's SPlisHSPlasH sources are compiled by oracle/build_ref.sh into
oracle/_ref/libref_f64.so (FP64, analytic cubic spline, the oracle protocol) and
driven through oracle/refsim.py.  Run in a checkout that has the reference tree:

    oracle/build_ref.sh && python tests/golden/gen_ref_steps.py

Each case advances a seeded scene with the reference for `warm` steps, rounds the
state to float32 (the state the FP32 device path can hold exactly), builds a fresh
reference simulation from that state and records one reference step.  Written next
to this script, by particle id:
  ref_step_<case>.npz   inputs: x, v, kappa, kappa_v, vdiff (float32), dt, xb
                        (float32), params (JSON); outputs (float64): density,
                        factor, density_adv, kappa, kappa_v, v, x, vdiff, dt_next,
                        time step counts (iterations, iterations_v, visco_iterations)
  The volume-map case (vmap_box) has no boundary particles: its boundary is a Bender2019
  volume map of the box, built by the oracle (oracle/vmap.c) from the box mesh and handed to
  the reference's Bender2019 code through the driver's Discregrid grid; the fixture records
  the map's cells per axis and box (vmap_res, vmap_box) so that a test rebuilds it.
  The two-model case (phases_visc) is a column of two fluid models (rest densities 1000 and
  500, the heavy one below) with their own Weiler2018 and XSPH coefficients; the fixture
  records the models (phase_counts, phase_density0, phase_viscosity, phase_viscosity_boundary,
  phase_xsph, phase_xsph_boundary).
  The solver-parameter cases: caps_cfl_iter (iteration caps below what the solvers need and the
  iteration-adapted CFL step size) and fixed_dt_nodiv (fixed step size, no divergence solve,
  a pressure-iteration minimum, XSPH with its boundary term).
  ref_run_cfl_iter.npz  25 steps of a compressed block with the iteration-adapted CFL step
                        size from its initial state: iteration counts and step sizes per step,
                        the final fields
  ref_kernel_table_delta.json  the same config-0 step with the reference's default
                        PrecomputedKernel<CubicKernel, 10000> against the analytic
                        kernel: max and mean relative difference per field
"""
import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refsim  # noqa: E402
from splishsplash_gb300 import scenes  # noqa: E402

OUT_FIELDS = ("density", "factor", "advected density", "p / rho^2", "p_v / rho^2", "velocity", "position",
              "velocity difference")
KEYS = {"density": "density", "factor": "factor", "advected density": "density_adv", "p / rho^2": "kappa",
        "p_v / rho^2": "kappa_v", "velocity": "v", "position": "x", "velocity difference": "vdiff"}


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def advanced_state(scene, warm, maps=None, phases=None):
    """The scene after `warm` reference steps, rounded to float32."""
    visc = scene.params.viscosityMethod == 6
    with refsim.RefSim(scene, volume_maps=maps, phases=phases) as r:
        for _ in range(warm):
            r.step()
        st = dict(x=f32(r.get("position")), v=f32(r.get("velocity")), kappa=f32(r.get("p / rho^2")),
                  kappa_v=f32(r.get("p_v / rho^2")),
                  vdiff=f32(r.get("velocity difference")) if visc else np.zeros((scene.n, 3)),
                  dt=float(r.stats()["dt"]) if warm else scene.params.timeStepSize)
    return st


def step_from(scene, st, analytic=True, maps=None, phases=None):
    """One reference step from state st; outputs by particle id."""
    sc = dataclasses.replace(scene, x=st["x"], v=st["v"])
    visc = scene.params.viscosityMethod == 6
    with refsim.RefSim(sc, analytic_kernel=analytic, volume_maps=maps, phases=phases) as r:
        r.set("p / rho^2", st["kappa"])
        r.set("p_v / rho^2", st["kappa_v"])
        if visc:
            r.set("velocity difference", st["vdiff"])
        r.set_time_step(st["dt"])
        s = r.step()
        out = {KEYS[f]: r.get(f) for f in OUT_FIELDS if visc or f != "velocity difference"}
    out["dt_next"] = s["dt"]
    out["iterations"] = s["iterations"]
    out["iterations_v"] = s["iterations_v"]
    out["visco_iterations"] = s["visco_iterations"]
    return out


def viscous_column():
    """A 10x20x10 column with a shear velocity field and nu = 1, so that one step runs
    tens of pressure iterations and about ten Weiler2018 CG iterations."""
    sc = scenes.small_block(counts=(10, 20, 10), box=(0.6, 1.4, 0.6), viscosity=True)
    sc.v[:, 0] = 1.0 * (sc.x[:, 1] - sc.x[:, 1].mean())
    sc.v[:, 2] = 0.5 * np.sin(8.0 * sc.x[:, 0])
    sc.params.viscosity = 1.0
    return sc


VMAP_BOX = (0.8, 1.0, 0.8)
VMAP_RES = (10, 12, 10)


def vmap_box():
    """A 10x14x10 block with a shear velocity field in a volume-mapped 0.8 x 1.0 x 0.8 m box:
    Weiler2018 (nu = 0.2) with boundary viscosity 0.05, XSPH with its boundary term."""
    sc = scenes.small_block(counts=(10, 14, 10), box=VMAP_BOX, viscosity=True)
    sc.v[:, 0] = 1.0 * (sc.x[:, 1] - sc.x[:, 1].mean())
    sc.v[:, 2] = 0.5 * np.sin(8.0 * sc.x[:, 0])
    sc.xb = np.zeros((0, 3))
    sc.params.viscosity = 0.2
    sc.params.viscosityBoundary = 0.05
    sc.params.xsphBoundary = 0.1
    return sc


def box_volume_map(support, res=VMAP_RES, box=VMAP_BOX):
    import oracle
    v, f = scenes.box_mesh((0, 0, 0), box)
    return oracle.VolumeMap(res).build(v, f, support, invert=True)


PHASES = dict(density0=(1000.0, 500.0), viscosity=(0.3, 0.05), viscosity_boundary=(0.05, 0.0),
              xsph=(0.01, 0.1), xsph_boundary=(0.1, 0.0))


def phases_visc():
    """An 8x10x8 column, its lower half fluid model 0 (rest density 1000) and upper half model 1
    (500), particles ordered by height; Weiler2018 and XSPH with per-model coefficients."""
    sc = scenes.small_block(counts=(8, 10, 8), box=(0.6, 0.8, 0.6), corner=(0.05, 0.05, 0.05),
                            velocity=(0.2, -0.3, 0.1), viscosity=True)
    order = np.argsort(sc.x[:, 1], kind="stable")
    sc.x, sc.v = sc.x[order].copy(), sc.v[order].copy()
    n0 = sc.n // 2
    return sc, dict(counts=(n0, sc.n - n0), **PHASES)


def block12():
    return scenes.small_block(counts=(12, 12, 12), box=(0.8, 0.8, 0.8), velocity=(0.3, 0.0, -0.2))


def caps_cfl_iter():
    """The viscous column with the solvers capped below what they need (4 pressure, 2 divergence
    and 4 CG iterations) and the iteration-adapted CFL step size (cflMethod 2)."""
    sc = viscous_column()
    p = sc.params
    p.maxIterations, p.maxIterationsV, p.viscoMaxIter, p.cflMethod = 4, 2, 4, 2
    return sc


def fixed_dt_nodiv():
    """The 12^3 block at a fixed step size (cflMethod 0, 2 ms), without the divergence solver,
    at least 5 pressure iterations, XSPH 0.05 with a boundary term of 0.1 and no viscosity."""
    sc = block12()
    p = sc.params
    p.cflMethod, p.timeStepSize, p.enableDivergenceSolver, p.minIterations = 0, 0.002, False, 5
    p.xsph, p.xsphBoundary = 0.05, 0.1
    return sc


def cases():
    return {
        "block12": (block12(), 30),
        "column_visc": (viscous_column(), 70),
        "dambreak8k_step203": (scenes.dambreak_8k(), 202),
        "vmap_box": (vmap_box(), 40),
        "phases_visc": (phases_visc()[0], 30),
        "caps_cfl_iter": (caps_cfl_iter(), 40),
        "fixed_dt_nodiv": (fixed_dt_nodiv(), 30),
    }


RUN_STEPS = 25


def cfl_iter_block():
    """A 12^3 block compressed to 0.84 of its spacing (30 % over the rest density) with the
    iteration-adapted CFL step size (cflMethod 2): tens of pressure iterations in its first
    steps shrink the step size (x 0.9 after more than 10), the expanding block then limits it by
    the velocity CFL, and the few iterations after grow it (x 1.1 after fewer than 5)."""
    sc = scenes.small_block(counts=(12, 12, 12), box=(1.0, 1.0, 1.0), corner=(0.2, 0.2, 0.2))
    c = sc.x.mean(axis=0)
    sc.x = c + 0.84 * (sc.x - c)
    sc.params.cflMethod = 2
    return sc


def run_fixture():
    """ref_run_cfl_iter.npz: RUN_STEPS reference steps of cfl_iter_block from its float32
    initial state, each step's iteration counts and step sizes, and the final fields, so that a
    run (the CFL adaptation reads the previous step's pressure iterations) can be followed."""
    scene = cfl_iter_block().as_float32()
    its, dts = [], []
    with refsim.RefSim(scene) as r:
        for _ in range(RUN_STEPS):
            s = r.step()
            its.append((s["iterations"], s["iterations_v"], s["visco_iterations"]))
            dts.append((s["dt_old"], s["dt"]))
        visc = scene.params.viscosityMethod == 6
        out = {KEYS[f]: r.get(f) for f in OUT_FIELDS
               if f != "advected density" and (visc or f != "velocity difference")}
    np.savez_compressed(
        os.path.join(HERE, "ref_run_cfl_iter.npz"), params=json.dumps(dataclasses.asdict(scene.params)),
        x=scene.x.astype(np.float32), v=scene.v.astype(np.float32), xb=scene.xb.astype(np.float32),
        box_min=scene.box_min, box_max=scene.box_max, iterations=np.array(its), dt=np.array(dts),
        **{f"out_{k}": v for k, v in out.items()})
    print("run cfl_iter", scene.n, "particles", RUN_STEPS, "steps; iterations", its[-1], "dt", dts[-1])


def main():
    only = set(sys.argv[1:])
    for name, (scene, warm) in cases().items():
        if only and name not in only:
            continue
        scene = scene.as_float32()
        maps = [box_volume_map(scene.params.supportRadius)] if name == "vmap_box" else None
        phases = phases_visc()[1] if name == "phases_visc" else None
        st = advanced_state(scene, warm, maps, phases)
        out = step_from(scene, st, maps=maps, phases=phases)
        params = dataclasses.asdict(scene.params)
        extra = dict(vmap_res=np.array(VMAP_RES), vmap_box=np.array(VMAP_BOX)) if maps else {}
        if phases:
            extra = {f"phase_{k}": np.array(v) for k, v in phases.items()}
        np.savez_compressed(
            os.path.join(HERE, f"ref_step_{name}.npz"),
            params=json.dumps(params), warm=warm,
            x=st["x"].astype(np.float32), v=st["v"].astype(np.float32), kappa=st["kappa"].astype(np.float32),
            kappa_v=st["kappa_v"].astype(np.float32), vdiff=st["vdiff"].astype(np.float32), dt=st["dt"],
            xb=scene.xb.astype(np.float32), box_min=scene.box_min, box_max=scene.box_max, **extra,
            **{f"out_{k}": v for k, v in out.items()})
        print(name, scene.n, "particles, warm", warm, "iterations", out["iterations"], out["iterations_v"],
              out["visco_iterations"])
    if not only or "run_cfl_iter" in only:
        run_fixture()
    if only and "dambreak8k_step203" not in only:
        return
    # lookup-table kernel against the analytic kernel, on the config-0 step above
    scene, warm = cases()["dambreak8k_step203"]
    scene = scene.as_float32()
    st = advanced_state(scene, warm)
    a = step_from(scene, st, analytic=True)
    t = step_from(scene, st, analytic=False)
    delta = {"case": f"dambreak_8k, one step after {warm} steps, FP64 reference build",
             "iterations": {"analytic": [a["iterations"], a["iterations_v"]],
                            "table": [t["iterations"], t["iterations_v"]]}}
    for k in ("density", "factor", "kappa", "kappa_v", "v", "x"):
        ra, rt = np.asarray(a[k]), np.asarray(t[k])
        if ra.ndim == 2:
            d = np.linalg.norm(rt - ra, axis=1)
            den = np.maximum(np.linalg.norm(ra, axis=1), 1e-3 if k == "v" else 1e-12)
        else:
            d = np.abs(rt - ra)
            floor = {"density": 1e-3, "factor": float(np.median(np.abs(ra))),
                     "kappa": 1e-3 * float(np.max(np.abs(ra))) or 1e-30,
                     "kappa_v": 1e-3 * float(np.max(np.abs(ra))) or 1e-30}[k]
            den = np.maximum(np.abs(ra), floor)
        rel = d / den
        delta[k] = {"max_rel": float(rel.max()), "mean_rel": float(rel.mean())}
    with open(os.path.join(HERE, "ref_kernel_table_delta.json"), "w") as f:
        json.dump(delta, f, indent=1)
    print(json.dumps(delta))


if __name__ == "__main__":
    main()
