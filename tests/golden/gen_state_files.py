"""Generate the particle-state-file fixtures (the reference's per-fluid-model state files,
SimulatorBase::writeFluidParticlesState / readFluidParticlesState).

    python tests/golden/gen_state_files.py --side reference --out tests/golden
        (where the reference tree is present: the reference's FP64 build writes its state
        file through partio, reads it back and records one step from it)
    python tests/golden/gen_state_files.py --side device --out <dir>
        (on a GPU: the device writes its state file with sphgb_save_particle_state, a fresh
        context loads it with sphgb_load_particle_state and records one step from it; copy
        the two outputs to tests/golden)

Scene: a 10 x 20 x 10 column (r = 0.025) with a shear velocity field and Weiler2018
viscosity nu = 0.2, advanced 40 steps before the state is written.  Outputs, by particle id:
  <side>_state_column.bgeo   the state file
  <side>_state_column.npz    params (JSON), dt and time of the state, the state's fields as
                             stored (float32), and the step taken from the file: density,
                             kappa, kappa_v, velocity, position, velocity difference,
                             iteration counts and the next step size
"""
import argparse
import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from splishsplash_gb300 import scenes  # noqa: E402

WARM = 40


def column():
    sc = scenes.small_block(counts=(10, 20, 10), box=(0.6, 1.4, 0.6), viscosity=True)
    sc.v[:, 0] = 1.0 * (sc.x[:, 1] - sc.x[:, 1].mean())
    sc.v[:, 2] = 0.5 * np.sin(8.0 * sc.x[:, 0])
    sc.params.viscosity = 0.2
    return sc.as_float32()


def reference_side(out):
    import ctypes

    import refbuild
    import refsim
    tree = refbuild.reference_tree()
    lib = refbuild.state_library(tree)
    L = refsim.lib("f64", lib)
    L.state_write.argtypes = [ctypes.c_char_p]
    L.state_read.argtypes = [ctypes.c_char_p]
    sc = column()
    path = os.path.join(out, "reference_state_column.bgeo")
    with refsim.RefSim(sc, library=lib) as r:
        for _ in range(WARM):
            st = r.step()
        assert L.state_write(path.encode()) > 0
        assert L.state_read(path.encode()) > 0   # continue from the values as stored
        stored = dict(x=r.get("position"), v=r.get("velocity"), kappa=r.get("p / rho^2"),
                      kappa_v=r.get("p_v / rho^2"), vdiff=r.get("velocity difference"))
        dt, time = st["dt"], st["time"]
        s = r.step()
        nxt = dict(density=r.get("density"), factor=r.get("factor"), kappa=r.get("p / rho^2"),
                   kappa_v=r.get("p_v / rho^2"), v=r.get("velocity"), x=r.get("position"),
                   vdiff=r.get("velocity difference"))
    save(out, "reference", sc, dt, time, stored, nxt, s["iterations"], s["iterations_v"], s["visco_iterations"],
         s["dt"])


def device_side(out):
    from splishsplash_gb300.dfsph import TimeStepDFSPH
    sc = column()
    path = os.path.join(out, "device_state_column.bgeo")
    ts = TimeStepDFSPH(sc, use_graph=True)
    for _ in range(WARM):
        st = ts.step()
    ts.ctx.save_particle_state(path)
    dt, time = ts.getTimeStepSize(), st["time"]
    ts.close()
    ts = TimeStepDFSPH(sc, use_graph=False)
    ts.ctx.load_particle_state(path)
    ts.setTimeStepSize(dt)
    ts.ctx.set_time(time)
    m = ts.getFluidModel()
    stored = dict(x=m.getFieldBuffer("position"), v=m.getFieldBuffer("velocity"), kappa=m.getFieldBuffer("p / rho^2"),
                  kappa_v=m.getFieldBuffer("p_v / rho^2"), vdiff=m.getFieldBuffer("velocity difference"))
    s = ts.step()
    nxt = dict(density=m.getFieldBuffer("density"), factor=m.getFieldBuffer("factor"),
               kappa=m.getFieldBuffer("p / rho^2"), kappa_v=m.getFieldBuffer("p_v / rho^2"),
               v=m.getFieldBuffer("velocity"), x=m.getFieldBuffer("position"),
               vdiff=m.getFieldBuffer("velocity difference"))
    ts.close()
    save(out, "device", sc, dt, time, stored, nxt, s["iterations"], s["iterations_v"], s["visco_iterations"],
         s["dt_next"])


def save(out, side, sc, dt, time, stored, nxt, it, itv, itc, dt_next):
    np.savez_compressed(
        os.path.join(out, f"{side}_state_column.npz"), params=json.dumps(dataclasses.asdict(sc.params)),
        xb=sc.xb.astype(np.float32), box_min=sc.box_min, box_max=sc.box_max, dt=dt, time=time,
        **{f"stored_{k}": v.astype(np.float32) for k, v in stored.items()},
        **{f"next_{k}": v for k, v in nxt.items()}, iterations=it, iterations_v=itv, visco_iterations=itc,
        dt_next=dt_next)
    print(side, "state written; next step iterations", it, itv, itc)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--side", choices=["reference", "device"], required=True)
    ap.add_argument("--out", default=HERE)
    a = ap.parse_args()
    os.makedirs(a.out, exist_ok=True)
    (reference_side if a.side == "reference" else device_side)(a.out)
