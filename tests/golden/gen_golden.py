"""Generate the committed golden fixtures from the reference's own code.

Run in a checkout that has the reference tree (default path from
SPH_REFERENCE_ROOT, else the container's read-only mount):

    oracle/build_ref.sh && python tests/golden/gen_golden.py

Fixtures written next to this script:
  kernel_ref.npz  -- SPH::CubicKernel (FP64 build) and SPH::CubicKernel_AVX
                     (FP32 AVX build) W / gradW at sampled offsets, support 0.1
                     (the support radius of Tests/Kernel/KernelTests.cpp:19).
  cg_ref.npz      -- Eigen ConjugateGradient + BlockJacobiPreconditioner3D from
                     SPlisHSPlasH/Utilities/MatrixFreeSolver.h on a Weiler2018
                     system of a small jittered block (operator from the oracle).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from splishsplash_gb300 import scenes  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def kernel_points(support=0.1, seed=11):
    rng = np.random.default_rng(seed)
    pts = [rng.uniform(-1.2 * support, 1.2 * support, size=(2000, 3))]
    # the KernelTests lattice rows through the origin (KernelTests.cpp:124-170)
    steps = 50
    st = 2.0 * support / (steps - 1)
    line = -support + np.arange(steps) * st
    pts.append(np.stack([np.zeros(steps), np.zeros(steps), line], 1))
    # tiny offsets (KernelTests.cpp:172-225)
    width = 1e-5
    line2 = -width + np.arange(200) * (width / 199)
    pts.append(np.stack([np.zeros(200), np.zeros(200), line2], 1))
    # exact branch points q = 0, 0.5, 1 and just beyond
    for q in (0.0, 0.25, 0.5, 0.75, 1.0, 1.0 + 1e-7):
        pts.append(np.array([[q * support, 0.0, 0.0], [0.0, q * support, 0.0]]))
    return np.concatenate(pts, 0)


def run(exe, *args):
    subprocess.run([os.path.join(REF, exe)] + [str(a) for a in args], check=True)


def gen_kernel():
    support = 0.1
    r = kernel_points(support)
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.f64")
        r.astype(np.float64).tofile(fin)
        run("ref_pin_f64", "kernel", support, fin, os.path.join(td, "o64"))
        o64 = np.fromfile(os.path.join(td, "o64"), np.float64).reshape(-1, 4)
        out = dict(r=r, support=support, cubic_f64=o64)
        if os.path.exists(os.path.join(REF, "ref_pin_f32")):
            run("ref_pin_f32", "kernel", support, fin, os.path.join(td, "o32"))
            o32 = np.fromfile(os.path.join(td, "o32"), np.float64).reshape(2, -1, 4)
            out["cubic_f32"] = o32[0]
            out["cubic_avx_f32"] = o32[1]
    np.savez_compressed(os.path.join(HERE, "kernel_ref.npz"), **out)
    print("kernel_ref.npz:", r.shape[0], "points")


def gen_cg():
    sc = scenes.small_block(counts=(6, 6, 6), radius=0.025, seed=21, box=(0.6, 0.6, 0.6), viscosity=True)
    rng = np.random.default_rng(5)
    sc.v[:] = rng.uniform(-0.3, 0.3, size=sc.v.shape)
    sc = sc.as_float32()
    sim = oracle.OracleSim(sc)
    # densities of the initial positions via one oracle step on a copy
    probe = oracle.OracleSim(sc)
    probe.step()
    density = probe.density.copy()
    vdiff = rng.uniform(-0.01, 0.01, size=(sc.n, 3))
    dt = 0.002
    tol = 1e-6
    max_iter = 100
    header = np.array([sc.n, sc.nb, sc.params.particleRadius, sc.params.density0, sc.params.viscosity,
                       0.0, dt, tol, max_iter], np.float64)
    blob = np.concatenate([header, sc.x.ravel(), sc.v.ravel(), density, vdiff.ravel(), sim.xb.ravel(),
                           sim.Vb.astype(np.float64)])
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "cg.f64")
        blob.tofile(fin)
        run("ref_pin_f64", "cg", fin, os.path.join(td, "out"))
        res = np.fromfile(os.path.join(td, "out"), np.float64)
    np.savez_compressed(os.path.join(HERE, "cg_ref.npz"), x=sc.x, v=sc.v, density=density, vdiff=vdiff,
                        xb=sim.xb, Vb=sim.Vb, radius=sc.params.particleRadius, density0=sc.params.density0,
                        viscosity=sc.params.viscosity, dt=dt, tol=tol, max_iter=max_iter,
                        iterations=res[0], error=res[1], solution=res[2:].reshape(-1, 3))
    print("cg_ref.npz: n =", sc.n, "iterations", res[0], "error", res[1])


if __name__ == "__main__":
    gen_kernel()
    gen_cg()
