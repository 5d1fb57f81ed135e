"""Pins the CPU oracle against the reference's own code (fixtures in tests/golden/,
made by tests/golden/gen_golden.py from oracle/_ref builds of the reference sources)
and against the reference's kernel tests (Tests/Kernel/KernelTests.cpp)."""
import os

import numpy as np
import pytest

import oracle
from splishsplash_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_kernel_normalized_positive():
    # Tests/Kernel/KernelTests.cpp:17-47 (FP64 tolerance 1e-5)
    h = 4.0 * 0.025
    steps = 50
    st = 2.0 * h / (steps - 1)
    V = st ** 3
    c = -h + np.arange(steps) * st
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    W = np.array([oracle.kernel_W(np.linalg.norm(p), h) for p in pts])
    G = np.array([oracle.kernel_gradW(-p, h) for p in pts])
    assert abs(W.sum() * V - 1.0) < 1e-5
    assert np.linalg.norm(G.sum(0) * V) < 1e-5
    assert (W >= -1e-5).all()


def test_kernel_matches_reference_cubic_fp64():
    g = np.load(os.path.join(GOLDEN, "kernel_ref.npz"))
    h = float(g["support"])
    ref = g["cubic_f64"]
    for r, row in zip(g["r"], ref):
        assert oracle.kernel_W(np.linalg.norm(r), h) == pytest.approx(row[0], rel=1e-12, abs=1e-9)
        np.testing.assert_allclose(oracle.kernel_gradW(r, h), row[1:], rtol=1e-12, atol=1e-9)


def test_reference_avx_kernel_agrees_with_analytic():
    # KernelTests.cpp:124-231 bars: |W_avx - W| <= 1e-3, |gradW_avx - gradW| <= 3e-2
    g = np.load(os.path.join(GOLDEN, "kernel_ref.npz"))
    if "cubic_avx_f32" not in g:
        pytest.skip("fixture made without the AVX build")
    h = float(g["support"])
    for r, row in zip(g["r"], g["cubic_avx_f32"]):
        assert abs(row[0] - oracle.kernel_W(np.linalg.norm(r), h)) <= 1e-3
        assert np.linalg.norm(row[1:] - oracle.kernel_gradW(r, h)) <= 3e-2


def test_cg_matches_reference_eigen_blockjacobi():
    import ctypes
    g = np.load(os.path.join(GOLDEN, "cg_ref.npz"))
    p = scenes.SPHParams(particleRadius=float(g["radius"]), density0=float(g["density0"]),
                         viscosity=float(g["viscosity"]), viscosityMethod=6,
                         viscoMaxError=float(g["tol"]), viscoMaxIter=int(g["max_iter"]))
    n, nb = g["x"].shape[0], g["xb"].shape[0]
    st = oracle.OrcState()
    keep = {}
    for name in ("x", "v", "density", "vdiff", "xb", "Vb"):
        keep[name] = np.ascontiguousarray(g[name], np.float64)
        setattr(st, name, keep[name].ctypes.data_as(ctypes.c_void_p))
    st.n, st.nb = n, nb
    cp = oracle.make_params(p)
    xs = np.zeros((n, 3), np.float64)
    it = ctypes.c_uint(0)
    err = ctypes.c_double(0)
    rc = oracle.lib().orc_weiler_solve(ctypes.byref(st), ctypes.byref(cp), float(g["dt"]),
                                       xs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(it), ctypes.byref(err))
    assert rc == 0
    assert it.value == int(g["iterations"])
    np.testing.assert_allclose(xs, g["solution"], rtol=1e-10, atol=1e-12)
    assert err.value == pytest.approx(float(g["error"]), rel=1e-6)


def test_neighbor_search_matches_brute_force():
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 0.5, size=(700, 3))
    y = rng.uniform(-0.05, 0.55, size=(300, 3))
    h = 0.1
    for same, pts in ((True, x), (False, y)):
        off, idx = oracle.neighbors(x, pts, h, same, fp32=False)
        d2 = ((x[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
        for i in range(x.shape[0]):
            want = np.nonzero(d2[i] < h * h)[0]
            if same:
                want = want[want != i]
            np.testing.assert_array_equal(idx[off[i]:off[i + 1]], want)


def test_fp32_predicate_is_float_arithmetic():
    # pairs at exactly the support radius on an unjittered lattice: the float
    # predicate decides ties by float rounding of dx*dx + dy*dy + dz*dz
    sc = scenes.small_block(counts=(5, 5, 5), jitter=0.0)
    x = sc.x.astype(np.float32)
    h = sc.params.supportRadius
    off, idx = oracle.neighbors(x.astype(np.float64), x.astype(np.float64), h, True, fp32=True)
    h2f = np.float32(h * h)
    for i in range(0, x.shape[0], 7):
        d = x[i] - x
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        want = np.nonzero(d2 < h2f)[0]
        want = want[want != i]
        np.testing.assert_array_equal(idx[off[i]:off[i + 1]], want)


def test_oracle_dambreak_runs_stable():
    sim = oracle.OracleSim(scenes.dambreak_8k().as_float32())
    for _ in range(60):
        sim.step()
    st = sim.stats()
    assert np.isfinite(sim.x).all() and np.isfinite(sim.v).all()
    assert st["avg_density_err"] <= 0.01 * 0.01 * 1000.0 + 1e-12 or st["iterations"] == 100
    assert (sim.x > -0.1).all() and (sim.x < 2.1).all()
