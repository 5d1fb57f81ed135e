"""sphgb_boundary_volume_noalloc: the allocation-free boundary-volume entry point.

Callers that cannot allocate device memory (work recorded during CUDA stream
capture, hosts with a fixed device-memory budget) pass their own device input and
output buffers; the scratch is a static device array inside the library.  This
test calls the entry point through the C ABI twice in a row with different scenes (the
second call reuses scratch left by the first) and checks both results against the volumes of
the allocating path (sphgb_upload_boundary + sphgb_download), to the FP32 volume
tolerance used elsewhere (1e-6 relative).  The file name makes pytest collect it
last.
"""
import ctypes

import numpy as np
import pytest

from splishsplash_gb300 import native, scenes

pytestmark = pytest.mark.gpu


def _volumes_allocating(sc):
    ctx = native.Context()
    ctx.set_params(sc.params)
    ctx.upload_boundary(sc.xb)
    ctx.upload_fluid(sc.x, sc.v)
    vb = ctx.download("boundary volume")
    ctx.close()
    return vb


def test_noalloc_boundary_volume_matches_allocating_path_twice():
    """Two calls in a row with different data: a larger box first, then a smaller, shifted one, so
    that cell ranges or particle entries left in the scratch by the first call would show up."""
    import torch

    L = native.load()
    f = L.sphgb_boundary_volume_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                  ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int

    first = scenes.dambreak_8k().as_float32()
    second = scenes.small_block(counts=(6, 6, 6), box=(0.7, 0.5, 0.6)).as_float32()
    shift = np.array([0.31, 0.12, 0.23])
    second.xb = (second.xb + shift).astype(np.float32).astype(np.float64)
    second.x = (second.x + shift).astype(np.float32).astype(np.float64)
    stream = torch.cuda.current_stream()
    for sc in (first, second):
        want = _volumes_allocating(sc)
        xb = torch.tensor(sc.xb, dtype=torch.float32, device="cuda").contiguous()
        lo = (ctypes.c_double * 3)(*np.min(sc.xb, 0).tolist())
        hi = (ctypes.c_double * 3)(*np.max(sc.xb, 0).tolist())
        out = torch.full((sc.nb,), -1.0, dtype=torch.float32, device="cuda")
        rc = f(xb.data_ptr(), sc.nb, sc.params.particleRadius, lo, hi, out.data_ptr(), stream.cuda_stream)
        assert rc == native.OK
        stream.synchronize()
        got = out.cpu().numpy().astype(np.float64)
        assert np.all(got > 0)
        np.testing.assert_allclose(got, want, rtol=1e-6, atol=0)


def test_noalloc_rejects_sizes_beyond_its_limits():
    import torch

    L = native.load()
    f = L.sphgb_boundary_volume_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                  ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    lo = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    hi = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    xb = torch.zeros((100, 3), dtype=torch.float32, device="cuda")
    out = torch.zeros((100,), dtype=torch.float32, device="cuda")
    # more particles than the static scratch holds: SPHGB_ERR_CAPACITY, nothing launched
    assert f(xb.data_ptr(), 65537, 0.025, lo, hi, out.data_ptr(), None) == 3
    # a box needing more cells than the scratch cell table: SPHGB_ERR_GRID, nothing launched
    big = (ctypes.c_double * 3)(100.0, 100.0, 100.0)
    assert f(xb.data_ptr(), 100, 0.025, lo, big, out.data_ptr(), None) == 6
    # an extent beyond any grid, or not finite: rejected before any cell count is formed
    huge = (ctypes.c_double * 3)(1e300, 1.0, 1.0)
    assert f(xb.data_ptr(), 100, 0.025, lo, huge, out.data_ptr(), None) == 6
    inf = (ctypes.c_double * 3)(float("inf"), 1.0, 1.0)
    assert f(xb.data_ptr(), 100, 0.025, lo, inf, out.data_ptr(), None) == 1
    assert f(xb.data_ptr(), 100, 1e-300, lo, hi, out.data_ptr(), None) == 6
