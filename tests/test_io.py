"""Particle export (legacy VTK, like the reference's ParticleExporter_VTK; partio BGEO, like
ParticleExporter_Partio) and state files, all produced from the device copy.  A state file
restores a context exactly: the loaded context continues bit for bit."""
import gzip
import os
import re
import struct
import tempfile

import numpy as np
import pytest

from splishsplash_gb300 import native, scenes
from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

pytestmark = pytest.mark.gpu


def read_vtk(path):
    """Legacy VTK 4.1 binary unstructured grid of vertex cells, big-endian."""
    raw = open(path, "rb").read()
    pos = 0

    def line():
        nonlocal pos
        e = raw.index(b"\n", pos)
        s = raw[pos:e].decode()
        pos = e + 1
        return s

    def block(count, dtype):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a

    assert line() == "# vtk DataFile Version 4.1"
    line()
    assert line() == "BINARY"
    assert line() == "DATASET UNSTRUCTURED_GRID"
    m = re.match(r"POINTS (\d+) (float|double)", line())
    n, real = int(m.group(1)), (">f4" if m.group(2) == "float" else ">f8")
    out = {"position": block(3 * n, real).reshape(n, 3)}
    line()
    assert line() == f"CELLS {n} {2 * n}"
    cells = block(2 * n, ">u4").reshape(n, 2)
    assert (cells[:, 0] == 1).all() and (cells[:, 1] == np.arange(n)).all()
    line()
    assert line() == f"CELL_TYPES {n}"
    assert (block(n, ">i4") == 1).all()
    line()
    assert line() == f"POINT_DATA {n}"
    assert line() == "SCALARS id unsigned_int 1"
    assert line() == "LOOKUP_TABLE id_table"
    out["id"] = block(n, ">u4")
    line()
    k = int(re.match(r"FIELD FieldData (\d+)", line()).group(1))
    for _ in range(k):
        name, comps, cnt, typ = line().split()
        a = block(int(comps) * int(cnt), ">u4" if typ == "unsigned_int" else real)
        out[name] = a.reshape(int(cnt), int(comps)) if int(comps) > 1 else a
        line()
    assert pos == len(raw)
    return out


def read_bgeo(path):
    """partio's classic BGEO (version 5), plain or one gzip member: {name: array, "_types": ...}"""
    raw = open(path, "rb").read()
    compressed = raw[:2] == b"\x1f\x8b"
    if compressed:
        raw = gzip.decompress(raw)      # checks the member's CRC-32 and length
    magic, vc, version = struct.unpack_from(">icI", raw, 0)
    assert magic == 0x4267656F and vc == b"V" and version == 5
    n, nprim, npg, nprg, npa, nva, nra, nda = struct.unpack_from(">8I", raw, 9)
    assert (nprim, npg, nprg, nva, nra, nda) == (0, 0, 0, 0, 0, 0)
    pos = 9 + 32
    attrs = []
    for _ in range(npa):
        (ln,) = struct.unpack_from(">H", raw, pos)
        name = raw[pos + 2:pos + 2 + ln].decode()
        pos += 2 + ln
        size, typ = struct.unpack_from(">Hi", raw, pos)
        pos += 6
        assert struct.unpack_from(f">{size}i", raw, pos) == (0,) * size     # defaults
        pos += 4 * size
        attrs.append((name, size, typ))
    words = 4 + sum(a[1] for a in attrs)
    rec = np.frombuffer(raw, dtype=">u4", count=n * words, offset=pos).reshape(n, words)
    pos += rec.nbytes
    assert raw[pos:] == b"\x00\xff"
    out = {"_types": {a[0]: (a[1], a[2]) for a in attrs}, "_compressed": compressed}
    out["position"] = rec[:, :3].view(">f4").astype(np.float32)
    assert (rec[:, 3].view(">f4") == 1.0).all()
    col = 4
    for name, size, typ in attrs:
        a = rec[:, col:col + size]
        a = a.view(">i4").astype(np.int64) if typ == 1 else a.view(">f4").astype(np.float32)
        out[name] = a if size > 1 else a[:, 0]
        col += size
    return out


BGEO_FIELDS = ("density", "velocity", "p / rho^2", "fluid neighbors")


def check_bgeo(b, ref, n):
    assert b["_types"] == {"id": (1, 1), "density": (1, 0), "velocity": (3, 5), "p / rho^2": (1, 0),
                           "fluid neighbors": (1, 1)}
    np.testing.assert_array_equal(b["id"], np.arange(n))
    for f in ("position",) + BGEO_FIELDS:
        np.testing.assert_array_equal(b[f], ref[f])


def bgeo_reference(ts):
    m = ts.getFluidModel()
    ref = {f: m.getFieldBuffer(f, np.float32) for f in ("position", "density", "velocity", "p / rho^2")}
    ref["fluid neighbors"] = ts.ctx.download("fluid neighbors").astype(np.int64)
    return ref


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bgeo_export_matches_downloads(precision):
    """plain and compressed, waited and overlapping a step; FP64 values are stored as floats"""
    sc = scenes.small_block(counts=(10, 10, 10), box=(0.8, 0.8, 0.8), velocity=(0.2, 0.0, 0.0))
    ts = TimeStepDFSPH(sc, precision=precision)
    for _ in range(5):
        ts.step()
    ref = bgeo_reference(ts)
    with tempfile.TemporaryDirectory() as d:
        paths = [os.path.join(d, f"ParticleData_Fluid_{k}.bgeo") for k in range(3)]
        ts.ctx.export_bgeo(paths[0], BGEO_FIELDS, level=-1)
        ts.ctx.export_bgeo(paths[1], BGEO_FIELDS, level=0)
        ts.ctx.export_bgeo(paths[2], BGEO_FIELDS, level=6, wait=False)   # overlaps the next step
        ts.step()
        ts.ctx.export_wait()
        for p, comp in zip(paths, (True, False, True)):
            b = read_bgeo(p)
            assert b["_compressed"] == comp
            check_bgeo(b, ref, sc.n)
        assert not np.array_equal(read_bgeo(paths[2])["position"], bgeo_reference(ts)["position"])
    ts.close()


def test_bgeo_export_of_many_pieces():
    """about 3.6 MB of records: several compression pieces joined into one gzip member; levels 1 and
    9 give the same content, and the file is smaller than the plain one"""
    sc = scenes.small_block(counts=(50, 40, 50), radius=0.01, box=(1.2, 1.0, 1.2), velocity=(0.1, 0.0, 0.2))
    ts = TimeStepDFSPH(sc)
    ts.step()
    ref = bgeo_reference(ts)
    with tempfile.TemporaryDirectory() as d:
        sizes = {}
        for level in (0, 1, 9):
            p = os.path.join(d, f"l{level}.bgeo")
            ts.ctx.export_bgeo(p, BGEO_FIELDS, level=level)
            check_bgeo(read_bgeo(p), ref, sc.n)
            sizes[level] = os.path.getsize(p)
        assert sizes[0] > 3_000_000 and sizes[9] <= sizes[1] < sizes[0]
    ts.close()


def test_bgeo_export_refusals():
    sc = scenes.small_block(counts=(4, 4, 4))
    ts = TimeStepDFSPH(sc)
    ts.step()
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "x.bgeo")
        for kwargs in (dict(level=10), dict(level=-2), dict(fields=("position",)), dict(fields=("id",))):
            with pytest.raises(native.SphgbError) as e:
                ts.ctx.export_bgeo(p, **kwargs)
            assert native.ERR_NAMES[e.value.code] == "ARGUMENT"
        with pytest.raises(native.SphgbError):
            ts.ctx.export_bgeo(os.path.join(d, "missing", "x.bgeo"))
    ts.close()


def test_vtk_export_matches_downloads_and_overlaps_a_step():
    sc = scenes.small_block(counts=(10, 10, 10), box=(0.8, 0.8, 0.8), velocity=(0.2, 0.0, 0.0))
    ts = TimeStepDFSPH(sc)
    for _ in range(5):
        ts.step()
    fields = ("density", "velocity", "p / rho^2", "fluid neighbors")
    m = ts.getFluidModel()
    ref = {f: m.getFieldBuffer(f, np.float32) for f in ("position", "density", "velocity", "p / rho^2")}
    ref["fluid neighbors"] = ts.ctx.download("fluid neighbors")
    with tempfile.TemporaryDirectory() as d:
        p1, p2 = os.path.join(d, "a.vtk"), os.path.join(d, "b.vtk")
        ts.ctx.export_vtk(p1, fields, wait=True)
        ts.ctx.export_vtk(p2, fields, wait=False)   # the copy and the write overlap the next step
        ts.step()
        ts.ctx.export_wait()
        for p in (p1, p2):
            v = read_vtk(p)
            np.testing.assert_array_equal(v["id"], np.arange(sc.n))
            np.testing.assert_array_equal(v["position"], ref["position"])
            np.testing.assert_array_equal(v["density"], ref["density"])
            np.testing.assert_array_equal(v["velocity"], ref["velocity"])
            np.testing.assert_array_equal(v["p_/_rho^2"], ref["p / rho^2"])
            np.testing.assert_array_equal(v["fluid_neighbors"], ref["fluid neighbors"])
        # the exported state is the one before the step
        assert not np.array_equal(read_vtk(p2)["position"], m.getFieldBuffer("position", np.float32))
    ts.close()


@pytest.mark.parametrize("viscosity", [False, True])
def test_state_file_restores_a_context_bit_for_bit(viscosity):
    sc = scenes.small_block(counts=(12, 12, 12), box=(0.8, 1.0, 0.8), viscosity=viscosity, velocity=(0.4, 0.0, 0.1))
    a = TimeStepDFSPH(sc)
    for _ in range(15):
        a.step()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "state.bin")
        a.ctx.save_state(path)
        sa = [a.step() for _ in range(10)]
        b = native.Context(use_graph=True)
        b.load_state(path)
        sb = [b.step() for _ in range(10)]
    for x, y in zip(sa, sb):
        for key in ("iterations", "iterations_v", "visco_iterations", "dt_used", "time", "avg_density_err"):
            assert x[key] == y[key], key
    for f in ("position", "velocity", "p / rho^2", "p_v / rho^2", "velocity difference", "density"):
        np.testing.assert_array_equal(a.ctx.download(f), b.download(f), err_msg=f)
    a.close()
    b.close()


def test_state_file_restores_a_batch():
    ens = scenes.ensemble(num_scenes=4, seed=11, n_min=2000, n_max=4000)
    a = BatchedTimeStepDFSPH(ens)
    for _ in range(8):
        a.step()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "state.bin")
        a.ctx.save_state(path)
        for _ in range(6):
            a.step()
        b = native.Context(use_graph=True)
        b.load_state(path)
        assert b.num_scenes() == 4
        for _ in range(6):
            b.step()
    assert [s["time"] for s in a.scene_stats()] == [s["time"] for s in b.scene_stats()]
    np.testing.assert_array_equal(a.ctx.download("position"), b.download("position"))
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batched_field_transfers_equal_single_ones(precision):
    """sphgb_download_fields / sphgb_upload_fields: the same values as one call per field, in
    float32 and float64 targets; an unknown or non-uploadable field is refused."""
    sc = scenes.small_block(counts=(9, 8, 7), viscosity=True, velocity=(0.2, 0.0, -0.1)).as_float32()
    ts = TimeStepDFSPH(sc, precision=precision)
    try:
        for _ in range(4):
            ts.step()
        ctx = ts.ctx
        names = ("position", "velocity", "density", "p / rho^2", "p_v / rho^2", "velocity difference")
        for dt in (np.float32, np.float64):
            single = {k: ctx.download(k, dtype=dt) for k in names}
            many = ctx.download_fields({k: np.zeros_like(v) for k, v in single.items()})
            for k in names:
                np.testing.assert_array_equal(many[k], single[k])
        rng = np.random.default_rng(5)
        new = {"velocity": rng.uniform(-1, 1, (sc.n, 3)).astype(np.float32),
               "p / rho^2": rng.uniform(0, 1e-4, sc.n).astype(np.float32)}
        ctx.upload_fields(new)
        for k, v in new.items():
            np.testing.assert_array_equal(ctx.download(k, dtype=np.float32), v)
        with pytest.raises(native.SphgbError):
            ctx.upload_fields({"density": np.zeros(sc.n, np.float32)})
    finally:
        ts.close()


@pytest.mark.parametrize("batch", [False, True])
def test_transfers_through_mapped_host_memory_match_staged_ones(batch):
    """Fields to and from page-locked host buffers and the context's device memory are written
    and read by the device directly, in particle-id order; the values equal those of the staged
    copies into pageable buffers, in float32 and float64, for one scene and for a batch of
    scenes, also for buffers off a 16-byte boundary."""
    torch = pytest.importorskip("torch")
    if batch:
        sc = [scenes.small_block(counts=(9, 8, 7), seed=1, velocity=(0.2, 0.0, -0.1)).as_float32(),
              scenes.small_block(counts=(6, 6, 6), seed=2, velocity=(-0.1, 0.3, 0.0)).as_float32()]
        ts = BatchedTimeStepDFSPH(sc)
    else:
        sc = scenes.small_block(counts=(9, 8, 7), viscosity=True, velocity=(0.2, 0.0, -0.1)).as_float32()
        ts = TimeStepDFSPH(sc)
    try:
        for _ in range(3):
            ts.step()
        ctx = ts.ctx
        n, _ = ctx.num_particles()
        names = ("position", "velocity", "density", "p / rho^2", "p_v / rho^2", "factor")
        shape = {k: (n, 3) if k in ("position", "velocity") else (n,) for k in names}
        pin = lambda shp, dt: torch.empty(shp, dtype=dt, pin_memory=True).numpy()
        # a buffer one element past a 16-byte boundary takes the 4-byte path of the same kernels
        off = lambda shp, dt: pin(int(np.prod(shp)) + 1, dt)[1:].reshape(shp)
        dev = lambda shp, dt: torch.empty(shp, dtype=dt, device="cuda")
        host = lambda a: a.cpu().numpy() if hasattr(a, "cpu") else a
        for dt, tdt in ((np.float32, torch.float32), (np.float64, torch.float64)):
            staged = ctx.download_fields({k: np.zeros(shape[k], dt) for k in names})
            for make in (pin, off, dev):
                direct = ctx.download_fields({k: make(shape[k], tdt) for k in names})
                for k in names:
                    np.testing.assert_array_equal(host(direct[k]), staged[k], err_msg=k)
        rng = np.random.default_rng(11)
        v = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
        kap = rng.uniform(0, 1e-4, n).astype(np.float32)
        for make in (pin, off, dev):
            vp, kp = make((n, 3), torch.float32), make((n,), torch.float32)
            vp[:] = torch.from_numpy(v) if make is dev else v
            kp[:] = torch.from_numpy(kap) if make is dev else kap
            torch.cuda.synchronize()   # device buffers are read on the context's stream
            ctx.upload_fields({"velocity": vp, "p / rho^2": kp})
            np.testing.assert_array_equal(ctx.download("velocity", dtype=np.float32), v)
            np.testing.assert_array_equal(ctx.download("p / rho^2", dtype=np.float32), kap)
            v, kap = v[::-1].copy(), kap[::-1].copy()
    finally:
        ts.close()
