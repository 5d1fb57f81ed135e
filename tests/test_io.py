"""Particle export (legacy VTK, like the reference's ParticleExporter_VTK) and state files,
both produced from the device copy.  A state file restores a context exactly: the loaded
context continues bit for bit."""
import os
import re
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
