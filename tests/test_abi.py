"""The C-ABI library builds for sm_103a, loads, and exports every function that
include/sphgb300.h declares (no device calls: runs without a GPU)."""
import ctypes
import os
import re
import subprocess

from splishsplash_gb300 import build as b

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?[\w]+\s*\**\s*(sphgb_\w+)\s*\(", src, re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = b.build()
    assert os.path.exists(lib)
    names = declared_functions()
    assert "sphgb_step" in names and len(names) >= 20
    L = ctypes.CDLL(lib)
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (sphgb_\w+)", out))
    assert names <= exported


def test_library_is_built_for_sm_103a():
    assert "arch=compute_103a,code=sm_103a" in b.ARCH


def test_python_mirror_fails_loudly_without_gpu():
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from splishsplash_gb300 import native
    with pytest.raises(native.SphgbError):
        native.Context()


def test_field_ids_of_the_reference_field_names():
    """sphgb_field_id maps the reference's field names to the ids of the header (a host-only call)"""
    from splishsplash_gb300 import native
    L = ctypes.CDLL(b.build())
    L.sphgb_field_id.argtypes = [ctypes.c_char_p]
    L.sphgb_field_id.restype = ctypes.c_int
    for name, (fid, _) in native.FIELDS.items():
        if fid <= 18 and fid not in (14, 15):      # fluid fields; 14, 15 are boundary fields
            assert L.sphgb_field_id(name.encode()) == fid, name
    assert L.sphgb_field_id(b"velocity") == 1 and L.sphgb_field_id(b"p / rho^2") == 6
    assert L.sphgb_field_id(b"no such field") == -1 and L.sphgb_field_id(None) == -1
