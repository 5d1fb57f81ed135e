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
