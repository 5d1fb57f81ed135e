"""In-tree build of libsphgb300.so (sm_103a) with nvcc.

Each .cu translation unit is compiled in parallel, then linked into
splishsplash_gb300/_lib/libsphgb300.so.  A rebuild happens only when a source
or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libsphgb300.so")
HOSTDIR = os.path.join(PKG, "host")
HOST_LIB = os.path.join(LIBDIR, "libsphgb300_host.so")      # C++ plugin-interface layer over the C ABI
HOST_DEMO = os.path.join(LIBDIR, "sphgb_host_demo")          # driver of the C++ layer (tests)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(HOSTDIR, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h")) + \
        [os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not all(os.path.exists(f) for f in (LIB, HOST_LIB, HOST_DEMO)):
        return False
    t = min(os.path.getmtime(f) for f in (LIB, HOST_LIB, HOST_DEMO))
    return all(os.path.getmtime(d) <= t for d in _deps())


def build_host(verbose: bool = False) -> None:
    """g++: the C++ host layer (libsphgb300_host.so) and its driver, linked to libsphgb300.so."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    inc = ["-I", os.path.join(ROOT, "include"), "-I", HOSTDIR]
    rpath = "-Wl,-rpath,$ORIGIN"
    cmds = [
        [cxx, "-std=c++17", "-O2", "-Wall", "-fPIC", "-shared", *inc, os.path.join(HOSTDIR, "sphgb_host.cpp"),
         "-L", LIBDIR, "-lsphgb300", rpath, "-o", HOST_LIB + ".tmp"],
        [cxx, "-std=c++17", "-O2", "-Wall", *inc, os.path.join(HOSTDIR, "sphgb_host_demo.cpp"), "-L", LIBDIR,
         "-lsphgb300_host", "-lsphgb300", rpath, "-o", HOST_DEMO + ".tmp"],
    ]
    for cmd, out in zip(cmds, (HOST_LIB, HOST_DEMO)):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host build failed:\n{r.stdout}{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        os.replace(out + ".tmp", out)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    build_host(verbose)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
