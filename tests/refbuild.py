"""Test infrastructure: libraries built from the reference tree for the tests that need it.

* `reference_tree()`: the reference's source tree (SPH_REFERENCE_ROOT, else a "reference"
  folder beside this repository), or None.
* `plugin_fake_abi()`: the reference's library objects (oracle/build_ref.sh) with the
  reference-side plugin (splishsplash_gb300/plugin/), tests/plugin/plugin_glue.cpp, the
  oracle-backed stand-in of the C ABI (tests/plugin/fake_sphgb300.cpp) and the state-file glue
  of `state_library()`.
* `plugin_objects()`: the plugin's object files, for a link check against libsphgb300.so.
* `state_library()`: the reference's library objects with oracle/ref_driver.cpp and partio
  (vendored in the reference tree, extern/partio) plus tests/plugin/partio_state.cpp: the
  reference's particle state files written and read through partio.
Everything is written under oracle/_ref/ and rebuilt only when missing.
"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_OUT = os.path.join(ROOT, "oracle", "_ref")
PLUGIN = os.path.join(ROOT, "splishsplash_gb300", "plugin")


def reference_tree():
    env = os.environ.get("SPH_REFERENCE_ROOT")
    p = env if env else os.path.join(ROOT, "..", "reference")
    return os.path.abspath(p) if os.path.isfile(os.path.join(p, "SPlisHSPlasH", "TimeStep.cpp")) else None


def run(cmd, env=None):
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout[-3000:] + r.stderr[-3000:])


def _ref_objects(tree):
    if not os.path.exists(os.path.join(REF_OUT, "libref_f64.so")):
        run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], env={**os.environ, "SPH_REFERENCE_ROOT": tree})
    d = os.path.join(REF_OUT, "obj_ref_f64")
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".o"))


def _includes(tree):
    return ["-include", "cfloat", "-include", "memory", "-I", os.path.join(ROOT, "oracle", "shims"), "-I", tree,
            "-I", os.path.join(tree, "extern", "eigen"), "-I", os.path.join(tree, "extern"),
            "-I", os.path.join(ROOT, "include"), "-I", PLUGIN, "-I", os.path.join(ROOT, "oracle"),
            "-I", os.path.join(tree, "extern", "partio", "src", "lib")]


CXX = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-DUSE_DOUBLE", "-w"]


def _compile(tree, out_dir, name, src):
    obj = os.path.join(out_dir, name + ".o")
    if not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src):
        run(CXX + _includes(tree) + ["-c", src, "-o", obj])
    return obj


def plugin_objects(tree):
    out = os.path.join(REF_OUT, "plugin_test")
    os.makedirs(out, exist_ok=True)
    return {"plugin": _compile(tree, out, "plugin", os.path.join(PLUGIN, "TimeStepDFSPH_GB300.cpp")),
            "glue": _compile(tree, out, "glue", os.path.join(ROOT, "tests", "plugin", "plugin_glue.cpp"))}


def plugin_fake_abi(tree):
    out = os.path.join(REF_OUT, "plugin_test")
    os.makedirs(out, exist_ok=True)
    lib = os.path.join(out, "libplugin_fake_abi.so")
    objs = plugin_objects(tree)
    objs["fake"] = _compile(tree, out, "fake", os.path.join(ROOT, "tests", "plugin", "fake_sphgb300.cpp"))
    objs["state"] = _compile(tree, out, "partio_state", os.path.join(ROOT, "tests", "plugin", "partio_state.cpp"))
    # the oracle behind the stand-in (FP64 sph_oracle.c and vmap.c) is part of the reference
    # objects already: oracle/build_ref.sh links it under the driver's volume-map grid
    run(["g++", "-shared", "-fopenmp", "-Wl,--no-undefined", "-o", lib, *_ref_objects(tree), *objs.values(),
         *_partio_objects(tree), "-lz", "-lm"])
    return lib


def link_plugin_against(tree, libdir):
    """Links the plugin with the reference's objects against libsphgb300.so in libdir."""
    out = os.path.join(REF_OUT, "plugin_test", "libplugin_gb300.so")
    objs = plugin_objects(tree)
    run(["g++", "-shared", "-fopenmp", "-Wl,--no-undefined", "-o", out, *_ref_objects(tree), objs["plugin"],
         objs["glue"], "-L", libdir, "-lsphgb300", "-lm"])
    return out


def _partio_objects(tree):
    """partio's library objects, compiled once into oracle/_ref/partio/"""
    out = os.path.join(REF_OUT, "partio")
    os.makedirs(out, exist_ok=True)
    objs = []
    pio = os.path.join(tree, "extern", "partio", "src", "lib")
    # partio predates C++17 (std::ios::streampos): compiled as C++11, as its own build does
    for sub in ("core", "io"):
        for f in sorted(os.listdir(os.path.join(pio, sub))):
            if f.endswith(".cpp"):
                obj = os.path.join(out, f"partio_{sub}_{f[:-4]}.o")
                if not os.path.exists(obj):
                    run(["g++", "-std=c++11", "-O2", "-fPIC", "-w", "-DPARTIO_USE_ZLIB", "-I", pio,
                         "-c", os.path.join(pio, sub, f), "-o", obj])
                objs.append(obj)
    return objs


def state_library(tree):
    out = os.path.join(REF_OUT, "state_test")
    os.makedirs(out, exist_ok=True)
    lib = os.path.join(out, "libref_state_f64.so")
    ref_objs = _ref_objects(tree)
    src = os.path.join(ROOT, "tests", "plugin", "partio_state.cpp")
    if os.path.exists(lib) and all(os.path.getmtime(f) <= os.path.getmtime(lib) for f in ref_objs + [src]):
        return lib
    objs = [_compile(tree, out, "partio_state", src)]
    run(["g++", "-shared", "-fopenmp", "-Wl,--no-undefined", "-o", lib, *ref_objs, *objs, *_partio_objects(tree),
         "-lz", "-lm"])
    return lib
