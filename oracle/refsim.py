"""Test infrastructure: the reference's own DFSPH step, loaded from oracle/_ref.

`oracle/build_ref.sh` compiles the reference's SPlisHSPlasH sources (against the
stand-ins in `oracle/shims/`) with `oracle/ref_driver.cpp` into
`oracle/_ref/libref_f64.so` (FP64, scalar paths) and, on x86-64,
`oracle/_ref/libref_f32.so` (FP32 AVX with precomputeValues).  `RefSim` sets a scene
up and steps it through the reference's `TimeStep::step()`; fields come back in
particle-id order.  The reference's `Simulation` is a process-wide singleton, so only
one RefSim may be alive per process at a time.

Only tests/, the golden-fixture script and bench.py's CPU legs use this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

FIELDS = {"position": (0, 3), "velocity": (1, 3), "density": (2, 1), "acceleration": (3, 3), "factor": (4, 1),
          "advected density": (5, 1), "p / rho^2": (6, 1), "p_v / rho^2": (7, 1), "pressure acceleration": (8, 3),
          "velocity difference": (9, 3)}


class RefParams(ctypes.Structure):
    _fields_ = [("particleRadius", ctypes.c_double), ("density0", ctypes.c_double),
                ("gravitation", ctypes.c_double * 3), ("timeStepSize", ctypes.c_double),
                ("cflMethod", ctypes.c_int), ("cflFactor", ctypes.c_double), ("cflMinTimeStepSize", ctypes.c_double),
                ("cflMaxTimeStepSize", ctypes.c_double), ("minIterations", ctypes.c_int),
                ("maxIterations", ctypes.c_int), ("maxError", ctypes.c_double),
                ("enableDivergenceSolver", ctypes.c_int), ("maxIterationsV", ctypes.c_int),
                ("maxErrorV", ctypes.c_double), ("xsph", ctypes.c_double), ("xsphBoundary", ctypes.c_double),
                ("viscosityMethod", ctypes.c_int), ("viscosity", ctypes.c_double),
                ("viscosityBoundary", ctypes.c_double), ("viscoMaxIter", ctypes.c_int),
                ("viscoMaxError", ctypes.c_double), ("analyticKernel", ctypes.c_int), ("numThreads", ctypes.c_int),
                ("boundaryMethod", ctypes.c_int)]


class RefStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint), ("iterationsV", ctypes.c_uint), ("viscoIterations", ctypes.c_uint),
                ("pad", ctypes.c_uint), ("dtOld", ctypes.c_double), ("dt", ctypes.c_double),
                ("time", ctypes.c_double), ("stepSeconds", ctypes.c_double)]


_LIBS = {}


def available(precision: str = "f64") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_{precision}.so"))


def lib(precision: str = "f64", path: str = None) -> ctypes.CDLL:
    """The reference build of the given precision, or the library at `path` that links the
    same reference objects and driver (tests of the reference-side plugin)."""
    key = path or precision
    if key not in _LIBS:
        path = path or os.path.join(REF_DIR, f"libref_{precision}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing: run oracle/build_ref.sh where the reference tree is present")
        L = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        dp = ctypes.POINTER(ctypes.c_double)
        L.ref_create.argtypes = [ctypes.POINTER(RefParams), ctypes.c_uint, dp, dp, ctypes.c_uint, dp]
        L.ref_create.restype = ctypes.c_int
        L.ref_step.argtypes = [ctypes.POINTER(RefStats)]
        L.ref_step.restype = ctypes.c_int
        L.ref_get.argtypes = [ctypes.c_int, dp]
        L.ref_get.restype = ctypes.c_int
        L.ref_set.argtypes = [ctypes.c_int, dp]
        L.ref_set.restype = ctypes.c_int
        L.ref_boundary_volume.argtypes = [dp]
        L.ref_neighbor_counts.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint)]
        L.ref_set_time_step.argtypes = [ctypes.c_double]
        L.ref_set_time_step.restype = None
        L.ref_precision.restype = ctypes.c_int
        L.ref_timing.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint)]
        L.ref_timing.restype = ctypes.c_int
        L.ref_destroy.restype = None
        up = ctypes.POINTER(ctypes.c_uint)
        L.ref_add_volume_map.argtypes = [dp, dp, up, dp, dp, dp, dp]
        L.ref_add_volume_map.restype = ctypes.c_int
        L.ref_clear_volume_maps.restype = None
        L.ref_set_phases.argtypes = [ctypes.c_uint, up, dp, dp, dp, dp, dp]
        L.ref_set_phases.restype = ctypes.c_int
        L.ref_set_bodies.argtypes = [ctypes.c_uint, ctypes.c_uint, up, dp, ctypes.POINTER(ctypes.c_int)]
        L.ref_set_bodies.restype = ctypes.c_int
        L.ref_body_forces.argtypes = [dp, dp]
        L.ref_body_forces.restype = ctypes.c_int
        L.ref_clear_body_forces.restype = None
        L.ref_set_body_motion.argtypes = [ctypes.c_uint, dp, dp, dp, dp]
        L.ref_set_body_motion.restype = ctypes.c_int
        L.ref_set_map_motion.argtypes = [ctypes.c_uint, dp, dp, dp, dp, ctypes.c_double]
        L.ref_set_map_motion.restype = ctypes.c_int
        _LIBS[key] = L
    return _LIBS[key]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class RefSim:
    """One scene stepped by the reference.  analytic_kernel=True selects the analytic
    cubic spline after the parameters are read (the FP64 oracle protocol); False keeps
    the reference's default PrecomputedKernel<CubicKernel, 10000> for DFSPH.
    volume_maps: oracle.VolumeMap objects (static bodies): the boundary is then Bender2019
    with those maps instead of the scene's boundary particles.
    phases: dict(counts=..., density0=..., and optionally viscosity, viscosity_boundary, xsph,
    xsph_boundary per model): the particles in id order form that many fluid models.
    bodies: dict(body=..., center=..., dynamic=...): the boundary particles split into one
    Akinci2012 body each (body index per particle, reference points, dynamic flags); the forces on
    the dynamic ones accumulate (body_forces / clear_body_forces)."""

    _alive = False

    def __init__(self, scene, precision: str = "f64", analytic_kernel: bool = True, num_threads: int = 0,
                 library: str = None, volume_maps=None, phases=None, bodies=None):
        if RefSim._alive:
            raise RuntimeError("the reference's Simulation is a singleton: close the other RefSim first")
        self.L = lib(precision, library)
        self.n, self.nb = scene.n, scene.nb
        p = scene.params
        rp = RefParams()
        rp.particleRadius = p.particleRadius
        rp.density0 = p.density0
        rp.gravitation = (ctypes.c_double * 3)(*p.gravitation)
        rp.timeStepSize = p.timeStepSize
        rp.cflMethod = p.cflMethod
        rp.cflFactor = p.cflFactor
        rp.cflMinTimeStepSize = p.cflMinTimeStepSize
        rp.cflMaxTimeStepSize = p.cflMaxTimeStepSize
        rp.minIterations = p.minIterations
        rp.maxIterations = p.maxIterations
        rp.maxError = p.maxError
        rp.enableDivergenceSolver = int(p.enableDivergenceSolver)
        rp.maxIterationsV = p.maxIterationsV
        rp.maxErrorV = p.maxErrorV
        rp.xsph = p.xsph
        rp.xsphBoundary = p.xsphBoundary
        rp.viscosityMethod = p.viscosityMethod
        rp.viscosity = p.viscosity
        rp.viscosityBoundary = p.viscosityBoundary
        rp.viscoMaxIter = p.viscoMaxIter
        rp.viscoMaxError = p.viscoMaxError
        rp.analyticKernel = int(analytic_kernel)
        rp.numThreads = num_threads
        self.L.ref_clear_volume_maps()
        for vm in volume_maps or ():
            c = vm.m   # the oracle's orc_vmap: domain, cells per axis, pose
            res = np.array(list(c.res), np.uint32)
            arr = lambda a: np.array(list(a), np.float64)
            self.L.ref_add_volume_map(_dp(arr(c.dmin)), _dp(arr(c.dmax)),
                                      res.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                                      _dp(np.ascontiguousarray(vm.fields[0], np.float64)),
                                      _dp(np.ascontiguousarray(vm.fields[1], np.float64)),
                                      _dp(arr(c.R)), _dp(arr(c.t)))
        rp.boundaryMethod = 2 if volume_maps else 0
        self._phase_arrays = []
        if phases:
            cnt = np.ascontiguousarray(phases["counts"], np.uint32)
            arrs = [np.ascontiguousarray(phases[k], np.float64) if phases.get(k) is not None else None
                    for k in ("density0", "viscosity", "viscosity_boundary", "xsph", "xsph_boundary")]
            self._phase_arrays = [cnt] + arrs
            self.L.ref_set_phases(len(cnt), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                                  *[(_dp(a) if a is not None else None) for a in arrs])
        else:
            self.L.ref_set_phases(0, None, None, None, None, None, None)
        self.nbodies = 0
        if bodies:
            self._body = np.ascontiguousarray(bodies["body"], np.uint32)
            self._center = np.ascontiguousarray(bodies["center"], np.float64).reshape(-1, 3)
            self._dyn = np.ascontiguousarray(bodies["dynamic"], np.int32)
            self.nbodies = self._center.shape[0]
            self.L.ref_set_bodies(self.nbodies, self._body.size,
                                  self._body.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), _dp(self._center),
                                  self._dyn.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        else:
            self.L.ref_set_bodies(0, 0, None, None, None)
        x = np.ascontiguousarray(scene.x, np.float64)
        v = np.ascontiguousarray(scene.v, np.float64)
        xb = np.ascontiguousarray(scene.xb, np.float64).reshape(-1, 3)
        if xb.size == 0:
            xb = np.zeros((1, 3))
        rc = self.L.ref_create(ctypes.byref(rp), self.n, _dp(x), _dp(v), self.nb, _dp(xb))
        if rc != 0:
            self.L.ref_destroy()
            raise RuntimeError(f"ref_create failed: {rc}")
        RefSim._alive = True
        self.last = RefStats()

    def step(self) -> dict:
        rc = self.L.ref_step(ctypes.byref(self.last))
        if rc != 0:
            raise RuntimeError(f"ref_step failed: {rc}")
        return self.stats()

    def stats(self) -> dict:
        s = self.last
        return dict(iterations=s.iterations, iterations_v=s.iterationsV, visco_iterations=s.viscoIterations,
                    dt_old=s.dtOld, dt=s.dt, time=s.time, step_seconds=s.stepSeconds)

    def get(self, name: str) -> np.ndarray:
        f, dim = FIELDS[name]
        out = np.zeros(self.n * dim, np.float64)
        if self.L.ref_get(f, _dp(out)) != dim:
            raise RuntimeError(f"ref_get({name}) failed")
        return out.reshape(self.n, dim) if dim == 3 else out

    def set(self, name: str, values) -> None:
        f, dim = FIELDS[name]
        a = np.ascontiguousarray(values, np.float64).reshape(-1)
        if a.size != self.n * dim or self.L.ref_set(f, _dp(a)) != dim:
            raise RuntimeError(f"ref_set({name}) failed")

    def boundary_volume(self) -> np.ndarray:
        out = np.zeros(max(1, self.nb), np.float64)
        self.L.ref_boundary_volume(_dp(out))
        return out[: self.nb]

    def body_forces(self):
        """(force, torque) per body since the last clear, nbodies x 3 each"""
        f = np.zeros((max(1, self.nbodies), 3))
        t = np.zeros((max(1, self.nbodies), 3))
        self.L.ref_body_forces(_dp(f), _dp(t))
        return f[: self.nbodies], t[: self.nbodies]

    def clear_body_forces(self) -> None:
        self.L.ref_clear_body_forces()

    def set_body_motion(self, b, rotation, translation, velocity, omega) -> None:
        """Pose and velocity of body b for the next step; its particles are placed as the
        simulator places them (x = R x0 + t, v = w x (x - t) + v)."""
        a = [np.ascontiguousarray(q, np.float64).reshape(-1) for q in (rotation, translation, velocity, omega)]
        if self.L.ref_set_body_motion(int(b), *[_dp(q) for q in a]) != 0:
            raise RuntimeError("ref_set_body_motion failed")

    def set_map_motion(self, b, rotation, translation, velocity, omega, max_dist=0.0) -> None:
        """Pose, velocity and CFL radius of the body of volume map b for the next step."""
        a = [np.ascontiguousarray(q, np.float64).reshape(-1) for q in (rotation, translation, velocity, omega)]
        if self.L.ref_set_map_motion(int(b), *[_dp(q) for q in a], float(max_dist)) != 0:
            raise RuntimeError("ref_set_map_motion failed")

    def neighbor_counts(self):
        nf = np.zeros(self.n, np.uint32)
        nb = np.zeros(self.n, np.uint32)
        self.L.ref_neighbor_counts(nf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                                   nb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)))
        return nf, nb

    def timing(self, name: str):
        """(total ms, count) of the reference's own timer `name` since the library loaded."""
        t, c = ctypes.c_double(), ctypes.c_uint()
        self.L.ref_timing(name.encode(), ctypes.byref(t), ctypes.byref(c))
        return t.value, c.value

    def set_time_step(self, dt: float) -> None:
        self.L.ref_set_time_step(float(dt))

    def close(self) -> None:
        if RefSim._alive:
            self.L.ref_destroy()
            RefSim._alive = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
