"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs to
check (or time beside) the CUDA path.  Nothing in the product package imports
this module.  See sph_oracle.h for the pinning status of the restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


def build(quiet: bool = True) -> None:
    """Compile liboracle_f64.so / liboracle_f32.so with the committed Makefile."""
    out = subprocess.run(["make", "-C", HERE, "-s"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("radius", ctypes.c_double),
        ("density0", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("cfl_method", ctypes.c_int),
        ("cfl_factor", ctypes.c_double),
        ("cfl_min", ctypes.c_double),
        ("cfl_max", ctypes.c_double),
        ("min_iterations", ctypes.c_uint),
        ("max_iterations", ctypes.c_uint),
        ("max_error", ctypes.c_double),
        ("enable_divergence_solver", ctypes.c_int),
        ("max_iterations_v", ctypes.c_uint),
        ("max_error_v", ctypes.c_double),
        ("xsph_fluid", ctypes.c_double),
        ("xsph_boundary", ctypes.c_double),
        ("viscosity_method", ctypes.c_int),
        ("viscosity", ctypes.c_double),
        ("viscosity_boundary", ctypes.c_double),
        ("visco_max_iter", ctypes.c_uint),
        ("visco_max_error", ctypes.c_double),
        ("fp32_predicate", ctypes.c_int),
        ("num_threads", ctypes.c_int),
        ("boundary_method", ctypes.c_int),
    ]


class OrcVmap(ctypes.Structure):
    _fields_ = [
        ("dmin", ctypes.c_double * 3),
        ("dmax", ctypes.c_double * 3),
        ("res", ctypes.c_uint * 3),
        ("field", ctypes.c_void_p * 2),
        ("R", ctypes.c_double * 9),
        ("t", ctypes.c_double * 3),
        ("v", ctypes.c_double * 3),
        ("w", ctypes.c_double * 3),
        ("max_dist", ctypes.c_double),
    ]


class OrcState(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint),
        ("nb", ctypes.c_uint),
        ("x", ctypes.c_void_p),
        ("v", ctypes.c_void_p),
        ("a", ctypes.c_void_p),
        ("density", ctypes.c_void_p),
        ("factor", ctypes.c_void_p),
        ("density_adv", ctypes.c_void_p),
        ("kappa", ctypes.c_void_p),
        ("kappa_v", ctypes.c_void_p),
        ("pressure_accel", ctypes.c_void_p),
        ("vdiff", ctypes.c_void_p),
        ("xb", ctypes.c_void_p),
        ("Vb", ctypes.c_void_p),
        ("dt", ctypes.c_double),
        ("time", ctypes.c_double),
        ("iterations", ctypes.c_uint),
        ("iterations_v", ctypes.c_uint),
        ("visco_iterations", ctypes.c_uint),
        ("avg_density_err", ctypes.c_double),
        ("avg_density_err_v", ctypes.c_double),
        ("visco_error", ctypes.c_double),
        ("dt_old", ctypes.c_double),
        ("factor_raw", ctypes.c_void_p),
        ("density_adv_v", ctypes.c_void_p),
        ("num_fluid_neighbors", ctypes.c_void_p),
        ("num_boundary_neighbors", ctypes.c_void_p),
        ("body", ctypes.c_void_p),
        ("nbodies", ctypes.c_uint),
        ("body_center", ctypes.c_void_p),
        ("body_dynamic", ctypes.c_void_p),
        ("body_force", ctypes.c_void_p),
        ("body_torque", ctypes.c_void_p),
        ("vmaps", ctypes.c_void_p),
        ("nvmaps", ctypes.c_uint),
        ("vb", ctypes.c_void_p),
        ("nphase", ctypes.c_uint),
        ("phase_count", ctypes.c_void_p),
        ("phase_density0", ctypes.c_void_p),
        ("phase_viscosity", ctypes.c_void_p),
        ("phase_viscosity_boundary", ctypes.c_void_p),
        ("phase_xsph", ctypes.c_void_p),
        ("phase_xsph_boundary", ctypes.c_void_p),
    ]


_LIBS = {}


def lib(precision: str = "f64") -> ctypes.CDLL:
    if precision not in _LIBS:
        path = os.path.join(BUILD, f"liboracle_{precision}.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_step.argtypes = [ctypes.POINTER(OrcState), ctypes.POINTER(OrcParams)]
        L.orc_step.restype = ctypes.c_int
        L.orc_kernel_W.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_kernel_W.restype = ctypes.c_double
        L.orc_kernel_gradW.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.orc_kernel_gradW.restype = None
        L.orc_neighbors.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_uint]
        L.orc_neighbors.restype = ctypes.c_int
        L.orc_boundary_volume.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_void_p]
        L.orc_boundary_volume.restype = ctypes.c_int
        for name in ("orc_weiler_system",):
            f = getattr(L, name)
            f.argtypes = [ctypes.POINTER(OrcState), ctypes.POINTER(OrcParams), ctypes.c_double,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            f.restype = ctypes.c_int
        L.orc_weiler_matvec.argtypes = [ctypes.POINTER(OrcState), ctypes.POINTER(OrcParams), ctypes.c_double,
                                        ctypes.c_void_p, ctypes.c_void_p]
        L.orc_weiler_matvec.restype = ctypes.c_int
        L.orc_weiler_solve.argtypes = [ctypes.POINTER(OrcState), ctypes.POINTER(OrcParams), ctypes.c_double,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint),
                                       ctypes.POINTER(ctypes.c_double)]
        L.orc_weiler_solve.restype = ctypes.c_int
        L.orc_vmap_nodes.argtypes = [ctypes.c_void_p]
        L.orc_vmap_nodes.restype = ctypes.c_size_t
        L.orc_vmap_node_position.argtypes = [ctypes.POINTER(OrcVmap), ctypes.c_size_t, ctypes.c_void_p]
        L.orc_vmap_node_position.restype = None
        L.orc_vmap_interpolate.argtypes = [ctypes.POINTER(OrcVmap), ctypes.c_int, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
        L.orc_vmap_interpolate.restype = ctypes.c_int
        L.orc_vmap_build.argtypes = [ctypes.POINTER(OrcVmap), ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p,
                                     ctypes.c_uint, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_uint]
        L.orc_vmap_build.restype = ctypes.c_int
        _LIBS[precision] = L
    return _LIBS[precision]


def make_params(p, fp32_predicate: bool = True, num_threads: int = 0) -> OrcParams:
    """Convert an SPHParams (splishsplash_gb300.scenes) into the oracle's struct."""
    q = OrcParams()
    q.radius = p.particleRadius
    q.density0 = p.density0
    q.gravity = (ctypes.c_double * 3)(*p.gravitation)
    q.cfl_method = p.cflMethod
    q.cfl_factor = p.cflFactor
    q.cfl_min = p.cflMinTimeStepSize
    q.cfl_max = p.cflMaxTimeStepSize
    q.min_iterations = p.minIterations
    q.max_iterations = p.maxIterations
    q.max_error = p.maxError
    q.enable_divergence_solver = int(p.enableDivergenceSolver)
    q.max_iterations_v = p.maxIterationsV
    q.max_error_v = p.maxErrorV
    q.xsph_fluid = p.xsph
    q.xsph_boundary = p.xsphBoundary
    q.viscosity_method = p.viscosityMethod
    q.viscosity = p.viscosity
    q.viscosity_boundary = p.viscosityBoundary
    q.visco_max_iter = p.viscoMaxIter
    q.visco_max_error = p.viscoMaxError
    q.fp32_predicate = int(fp32_predicate)
    q.num_threads = num_threads
    return q


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class VolumeMap:
    """A Bender2019 volume map of one static body (oracle/vmap.c): signed distance and volume
    on the cubic serendipity grid, built from a triangle mesh or given node values."""

    def __init__(self, res, dmin=None, dmax=None, rotation=None, translation=None):
        self.L = lib("f64")
        self.m = OrcVmap()
        self.m.res = (ctypes.c_uint * 3)(*[int(r) for r in res])
        self.nodes = int(self.L.orc_vmap_nodes(_ptr(np.array(res, np.uint32))))
        self.fields = [np.zeros(self.nodes, np.float64), np.zeros(self.nodes, np.float64)]
        self.m.field = (ctypes.c_void_p * 2)(_ptr(self.fields[0]).value, _ptr(self.fields[1]).value)
        if dmin is not None:
            self.m.dmin = (ctypes.c_double * 3)(*dmin)
            self.m.dmax = (ctypes.c_double * 3)(*dmax)
        R = np.eye(3) if rotation is None else np.asarray(rotation, np.float64)
        self.m.R = (ctypes.c_double * 9)(*R.ravel())
        self.m.t = (ctypes.c_double * 3)(*(np.zeros(3) if translation is None else translation))

    def build(self, vertices, faces, support, thickness=0.0, invert=False, order=30):
        v = np.ascontiguousarray(vertices, np.float64)
        f = np.ascontiguousarray(faces, np.uint32)
        rc = self.L.orc_vmap_build(ctypes.byref(self.m), _ptr(v), v.shape[0], _ptr(f), f.shape[0], support,
                                   thickness, int(invert), order)
        if rc != 0:
            raise RuntimeError(f"orc_vmap_build failed: {rc}")
        return self

    def set_values(self, dmin, dmax, sdf, volume):
        self.m.dmin = (ctypes.c_double * 3)(*dmin)
        self.m.dmax = (ctypes.c_double * 3)(*dmax)
        self.fields[0][:] = sdf
        self.fields[1][:] = volume
        return self

    def node_positions(self):
        out = np.zeros((self.nodes, 3))
        p = np.zeros(3)
        for k in range(self.nodes):
            self.L.orc_vmap_node_position(ctypes.byref(self.m), k, _ptr(p))
            out[k] = p
        return out

    def interpolate(self, field, x):
        """(value, gradient) at body-local point x, or None outside the grid."""
        x = np.ascontiguousarray(x, np.float64)
        v = ctypes.c_double()
        g = np.zeros(3)
        ok = self.L.orc_vmap_interpolate(ctypes.byref(self.m), int(field), _ptr(x), ctypes.byref(v), _ptr(g))
        return (v.value, g) if ok else None


class OracleSim:
    """A scene advanced by the oracle; arrays live in numpy (AoS, n x 3)."""

    def __init__(self, scene, precision: str = "f64", fp32_predicate: bool = True, num_threads: int = 0):
        self.precision = precision
        dt = np.float64 if precision == "f64" else np.float32
        self.dtype = dt
        self.lib = lib(precision)
        self.params = scene.params
        self.cp = make_params(scene.params, fp32_predicate, num_threads)
        n, nb = scene.n, scene.nb
        self.n, self.nb = n, nb
        # own copies: stepping must not write into the scene's arrays
        self.x = np.array(scene.x, dtype=dt, order="C", copy=True)
        self.v = np.array(scene.v, dtype=dt, order="C", copy=True)
        self.a = np.zeros((n, 3), dt)
        self.density = np.zeros(n, dt)
        self.factor = np.zeros(n, dt)
        self.density_adv = np.zeros(n, dt)
        self.kappa = np.zeros(n, dt)
        self.kappa_v = np.zeros(n, dt)
        self.pressure_accel = np.zeros((n, 3), dt)
        self.vdiff = np.zeros((n, 3), dt)
        self.xb = np.array(scene.xb, dtype=dt, order="C", copy=True)
        self.Vb = np.zeros(nb, dt)
        self.factor_raw = np.zeros(n, dt)
        self.density_adv_v = np.zeros(n, dt)
        self.nf = np.zeros(n, np.uint32)
        self.nbn = np.zeros(n, np.uint32)
        self._support, self._fp32_predicate = scene.params.supportRadius, int(fp32_predicate)
        rc = self.lib.orc_boundary_volume(nb, _ptr(self.xb), scene.params.supportRadius,
                                          int(fp32_predicate), _ptr(self.Vb))
        if rc != 0:
            raise RuntimeError(f"orc_boundary_volume failed: {rc}")
        self.st = OrcState()
        self.st.n, self.st.nb = n, nb
        for name in ("x", "v", "a", "density", "factor", "density_adv", "kappa", "kappa_v",
                     "pressure_accel", "vdiff", "xb", "Vb", "factor_raw", "density_adv_v"):
            setattr(self.st, name, _ptr(getattr(self, name)))
        self.st.num_fluid_neighbors = _ptr(self.nf)
        self.st.num_boundary_neighbors = _ptr(self.nbn)
        self.st.dt = scene.params.timeStepSize
        self.st.time = 0.0

    def set_bodies(self, body, center, dynamic=None):
        """Bodies of the boundary particles (upload order), reference points and dynamic flags;
        forces accumulate in body_force / body_torque until clear_forces()."""
        self.body = None if body is None else np.ascontiguousarray(body, np.uint32)   # None: map b is body b
        self.body_center = np.ascontiguousarray(center, np.float64).reshape(-1, 3)
        nbodies = self.body_center.shape[0]
        self.body_dynamic = np.ones(nbodies, np.int32) if dynamic is None else np.ascontiguousarray(dynamic, np.int32)
        self.body_force = np.zeros((nbodies, 3), np.float64)
        self.body_torque = np.zeros((nbodies, 3), np.float64)
        self.st.body = _ptr(self.body)
        self.st.nbodies = nbodies
        self.st.body_center = _ptr(self.body_center)
        self.st.body_dynamic = _ptr(self.body_dynamic)
        self.st.body_force = _ptr(self.body_force)
        self.st.body_torque = _ptr(self.body_torque)

    def set_volume_maps(self, maps):
        """Bender2019 boundary: the bodies' VolumeMaps replace the boundary particles."""
        self._vmaps = list(maps)
        self._vmap_arr = (OrcVmap * max(1, len(self._vmaps)))(*[m.m for m in self._vmaps])
        self.st.vmaps = ctypes.cast(self._vmap_arr, ctypes.c_void_p)
        self.st.nvmaps = len(self._vmaps)
        self.cp.boundary_method = 2

    def set_map_motion(self, b, rotation=None, translation=None, velocity=(0, 0, 0), omega=(0, 0, 0), max_dist=None):
        """pose and velocity of the body of volume map b for the next steps; a body's force center
        follows its position; max_dist: the body's CFL radius (mesh vertices from their mean)"""
        m = self._vmap_arr[b]
        if max_dist is not None:
            m.max_dist = float(max_dist)
        if rotation is not None:
            m.R = (ctypes.c_double * 9)(*np.asarray(rotation, np.float64).ravel())
        if translation is not None:
            m.t = (ctypes.c_double * 3)(*np.asarray(translation, np.float64))
            if getattr(self, "body_center", None) is not None and b < len(self.body_center):
                self.body_center[b] = translation
        m.v = (ctypes.c_double * 3)(*np.asarray(velocity, np.float64))
        m.w = (ctypes.c_double * 3)(*np.asarray(omega, np.float64))

    def set_phases(self, counts, density0):
        """several fluid models: the particles in index order form len(counts) phases with the given
        rest densities"""
        self._phase_count = np.ascontiguousarray(counts, np.uint32)
        self._phase_density0 = np.ascontiguousarray(density0, np.float64)
        self.st.nphase = len(self._phase_count)
        self.st.phase_count = _ptr(self._phase_count)
        self.st.phase_density0 = _ptr(self._phase_density0)

    def set_phase_viscosity(self, viscosity, viscosity_boundary):
        """Weiler2018 nu and nu_b of each fluid model"""
        self._phase_nu = np.ascontiguousarray(viscosity, np.float64)
        self._phase_nub = np.ascontiguousarray(viscosity_boundary, np.float64)
        self.st.phase_viscosity = _ptr(self._phase_nu)
        self.st.phase_viscosity_boundary = _ptr(self._phase_nub)

    def set_phase_xsph(self, xsph, xsph_boundary):
        """XSPH fluid and boundary coefficients of each fluid model"""
        self._phase_xs = np.ascontiguousarray(xsph, np.float64)
        self._phase_xsb = np.ascontiguousarray(xsph_boundary, np.float64)
        self.st.phase_xsph = _ptr(self._phase_xs)
        self.st.phase_xsph_boundary = _ptr(self._phase_xsb)

    def set_boundary_state(self, xb, vb):
        """positions and velocities of the boundary particles for the next steps (moving
        Akinci2012 bodies; the volumes stay those of the initial shape, as for a rigid body)"""
        self.xb[:] = xb
        self.vb = np.array(vb, dtype=self.xb.dtype, order="C", copy=True).reshape(self.xb.shape)
        self.st.vb = _ptr(self.vb)

    def clear_forces(self):
        self.body_force[:] = 0.0
        self.body_torque[:] = 0.0

    def step(self):
        rc = self.lib.orc_step(ctypes.byref(self.st), ctypes.byref(self.cp))
        if rc != 0:
            raise RuntimeError(f"orc_step failed: {rc}")

    @property
    def dt(self):
        return self.st.dt

    @dt.setter
    def dt(self, value):
        self.st.dt = value

    def stats(self):
        s = self.st
        return dict(iterations=s.iterations, iterations_v=s.iterations_v, visco_iterations=s.visco_iterations,
                    avg_density_err=s.avg_density_err, avg_density_err_v=s.avg_density_err_v,
                    visco_error=s.visco_error, dt_old=s.dt_old, dt=s.dt, time=s.time)


def neighbors(x, y, support, same_set, fp32=True, precision="f64"):
    """CSR neighbour lists (offsets, indices) of points x against y."""
    L = lib(precision)
    dt = np.float64 if precision == "f64" else np.float32
    x = np.ascontiguousarray(x, dtype=dt)
    y = np.ascontiguousarray(y, dtype=dt)
    n, m = x.shape[0], y.shape[0]
    off = np.zeros(n + 1, np.uint32)
    rc = L.orc_neighbors(n, _ptr(x), m, _ptr(y), support, int(same_set), int(fp32), _ptr(off), None, 0)
    if rc != 0:
        raise RuntimeError(f"orc_neighbors failed: {rc}")
    idx = np.zeros(max(1, int(off[-1])), np.uint32)
    rc = L.orc_neighbors(n, _ptr(x), m, _ptr(y), support, int(same_set), int(fp32), _ptr(off), _ptr(idx),
                         idx.size)
    if rc != 0:
        raise RuntimeError(f"orc_neighbors failed: {rc}")
    return off, idx[: int(off[-1])]


def kernel_W(r, support):
    return lib().orc_kernel_W(float(r), float(support))


def kernel_gradW(r, support):
    r = np.ascontiguousarray(r, dtype=np.float64)
    out = np.zeros(3, np.float64)
    lib().orc_kernel_gradW(_ptr(r), float(support), _ptr(out))
    return out
