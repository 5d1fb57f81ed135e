"""ctypes binding of libsphgb300.so (include/sphgb300.h).

There is no CPU fallback: if the library cannot be loaded, or no CUDA device is
visible, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

SPHGB_ABI_VERSION = 1
OK = 0
ERR_NAMES = {1: "ARGUMENT", 2: "CUDA", 3: "CAPACITY", 4: "NONFINITE", 5: "STATE", 6: "GRID"}

PRECISION_FP32 = 0
PRECISION_FP64 = 1

FIELDS = {
    "position": (0, 3),
    "velocity": (1, 3),
    "acceleration": (2, 3),
    "density": (3, 1),
    "factor": (4, 1),
    "advected density": (5, 1),
    "p / rho^2": (6, 1),
    "p_v / rho^2": (7, 1),
    "pressure acceleration": (8, 3),
    "velocity difference": (9, 3),
    "id": (10, 1),
    "factor raw": (11, 1),
    "fluid neighbors": (12, 1),
    "boundary neighbors": (13, 1),
    "boundary volume": (14, 1),
    "boundary position": (15, 3),
    "features": (16, 10),
    "position high": (17, 3),
    "position low": (18, 3),
    "state": (19, 1),
    "object_id": (20, 1),
}
DTYPE_F32, DTYPE_F64, DTYPE_U32 = 0, 1, 2


class SphgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sphgb error {code} ({ERR_NAMES.get(code, '?')}): {msg}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int),
        ("device", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("max_fluid_neighbors", ctypes.c_uint32),
        ("max_boundary_neighbors", ctypes.c_uint32),
        ("use_graph", ctypes.c_int),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("particle_radius", ctypes.c_double),
        ("density0", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("cfl_method", ctypes.c_int),
        ("cfl_factor", ctypes.c_double),
        ("cfl_min_time_step", ctypes.c_double),
        ("cfl_max_time_step", ctypes.c_double),
        ("min_iterations", ctypes.c_uint32),
        ("max_iterations", ctypes.c_uint32),
        ("max_error", ctypes.c_double),
        ("enable_divergence_solver", ctypes.c_int),
        ("max_iterations_v", ctypes.c_uint32),
        ("max_error_v", ctypes.c_double),
        ("xsph", ctypes.c_double),
        ("xsph_boundary", ctypes.c_double),
        ("viscosity_method", ctypes.c_int),
        ("viscosity", ctypes.c_double),
        ("viscosity_boundary", ctypes.c_double),
        ("visco_max_iter", ctypes.c_uint32),
        ("visco_max_error", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_uint32),
        ("iterations_v", ctypes.c_uint32),
        ("visco_iterations", ctypes.c_uint32),
        ("max_fluid_neighbors", ctypes.c_uint32),
        ("max_boundary_neighbors", ctypes.c_uint32),
        ("flags", ctypes.c_uint32),
        ("avg_density_err", ctypes.c_double),
        ("avg_density_err_v", ctypes.c_double),
        ("visco_error", ctypes.c_double),
        ("dt_used", ctypes.c_double),
        ("dt_next", ctypes.c_double),
        ("time", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64),
        ("learned_used", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("ws_residual_classic", ctypes.c_double * 2),
        ("ws_residual_learned", ctypes.c_double * 2),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, ctypes.Array) else v
        return out


EXPORTS = [
    "sphgb_abi_version", "sphgb_create", "sphgb_destroy", "sphgb_last_error", "sphgb_default_params",
    "sphgb_set_params", "sphgb_get_params", "sphgb_upload_boundary", "sphgb_upload_boundary_f32",
    "sphgb_upload_fluid", "sphgb_upload_fluid_f32", "sphgb_set_time_step", "sphgb_get_time_step",
    "sphgb_set_time", "sphgb_step", "sphgb_sync", "sphgb_download", "sphgb_upload_field", "sphgb_neighbors",
    "sphgb_download_fields", "sphgb_upload_fields",
    "sphgb_num_particles", "sphgb_get_stream", "sphgb_profile_enable", "sphgb_profile_reset", "sphgb_profile_read",
    "sphgb_set_warmstart_mlp", "sphgb_set_feature_output", "sphgb_upload_scenes", "sphgb_num_scenes",
    "sphgb_scene_stats", "sphgb_set_warmstart_gate", "sphgb_set_lanes_per_particle", "sphgb_get_lanes_per_particle",
    "sphgb_export_vtk", "sphgb_export_wait", "sphgb_export_bgeo", "sphgb_field_id", "sphgb_save_state", "sphgb_load_state",
    "sphgb_set_boundary_bodies", "sphgb_boundary_forces", "sphgb_clear_boundary_forces",
    "sphgb_set_neighbor_staging", "sphgb_get_neighbor_staging", "sphgb_set_solver_block_threads",
    "sphgb_get_solver_block_threads",
    "sphgb_add_volume_map", "sphgb_add_volume_map_values", "sphgb_get_volume_map", "sphgb_clear_volume_maps",
    "sphgb_set_boundary_method", "sphgb_set_volume_map_motion", "sphgb_set_body_motion", "sphgb_set_fluid_phases",
    "sphgb_set_fluid_phase_viscosity", "sphgb_set_fluid_phase_xsph",
    "sphgb_set_volume_map_scene", "sphgb_save_particle_state", "sphgb_load_particle_state",
]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libsphgb300.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("libsphgb300.so is missing; run splishsplash_gb300.build.build()")
    L = ctypes.CDLL(_build.LIB)
    vp, u32, i32, dbl = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_double
    L.sphgb_abi_version.restype = i32
    L.sphgb_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
    L.sphgb_destroy.argtypes = [vp]
    L.sphgb_last_error.argtypes = [vp]
    L.sphgb_last_error.restype = ctypes.c_char_p
    L.sphgb_default_params.argtypes = [ctypes.POINTER(Params)]
    L.sphgb_set_params.argtypes = [vp, ctypes.POINTER(Params)]
    L.sphgb_get_params.argtypes = [vp, ctypes.POINTER(Params)]
    L.sphgb_upload_boundary.argtypes = [vp, vp, u32]
    L.sphgb_upload_boundary_f32.argtypes = [vp, vp, u32]
    L.sphgb_upload_fluid.argtypes = [vp, vp, vp, vp, u32]
    L.sphgb_upload_fluid_f32.argtypes = [vp, vp, vp, vp, u32]
    L.sphgb_set_time_step.argtypes = [vp, dbl]
    L.sphgb_get_time_step.argtypes = [vp, ctypes.POINTER(dbl)]
    L.sphgb_set_time.argtypes = [vp, dbl]
    L.sphgb_step.argtypes = [vp, ctypes.POINTER(Stats)]
    L.sphgb_sync.argtypes = [vp, ctypes.POINTER(Stats)]
    L.sphgb_download.argtypes = [vp, i32, vp, i32]
    L.sphgb_upload_field.argtypes = [vp, i32, vp, i32]
    L.sphgb_download_fields.argtypes = [vp, ctypes.c_uint32, vp, vp, i32]
    L.sphgb_upload_fields.argtypes = [vp, ctypes.c_uint32, vp, vp, i32]
    L.sphgb_neighbors.argtypes = [vp, i32, vp, vp, ctypes.c_size_t]
    L.sphgb_num_particles.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    L.sphgb_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.sphgb_set_warmstart_mlp.argtypes = [vp, vp]
    L.sphgb_set_feature_output.argtypes = [vp, i32]
    L.sphgb_upload_scenes.argtypes = [vp, u32, vp, vp, vp, vp, vp]
    L.sphgb_num_scenes.argtypes = [vp, ctypes.POINTER(u32)]
    L.sphgb_scene_stats.argtypes = [vp, u32, u32, ctypes.POINTER(Stats)]
    L.sphgb_set_warmstart_gate.argtypes = [vp, u32, u32]
    L.sphgb_set_lanes_per_particle.argtypes = [vp, u32]
    L.sphgb_get_lanes_per_particle.argtypes = [vp, ctypes.POINTER(u32), vp]
    L.sphgb_set_solver_block_threads.argtypes = [vp, u32]
    L.sphgb_get_solver_block_threads.argtypes = [vp, ctypes.POINTER(u32), vp]
    L.sphgb_export_vtk.argtypes = [vp, ctypes.c_char_p, vp, u32, i32]
    L.sphgb_export_wait.argtypes = [vp]
    L.sphgb_export_bgeo.argtypes = [vp, ctypes.c_char_p, vp, u32, i32, i32]
    L.sphgb_field_id.argtypes = [ctypes.c_char_p]
    L.sphgb_save_state.argtypes = [vp, ctypes.c_char_p]
    L.sphgb_load_state.argtypes = [vp, ctypes.c_char_p]
    L.sphgb_save_particle_state.argtypes = [vp, ctypes.c_char_p, i32]
    L.sphgb_load_particle_state.argtypes = [vp, ctypes.c_char_p]
    L.sphgb_set_boundary_bodies.argtypes = [vp, vp, u32, vp, vp]
    L.sphgb_boundary_forces.argtypes = [vp, vp, vp]
    L.sphgb_clear_boundary_forces.argtypes = [vp, i32]
    L.sphgb_set_neighbor_staging.argtypes = [vp, i32]
    L.sphgb_add_volume_map.argtypes = [vp, vp, u32, vp, u32, vp, dbl, i32, vp, vp, u32, ctypes.POINTER(u32)]
    L.sphgb_add_volume_map_values.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(u32)]
    L.sphgb_get_volume_map.argtypes = [vp, u32, vp, vp, vp, vp, vp]
    L.sphgb_clear_volume_maps.argtypes = [vp]
    L.sphgb_set_boundary_method.argtypes = [vp, i32]
    L.sphgb_set_volume_map_motion.argtypes = [vp, u32, vp, vp, vp, vp]
    L.sphgb_set_body_motion.argtypes = [vp, u32, vp, vp, vp, vp]
    L.sphgb_set_fluid_phases.argtypes = [vp, u32, vp, vp]
    L.sphgb_set_fluid_phase_viscosity.argtypes = [vp, u32, vp, vp]
    L.sphgb_set_fluid_phase_xsph.argtypes = [vp, u32, vp, vp]
    L.sphgb_set_volume_map_scene.argtypes = [vp, u32, u32]
    L.sphgb_get_neighbor_staging.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_float),
                                             ctypes.POINTER(ctypes.c_float)]
    L.sphgb_profile_enable.argtypes = [vp, i32]
    L.sphgb_profile_reset.argtypes = [vp]
    L.sphgb_profile_read.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(dbl)]
    for name in EXPORTS:
        if name != "sphgb_last_error":
            getattr(L, name).restype = i32
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def params_from(sp) -> Params:
    """SPHParams (scene-key names) -> sphgb_params."""
    q = Params()
    q.particle_radius = sp.particleRadius
    q.density0 = sp.density0
    q.gravity = (ctypes.c_double * 3)(*sp.gravitation)
    q.cfl_method = sp.cflMethod
    q.cfl_factor = sp.cflFactor
    q.cfl_min_time_step = sp.cflMinTimeStepSize
    q.cfl_max_time_step = sp.cflMaxTimeStepSize
    q.min_iterations = sp.minIterations
    q.max_iterations = sp.maxIterations
    q.max_error = sp.maxError
    q.enable_divergence_solver = int(sp.enableDivergenceSolver)
    q.max_iterations_v = sp.maxIterationsV
    q.max_error_v = sp.maxErrorV
    q.xsph = sp.xsph
    q.xsph_boundary = sp.xsphBoundary
    q.viscosity_method = sp.viscosityMethod
    q.viscosity = sp.viscosity
    q.viscosity_boundary = sp.viscosityBoundary
    q.visco_max_iter = sp.viscoMaxIter
    q.visco_max_error = sp.viscoMaxError
    return q


class Mlp:
    """The warm-start network (sphgb_mlp): BF16 tensor-core forward, hand-written backward/Adam."""

    def __init__(self, device: int = 0, seed: int = 1):
        self.L = load()
        L = self.L
        vp, u32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float
        L.sphgb_mlp_create.argtypes = [ctypes.c_int, u32, ctypes.POINTER(vp)]
        L.sphgb_mlp_destroy.argtypes = [vp]
        L.sphgb_mlp_last_error.argtypes = [vp]
        L.sphgb_mlp_last_error.restype = ctypes.c_char_p
        L.sphgb_mlp_num_params.restype = ctypes.c_int
        L.sphgb_mlp_get_params.argtypes = [vp, vp]
        L.sphgb_mlp_set_params.argtypes = [vp, vp]
        L.sphgb_mlp_set_output_scale.argtypes = [vp, f32, f32]
        L.sphgb_mlp_get_output_scale.argtypes = [vp, ctypes.POINTER(f32), ctypes.POINTER(f32)]
        L.sphgb_mlp_forward.argtypes = [vp, vp, u32, vp]
        L.sphgb_mlp_loss_grad.argtypes = [vp, vp, vp, vp, u32, ctypes.POINTER(f32), vp]
        L.sphgb_mlp_train.argtypes = [vp, vp, vp, vp, u32, u32, u32, f32, u32, vp]
        for name in ("sphgb_mlp_create", "sphgb_mlp_destroy", "sphgb_mlp_get_params", "sphgb_mlp_set_params",
                     "sphgb_mlp_set_output_scale", "sphgb_mlp_get_output_scale", "sphgb_mlp_forward",
                     "sphgb_mlp_loss_grad", "sphgb_mlp_train"):
            getattr(L, name).restype = ctypes.c_int
        h = ctypes.c_void_p()
        rc = L.sphgb_mlp_create(device, seed, ctypes.byref(h))
        if rc != OK:
            raise SphgbError(rc, "sphgb_mlp_create failed (no CUDA device?)")
        self.h = h
        self.n_params = int(L.sphgb_mlp_num_params())

    def _check(self, rc):
        if rc != OK:
            raise SphgbError(rc, self.L.sphgb_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.sphgb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._check(self.L.sphgb_mlp_get_params(self.h, _p(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        self._check(self.L.sphgb_mlp_set_params(self.h, _p(p)))

    def set_output_scale(self, scale_v: float, scale_p: float):
        self._check(self.L.sphgb_mlp_set_output_scale(self.h, scale_v, scale_p))

    def output_scale(self):
        a, b = ctypes.c_float(), ctypes.c_float()
        self._check(self.L.sphgb_mlp_get_output_scale(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], 2), np.float32)
        self._check(self.L.sphgb_mlp_forward(self.h, _p(X), X.shape[0], _p(Y)))
        return Y

    def loss_grad(self, X, T, mask=None):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        M = None if mask is None else np.ascontiguousarray(mask, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        self._check(self.L.sphgb_mlp_loss_grad(self.h, _p(X), _p(T), _p(M), X.shape[0], ctypes.byref(loss), _p(g)))
        return float(loss.value), g

    def train(self, X, T, mask=None, epochs=10, batch=4096, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        M = None if mask is None else np.ascontiguousarray(mask, np.float32)
        losses = np.zeros(epochs, np.float32)
        self._check(self.L.sphgb_mlp_train(self.h, _p(X), _p(T), _p(M), X.shape[0], epochs, batch, lr, seed,
                                           _p(losses)))
        return losses


def _is_tensor(a) -> bool:
    return hasattr(a, "data_ptr") and hasattr(a, "is_contiguous") and hasattr(a, "numel")


def _buffer(a):
    """(address, elements, numpy dtype, C-contiguous) of a numpy array or a torch tensor (host or
    device memory)"""
    if isinstance(a, np.ndarray):
        return a.ctypes.data, a.size, a.dtype, bool(a.flags["C_CONTIGUOUS"])
    if _is_tensor(a):
        dt = {"torch.float32": np.dtype(np.float32), "torch.float64": np.dtype(np.float64)}.get(str(a.dtype))
        return a.data_ptr(), a.numel(), dt, bool(a.is_contiguous())
    raise TypeError(f"expected a numpy array or a torch tensor, got {type(a).__name__}")


class Context:
    """One device-resident fluid model + static boundary (one sphgb_ctx)."""

    def __init__(self, precision: str = "fp32", device: int = 0, use_graph: bool = False,
                 max_fluid_neighbors: int = 0, max_boundary_neighbors: int = 0):
        self.L = load()
        cfg = Config()
        cfg.abi_version = SPHGB_ABI_VERSION
        cfg.device = device
        cfg.precision = PRECISION_FP64 if precision == "fp64" else PRECISION_FP32
        cfg.max_fluid_neighbors = max_fluid_neighbors
        cfg.max_boundary_neighbors = max_boundary_neighbors
        cfg.use_graph = int(use_graph)
        h = ctypes.c_void_p()
        rc = self.L.sphgb_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != OK:
            raise SphgbError(rc, "sphgb_create failed (no CUDA device?)")
        self.h = h
        self.precision = precision

    def _check(self, rc):
        if rc != OK:
            raise SphgbError(rc, self.L.sphgb_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.sphgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, sp):
        self._check(self.L.sphgb_set_params(self.h, ctypes.byref(params_from(sp))))

    def get_params(self) -> Params:
        q = Params()
        self._check(self.L.sphgb_get_params(self.h, ctypes.byref(q)))
        return q

    def upload_boundary(self, xb):
        xb = np.ascontiguousarray(xb, dtype=np.float64)
        self._check(self.L.sphgb_upload_boundary(self.h, _p(xb), xb.shape[0]))

    def upload_fluid(self, x, v, ids=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        idp = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        self._check(self.L.sphgb_upload_fluid(self.h, _p(x), _p(v), _p(idp), x.shape[0]))

    def upload_scenes(self, xs, vs, xbs):
        """A batch of independent scenes: per scene fluid positions / velocities (n_s x 3) and
        boundary positions (nb_s x 3).  Fields download in the concatenated scene order."""
        n = np.array([len(x) for x in xs], np.uint32)
        nb = np.array([len(b) for b in xbs], np.uint32)
        x = np.ascontiguousarray(np.concatenate(xs), np.float64)
        v = np.ascontiguousarray(np.concatenate(vs), np.float64)
        xb = np.ascontiguousarray(np.concatenate([np.reshape(b, (-1, 3)) for b in xbs]), np.float64)
        self._check(self.L.sphgb_upload_scenes(self.h, len(xs), _p(n), _p(nb), _p(x), _p(v),
                                               _p(xb) if xb.size else None))
        self.scene_sizes = n

    def num_scenes(self):
        k = ctypes.c_uint32()
        self._check(self.L.sphgb_num_scenes(self.h, ctypes.byref(k)))
        return k.value

    def scene_stats(self, first: int = 0, count: int = None):
        """Per-scene statistics of the last step (list of dicts)."""
        if count is None:
            count = self.num_scenes() - first
        arr = (Stats * max(count, 1))()
        self._check(self.L.sphgb_scene_stats(self.h, first, count, arr))
        return [arr[k].as_dict() for k in range(count)]

    def set_time_step(self, dt):
        self._check(self.L.sphgb_set_time_step(self.h, float(dt)))

    def get_time_step(self):
        d = ctypes.c_double()
        self._check(self.L.sphgb_get_time_step(self.h, ctypes.byref(d)))
        return d.value

    def set_time(self, t):
        self._check(self.L.sphgb_set_time(self.h, float(t)))

    def step(self, wait: bool = True):
        st = Stats()
        self._check(self.L.sphgb_step(self.h, ctypes.byref(st) if wait else None))
        return st.as_dict() if wait else None

    def sync(self):
        st = Stats()
        self._check(self.L.sphgb_sync(self.h, ctypes.byref(st)))
        return st.as_dict()

    def num_particles(self):
        n, nb = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.L.sphgb_num_particles(self.h, ctypes.byref(n), ctypes.byref(nb)))
        return n.value, nb.value

    def download(self, name: str, dtype=np.float64, out: np.ndarray = None) -> np.ndarray:
        """Field in particle-id order.  `out` (C-contiguous, right size and dtype, e.g. a
        pinned buffer) is filled in place when given."""
        fid, comp = FIELDS[name]
        n, nb = self.num_particles()
        m = nb if name.startswith("boundary") and name != "boundary neighbors" else n
        if name in ("id", "fluid neighbors", "boundary neighbors", "state", "object_id"):
            dtype = np.uint32
        if out is None:
            out = np.zeros((m, comp) if comp > 1 else (m,), dtype=dtype)
        if not out.flags["C_CONTIGUOUS"] or out.size != m * comp:
            raise ValueError("download target must be C-contiguous with n x components elements")
        dt = {np.dtype(np.float32): DTYPE_F32, np.dtype(np.float64): DTYPE_F64,
              np.dtype(np.uint32): DTYPE_U32}[out.dtype]
        self._check(self.L.sphgb_download(self.h, fid, _p(out), dt))
        return out

    def upload_field(self, name: str, values):
        """Set a field from particle-id ordered values (float32 or float64, no conversion copy)."""
        fid, comp = FIELDS[name]
        a = np.asarray(values)
        if a.dtype not in (np.float32, np.float64) or not a.flags["C_CONTIGUOUS"]:
            a = np.ascontiguousarray(a, dtype=np.float64)
        dt = DTYPE_F32 if a.dtype == np.float32 else DTYPE_F64
        self._check(self.L.sphgb_upload_field(self.h, fid, _p(a), dt))

    def download_fields(self, outs: dict) -> dict:
        """Several fields in one call: {name: out} with C-contiguous float32 (or all float64)
        targets of n x components elements, filled in place: numpy arrays, or torch tensors on
        the host (pinned ones are written by the device directly) or on the context's device."""
        names = list(outs)
        bufs = [_buffer(outs[k]) for k in names]
        dtypes = {b[2] for b in bufs}
        if len(dtypes) != 1 or next(iter(dtypes)) not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise ValueError("download_fields targets must all be float32 or all float64")
        n, _ = self.num_particles()
        for k, b in zip(names, bufs):
            if not b[3] or b[1] != n * FIELDS[k][1]:
                raise ValueError(f"download target {k!r} must be C-contiguous with n x components elements")
        fids = np.array([FIELDS[k][0] for k in names], np.int32)
        ptrs = (ctypes.c_void_p * len(bufs))(*[b[0] for b in bufs])
        dt = DTYPE_F32 if bufs[0][2] == np.float32 else DTYPE_F64
        self._check(self.L.sphgb_download_fields(self.h, len(bufs), _p(fids), ptrs, dt))
        return outs

    def upload_fields(self, values: dict):
        """Several fields in one call: {name: particle-id ordered values}, all float32 or all float64:
        numpy arrays (others are converted), or C-contiguous torch tensors on the host or on the
        context's device."""
        names = list(values)
        vals = [values[k] if _is_tensor(values[k]) else np.asarray(values[k]) for k in names]
        bufs = [_buffer(v) for v in vals]
        f32 = all(b[2] == np.float32 and b[3] for b in bufs)
        if not f32 and any(_is_tensor(v) for v in vals):
            if not all(b[2] == np.float64 and b[3] for b in bufs):
                raise ValueError("upload_fields tensors must be C-contiguous and all float32 or all float64")
        elif not f32:
            vals = [np.ascontiguousarray(v, dtype=np.float64) for v in vals]
            bufs = [_buffer(v) for v in vals]
        n, _ = self.num_particles()
        for k, b in zip(names, bufs):
            if b[1] != n * FIELDS[k][1]:
                raise ValueError(f"upload source {k!r} must hold n x components elements")
        fids = np.array([FIELDS[k][0] for k in names], np.int32)
        ptrs = (ctypes.c_void_p * len(bufs))(*[b[0] for b in bufs])
        self._check(self.L.sphgb_upload_fields(self.h, len(bufs), _p(fids), ptrs, DTYPE_F32 if f32 else DTYPE_F64))

    def set_warmstart_mlp(self, mlp):
        """Use a trained network for both warm starts (None: classic warm start only)."""
        self._check(self.L.sphgb_set_warmstart_mlp(self.h, None if mlp is None else mlp.h))

    def set_warmstart_gate(self, div_sweeps: int = 0, pressure_sweeps: int = 0):
        """Jacobi iterations both warm-start candidates run before they are compared, per
        solver (0: default, 1 divergence / max(minIterations, 4) pressure; 1: initial residuals)."""
        self._check(self.L.sphgb_set_warmstart_gate(self.h, int(div_sweeps), int(pressure_sweeps)))

    def set_lanes_per_particle(self, lanes: int = 0):
        """Lanes per particle of the neighbour passes (1, 2, 4; 0 = autotune on the next step)."""
        self._check(self.L.sphgb_set_lanes_per_particle(self.h, int(lanes)))

    def lanes_per_particle(self):
        """(lanes in use, autotuner trial step times in ms for 1, 2, 4 lanes)."""
        k = ctypes.c_uint32()
        t = np.zeros(3, np.float32)
        self._check(self.L.sphgb_get_lanes_per_particle(self.h, ctypes.byref(k), _p(t)))
        return int(k.value), [float(v) for v in t]

    def set_solver_block_threads(self, threads: int = 0):
        """Threads per block of the one-lane solver passes: 128, 256, 512 (one scene), 0 = autotune."""
        self._check(self.L.sphgb_set_solver_block_threads(self.h, int(threads)))

    def solver_block_threads(self):
        """(threads per block in use, autotuner trial step times in ms for 128, 256, 512)."""
        k = ctypes.c_uint32()
        t = np.zeros(3, np.float32)
        self._check(self.L.sphgb_get_solver_block_threads(self.h, ctypes.byref(k), _p(t)))
        return int(k.value), [float(v) for v in t]

    def set_boundary_bodies(self, body, center, dynamic=None):
        """Bodies of the boundary particles (BoundaryModel per rigid body): body[k] is the body of
        boundary particle k in upload order, center (nbodies x 3) the bodies' reference points
        for torques, dynamic (nbodies) which bodies collect forces (default all).  The fluid's
        forces on the dynamic bodies accumulate every step until clear_boundary_forces()."""
        center = np.ascontiguousarray(center, np.float64).reshape(-1, 3)
        nb = int(center.shape[0])
        if nb == 0:
            self._check(self.L.sphgb_set_boundary_bodies(self.h, None, 0, None, None))
            self._nbodies = 0
            return
        body = None if body is None else np.ascontiguousarray(body, np.uint32)   # None: volume-map bodies
        dyn = None if dynamic is None else np.ascontiguousarray(dynamic, np.int32)
        if dyn is not None and dyn.size != nb:
            raise ValueError("dynamic needs one flag per body")
        self._check(self.L.sphgb_set_boundary_bodies(self.h, _p(body), nb, _p(center), _p(dyn)))
        self._nbodies = nb

    def boundary_forces(self):
        """(force, torque), each nbodies x 3 float64: BoundaryModel::getForceAndTorque per body."""
        n = getattr(self, "_nbodies", 0)
        f = np.zeros((n, 3), np.float64)
        t = np.zeros((n, 3), np.float64)
        if n:
            self._check(self.L.sphgb_boundary_forces(self.h, _p(f), _p(t)))
        return f, t

    def clear_boundary_forces(self, body: int = -1):
        """BoundaryModel::clearForceAndTorque of one body (default: every body)."""
        self._check(self.L.sphgb_clear_boundary_forces(self.h, int(body)))

    # ---- Bender2019 volume maps ------------------------------------------------
    @staticmethod
    def volume_map_nodes(res):
        nx, ny, nz = (int(r) for r in res)
        return ((nx + 1) * (ny + 1) * (nz + 1) + 2 * nx * (ny + 1) * (nz + 1) + 2 * (nx + 1) * ny * (nz + 1)
                + 2 * (nx + 1) * (ny + 1) * nz)

    def add_volume_map(self, vertices, faces, res, thickness=0.0, invert=False, rotation=None, translation=None,
                       order=0):
        """Build the volume map of a static body from its triangle mesh; returns the body index."""
        v = np.ascontiguousarray(vertices, np.float64)
        f = np.ascontiguousarray(faces, np.uint32)
        r = np.ascontiguousarray(res, np.uint32)
        R = None if rotation is None else np.ascontiguousarray(rotation, np.float64)
        t = None if translation is None else np.ascontiguousarray(translation, np.float64)
        body = ctypes.c_uint32()
        self._check(self.L.sphgb_add_volume_map(self.h, _p(v), v.shape[0], _p(f), f.shape[0], _p(r), float(thickness),
                                                int(invert), _p(R), _p(t), int(order), ctypes.byref(body)))
        return int(body.value)

    def add_volume_map_values(self, res, box_min, box_max, distance, volume, rotation=None, translation=None):
        r = np.ascontiguousarray(res, np.uint32)
        lo = np.ascontiguousarray(box_min, np.float64)
        hi = np.ascontiguousarray(box_max, np.float64)
        d = np.ascontiguousarray(distance, np.float64)
        vol = np.ascontiguousarray(volume, np.float64)
        R = None if rotation is None else np.ascontiguousarray(rotation, np.float64)
        t = None if translation is None else np.ascontiguousarray(translation, np.float64)
        body = ctypes.c_uint32()
        self._check(self.L.sphgb_add_volume_map_values(self.h, _p(r), _p(lo), _p(hi), _p(d), _p(vol), _p(R), _p(t),
                                                       ctypes.byref(body)))
        return int(body.value)

    def volume_map(self, body):
        """(res, box_min, box_max, distance, volume) of a map; node values in FP64."""
        r = np.zeros(3, np.uint32)
        lo = np.zeros(3)
        hi = np.zeros(3)
        self._check(self.L.sphgb_get_volume_map(self.h, int(body), _p(r), _p(lo), _p(hi), None, None))
        n = self.volume_map_nodes(r)
        d = np.zeros(n)
        vol = np.zeros(n)
        self._check(self.L.sphgb_get_volume_map(self.h, int(body), None, None, None, _p(d), _p(vol)))
        return r, lo, hi, d, vol

    def clear_volume_maps(self):
        self._check(self.L.sphgb_clear_volume_maps(self.h))

    def set_boundary_method(self, method: int):
        """0 Akinci2012 boundary particles, 2 Bender2019 volume maps."""
        self._check(self.L.sphgb_set_boundary_method(self.h, int(method)))

    def set_volume_map_scene(self, body: int, scene: int):
        """the scene of a batch that volume map `body` belongs to (default 0)"""
        self._check(self.L.sphgb_set_volume_map_scene(self.h, int(body), int(scene)))

    def set_volume_map_motion(self, body: int, rotation=None, translation=None, velocity=None, omega=None):
        """Pose (row-major rotation, translation) and velocity / angular velocity of the body of
        volume map `body` for the next steps; None keeps the pose, zero velocities."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).ravel()
                for a in (rotation, translation, velocity, omega)]
        for a, n in zip(arrs, (9, 3, 3, 3)):
            if a is not None and a.size != n:
                raise ValueError("rotation needs 9 values, translation / velocity / omega 3")
        self._check(self.L.sphgb_set_volume_map_motion(self.h, int(body), *[None if a is None else _p(a) for a in arrs]))

    def set_fluid_phases(self, counts=(), density0=()):
        """Fluid phases: the particles in id order form len(counts) phases of the given rest
        densities; () returns to one phase."""
        c = np.ascontiguousarray(counts, np.uint32)
        d = np.ascontiguousarray(density0, np.float64)
        if c.size != d.size:
            raise ValueError("one rest density per phase")
        self._check(self.L.sphgb_set_fluid_phases(self.h, c.size, _p(c) if c.size else None, _p(d) if d.size else None))

    def set_fluid_phase_viscosity(self, viscosity=(), viscosity_boundary=()):
        """Weiler2018 nu and nu_b per fluid phase (each model's own); () returns to the shared
        parameters."""
        a = np.ascontiguousarray(viscosity, np.float64)
        b = np.ascontiguousarray(viscosity_boundary, np.float64)
        if a.size != b.size:
            raise ValueError("one boundary viscosity per phase")
        self._check(self.L.sphgb_set_fluid_phase_viscosity(self.h, a.size, _p(a) if a.size else None,
                                                           _p(b) if b.size else None))

    def set_fluid_phase_xsph(self, xsph=(), xsph_boundary=()):
        """XSPH fluid and boundary coefficients per fluid phase (each model's own); () returns to
        the shared parameters."""
        a = np.ascontiguousarray(xsph, np.float64)
        b = np.ascontiguousarray(xsph_boundary, np.float64)
        if a.size != b.size:
            raise ValueError("one boundary coefficient per phase")
        self._check(self.L.sphgb_set_fluid_phase_xsph(self.h, a.size, _p(a) if a.size else None,
                                                      _p(b) if b.size else None))

    def set_body_motion(self, body: int, rotation=None, translation=None, velocity=None, omega=None):
        """Pose and velocity of boundary body `body` (its particles uploaded in body coordinates) for
        the next steps; None keeps the pose, zero velocities."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).ravel()
                for a in (rotation, translation, velocity, omega)]
        for a, n in zip(arrs, (9, 3, 3, 3)):
            if a is not None and a.size != n:
                raise ValueError("rotation needs 9 values, translation / velocity / omega 3")
        self._check(self.L.sphgb_set_body_motion(self.h, int(body), *[None if a is None else _p(a) for a in arrs]))

    def set_neighbor_staging(self, mode: int = 0):
        """Shared-memory staging of the solver passes: 0 autotuned (default), 1 off, 2 on."""
        self._check(self.L.sphgb_set_neighbor_staging(self.h, int(mode)))

    def neighbor_staging(self):
        """(in use, fraction of the last step's blocks staged, autotuner trial step ms)."""
        a = ctypes.c_int()
        f = ctypes.c_float()
        t = ctypes.c_float()
        self._check(self.L.sphgb_get_neighbor_staging(self.h, ctypes.byref(a), ctypes.byref(f), ctypes.byref(t)))
        return bool(a.value), float(f.value), float(t.value)

    def export_vtk(self, path: str, fields=(), wait: bool = True):
        """Legacy VTK file of all fluid particles (positions, ids and the named fields), written
        from the device copy; with wait=False the copy and the write overlap the next steps."""
        ids = np.array([FIELDS[f][0] for f in fields], np.int32)
        self._check(self.L.sphgb_export_vtk(self.h, os.fsencode(path), _p(ids) if ids.size else None, ids.size,
                                            int(wait)))

    def export_bgeo(self, path: str, fields=(), level: int = -1, wait: bool = True):
        """Partio BGEO file of all fluid particles (position, id and the named scalar / vector
        fields), gzip-compressed at zlib level `level` (-1: zlib's default) or plain (0)."""
        ids = np.array([FIELDS[f][0] for f in fields], np.int32)
        self._check(self.L.sphgb_export_bgeo(self.h, os.fsencode(path), _p(ids) if ids.size else None, ids.size,
                                             int(level), int(wait)))

    def export_wait(self):
        self._check(self.L.sphgb_export_wait(self.h))

    def save_state(self, path: str):
        self._check(self.L.sphgb_save_state(self.h, os.fsencode(path)))

    def save_particle_state(self, path: str, level: int = -1):
        """The reference's per-fluid-model state file (SimulatorBase::writeFluidParticlesState):
        partio BGEO with id, state, object_id, position, velocity, p / rho^2, p_v / rho^2 and,
        with Weiler2018, velocity difference."""
        self._check(self.L.sphgb_save_particle_state(self.h, os.fsencode(path), int(level)))

    def load_particle_state(self, path: str):
        """Reads such a file (SimulatorBase::readFluidParticlesState) into the fluid, by id."""
        self._check(self.L.sphgb_load_particle_state(self.h, os.fsencode(path)))

    def load_state(self, path: str):
        self._check(self.L.sphgb_load_state(self.h, os.fsencode(path)))

    def set_feature_output(self, on: bool = True):
        self._check(self.L.sphgb_set_feature_output(self.h, int(on)))

    def stream(self) -> int:
        """cudaStream_t (as an integer) that every kernel of this context runs on."""
        p = ctypes.c_void_p()
        self._check(self.L.sphgb_get_stream(self.h, ctypes.byref(p)))
        return int(p.value or 0)

    def profile(self, on: bool = True):
        self._check(self.L.sphgb_profile_enable(self.h, int(on)))

    def profile_reset(self):
        self._check(self.L.sphgb_profile_reset(self.h))

    def profile_read(self):
        """{kernel name: (launches, total ms)} of the CUDA-event timing since the last reset."""
        out = {}
        k = 0
        while True:
            name = ctypes.c_char_p()
            cnt = ctypes.c_uint64()
            ms = ctypes.c_double()
            rc = self.L.sphgb_profile_read(self.h, k, ctypes.byref(name), ctypes.byref(cnt), ctypes.byref(ms))
            if rc != OK:
                break
            out[name.value.decode()] = (int(cnt.value), float(ms.value))
            k += 1
        return out

    def neighbors(self, kind: int = 0):
        """CSR (offsets, indices) of the last step's lists, in particle-id numbering."""
        n, _ = self.num_particles()
        off = np.zeros(n + 1, np.uint32)
        self._check(self.L.sphgb_neighbors(self.h, kind, _p(off), None, 0))
        idx = np.zeros(max(1, int(off[-1])), np.uint32)
        self._check(self.L.sphgb_neighbors(self.h, kind, _p(off), _p(idx), idx.size))
        return off, idx[: int(off[-1])]
