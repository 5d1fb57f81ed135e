"""Synthetic dam-break scenes and the DFSPH parameter block.

Scenes are generated on the host in FP64 from a seed: a jittered particle
lattice for the fluid and a single-layer lattice on the six faces of a closed
box for the Akinci2012 boundary (the reference samples wall meshes at scene
set-up, ``Simulator/StaticBoundarySimulator.cpp:96-133``; a lattice on the box
faces is the same kind of sampling for an axis-aligned box).

The fluid lattice order follows ``SimulatorBase::createFluidBlocks``
(``Simulator/SimulatorBase.cpp:1418-1526``): x outermost, z innermost, and the
particle id equals the creation index (``FluidModel.cpp:306-315``).

Parameter names mirror the reference's scene-file keys
(``Simulation.cpp:163-277``, ``TimeStepDFSPH.cpp:73-115``, ``XSPH.cpp:27-42``,
``Viscosity_Weiler2018.cpp:43-74``).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np


@dataclasses.dataclass
class SPHParams:
    """Scene parameters; field names follow the reference scene JSON keys."""

    particleRadius: float = 0.025
    density0: float = 1000.0
    gravitation: tuple = (0.0, -9.81, 0.0)
    timeStepSize: float = 0.001          # TimeManager.cpp:12
    cflMethod: int = 1
    cflFactor: float = 1.0               # "CFL 0.4": the 0.4 is inside the rule itself
    cflMinTimeStepSize: float = 1e-4
    cflMaxTimeStepSize: float = 5e-3
    # DFSPH block
    minIterations: int = 2
    maxIterations: int = 100
    maxError: float = 0.01               # percent
    enableDivergenceSolver: bool = True
    maxIterationsV: int = 100
    maxErrorV: float = 0.1               # percent
    # XSPH block
    xsph: float = 0.01
    xsphBoundary: float = 0.0
    # viscosity: 0 none, 6 Weiler et al. 2018
    viscosityMethod: int = 0
    viscosity: float = 0.01
    viscosityBoundary: float = 0.0
    viscoMaxIter: int = 100
    viscoMaxError: float = 1e-3

    @property
    def supportRadius(self) -> float:
        return 4.0 * self.particleRadius   # Simulation.cpp:283

    @property
    def volume(self) -> float:
        d = 2.0 * self.particleRadius      # FluidModel.cpp:234-253
        return 0.8 * d * d * d


@dataclasses.dataclass
class Scene:
    name: str
    x: np.ndarray            # (n, 3) float64 fluid positions
    v: np.ndarray            # (n, 3) float64 fluid velocities
    xb: np.ndarray           # (nb, 3) float64 boundary positions
    params: SPHParams
    box_min: np.ndarray
    box_max: np.ndarray

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def nb(self) -> int:
        return int(self.xb.shape[0])

    def as_float32(self) -> "Scene":
        """Round positions/velocities to float32 (the state the FP32 device path starts from)."""
        return dataclasses.replace(
            self,
            x=self.x.astype(np.float32).astype(np.float64),
            v=self.v.astype(np.float32).astype(np.float64),
            xb=self.xb.astype(np.float32).astype(np.float64),
        )


def fluid_block(counts, spacing, corner, radius, rng: Optional[np.random.Generator], jitter=0.01):
    """Jittered lattice block; order x outer, y, z inner (SimulatorBase.cpp:1476-1480)."""
    nx, ny, nz = counts
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    x = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64) * spacing
    x += np.asarray(corner, dtype=np.float64)
    if rng is not None and jitter > 0:
        x += rng.uniform(-jitter * radius, jitter * radius, size=x.shape)
    return x


def box_walls(box_min, box_max, spacing):
    """Single-layer lattice on the six faces of an axis-aligned box.

    Count = nx*ny*nz - (nx-2)*(ny-2)*(nz-2) with n = round(L/spacing)+1 per axis.
    """
    box_min = np.asarray(box_min, dtype=np.float64)
    box_max = np.asarray(box_max, dtype=np.float64)
    n = np.rint((box_max - box_min) / spacing).astype(np.int64) + 1
    pts = []
    nx, ny, nz = (int(v) for v in n)
    # z faces (full), y faces (without z rims), x faces (without y/z rims)
    for k in (0, nz - 1):
        i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        pts.append(np.stack([i.ravel(), j.ravel(), np.full(i.size, k)], 1))
    for j in (0, ny - 1):
        i, k = np.meshgrid(np.arange(nx), np.arange(1, nz - 1), indexing="ij")
        pts.append(np.stack([i.ravel(), np.full(i.size, j), k.ravel()], 1))
    for i in (0, nx - 1):
        j, k = np.meshgrid(np.arange(1, ny - 1), np.arange(1, nz - 1), indexing="ij")
        pts.append(np.stack([np.full(j.size, i), j.ravel(), k.ravel()], 1))
    idx = np.concatenate(pts, 0).astype(np.float64)
    step = (box_max - box_min) / (n - 1)
    return box_min + idx * step


def box_mesh(box_min, box_max):
    """Closed triangle mesh of an axis-aligned box: 8 vertices, 12 triangles wound
    counter-clockwise seen from outside (outward normals), for volume-map boundaries."""
    lo = np.asarray(box_min, dtype=np.float64)
    hi = np.asarray(box_max, dtype=np.float64)
    v = np.array([[hi[0] if i & 1 else lo[0], hi[1] if i & 2 else lo[1], hi[2] if i & 4 else lo[2]]
                  for i in range(8)])
    f = np.array([[0, 2, 3], [0, 3, 1], [4, 5, 7], [4, 7, 6], [0, 1, 5], [0, 5, 4],
                  [2, 6, 7], [2, 7, 3], [0, 4, 6], [0, 6, 2], [1, 3, 7], [1, 7, 5]], dtype=np.uint32)
    return v, f


def sphere_surface(center, radius, spacing):
    """Fibonacci sampling of a sphere surface at roughly the given spacing."""
    area = 4.0 * math.pi * radius * radius
    m = max(1, int(round(area / (spacing * spacing))))
    k = np.arange(m, dtype=np.float64) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / m)
    theta = math.pi * (1.0 + 5.0 ** 0.5) * k
    p = np.stack([np.cos(theta) * np.sin(phi), np.cos(phi), np.sin(theta) * np.sin(phi)], 1)
    return np.asarray(center, dtype=np.float64) + radius * p


def dambreak_8k(seed: int = 1000) -> Scene:
    """20x20x20 block, spacing 0.05, r=0.025, corner (0.1,0.1,0.1), closed 2 m box."""
    p = SPHParams(particleRadius=0.025)
    rng = np.random.default_rng(seed)
    x = fluid_block((20, 20, 20), 0.05, (0.1, 0.1, 0.1), p.particleRadius, rng)
    xb = box_walls((0, 0, 0), (2, 2, 2), 0.05)
    return Scene("dambreak_8k", x, np.zeros_like(x), xb, p, np.zeros(3), np.full(3, 2.0))


def dambreak_1m(seed: int = 1001, viscosity: bool = True, nz: int = 128) -> Scene:
    """128x64x128 block (1,048,576), spacing 0.02, r=0.01, in a 6x3x3 m box; walls at 0.012 m
    (625,002 boundary particles); Weiler2018 viscosity nu=0.01.  `nz` < 128 gives the same
    scene with a shorter block (profiling captures)."""
    p = SPHParams(particleRadius=0.01, viscosityMethod=6 if viscosity else 0, viscosity=0.01,
                  viscoMaxError=1e-3, viscoMaxIter=100)
    rng = np.random.default_rng(seed)
    x = fluid_block((128, 64, nz), 0.02, (0.02, 0.02, 0.02), p.particleRadius, rng)
    xb = box_walls((0, 0, 0), (6, 3, 3), 0.012)
    name = "dambreak_1m" if nz == 128 else f"dambreak_128x64x{nz}"
    return Scene(name, x, np.zeros_like(x), xb, p, np.zeros(3), np.array([6.0, 3.0, 3.0]))


def precision_4m(seed: int = 1002, counts=(256, 64, 256)) -> Scene:
    """256x64x256 block (4,194,304) at 0.02 in an 11x3x11 m box, walls at 0.0125 m
    (2,393,602 boundary particles).  `counts` shrinks the block for quick runs."""
    p = SPHParams(particleRadius=0.01, viscosityMethod=6, viscosity=0.01)
    rng = np.random.default_rng(seed)
    x = fluid_block(tuple(counts), 0.02, (0.02, 0.02, 0.02), p.particleRadius, rng)
    xb = box_walls((0, 0, 0), (11, 3, 11), 0.0125)
    return Scene("precision_4m", x, np.zeros_like(x), xb, p, np.zeros(3), np.array([11.0, 3.0, 11.0]))


def ensemble(num_scenes: int = 256, seed: int = 1003, n_min=2000, n_max=60000) -> List[Scene]:
    """Independent dam breaks: N_i log-uniform in [n_min, n_max], aspect ratios uniform in
    [0.5, 2], spacing 2r with r=0.025, box edge 2.5x the block's max extent, one initial
    velocity per scene uniform in [-0.5, 0.5]^3."""
    rng = np.random.default_rng(seed)
    r = 0.025
    sp = 2 * r
    scenes = []
    for s in range(num_scenes):
        target = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        ax, az = rng.uniform(0.5, 2.0, size=2)
        # counts nx:ny:nz = ax:1:az with nx*ny*nz ~ target
        ny = max(2, int(round((target / (ax * az)) ** (1.0 / 3.0))))
        nx = max(2, int(round(ax * ny)))
        nz = max(2, int(round(az * ny)))
        ext = np.array([nx, ny, nz], dtype=np.float64) * sp
        edge = 2.5 * ext.max()
        edge = math.ceil(edge / sp) * sp
        p = SPHParams(particleRadius=r)
        x = fluid_block((nx, ny, nz), sp, (2 * r, 2 * r, 2 * r), r, rng)
        v0 = rng.uniform(-0.5, 0.5, size=3)
        v = np.broadcast_to(v0, x.shape).copy()
        xb = box_walls((0, 0, 0), (edge, edge, edge), sp)
        scenes.append(Scene(f"ensemble_{s}", x, v, xb, p, np.zeros(3), np.full(3, edge)))
    return scenes


def learned_2m(seed: int = 1004) -> Scene:
    """128^3 block at 0.02 in a 6x4x6 m box with a unit-sphere obstacle at the centre.
    Fluid particles within 1+2r of the sphere centre are removed."""
    p = SPHParams(particleRadius=0.01)
    rng = np.random.default_rng(seed)
    c = np.array([3.0, 2.0, 3.0])
    ext = 128 * 0.02
    corner = c - ext / 2.0 + np.array([0.0, 0.0, 0.0])
    corner[1] = 0.02
    x = fluid_block((128, 128, 128), 0.02, corner, p.particleRadius, rng)
    keep = np.linalg.norm(x - c, axis=1) > 1.0 + 2 * p.particleRadius
    x = x[keep]
    xb = np.concatenate([box_walls((0, 0, 0), (6, 4, 6), 0.012), sphere_surface(c, 1.0, 0.012)], 0)
    return Scene("learned_2m", x, np.zeros_like(x), xb, p, np.zeros(3), np.array([6.0, 4.0, 6.0]))


def settling_sphere(counts=(64, 64, 64), box=(3.0, 2.0, 3.0), sphere_radius=0.5, seed: int = 2000) -> Scene:
    """A smaller scene of the learned-warm-start configuration's kind: a jittered block at
    0.02 m (r = 0.01) falling around a sphere obstacle at the box centre (fluid within
    radius + 2r of the centre removed), walls and sphere sampled at 0.012 m."""
    p = SPHParams(particleRadius=0.01)
    rng = np.random.default_rng(seed)
    box = np.asarray(box, dtype=np.float64)
    c = box / 2.0
    ext = np.asarray(counts, dtype=np.float64) * 0.02
    corner = c - ext / 2.0
    corner[1] = 0.02
    x = fluid_block(tuple(counts), 0.02, corner, p.particleRadius, rng)
    x = x[np.linalg.norm(x - c, axis=1) > sphere_radius + 2 * p.particleRadius]
    xb = np.concatenate([box_walls((0, 0, 0), box, 0.012), sphere_surface(c, sphere_radius, 0.012)], 0)
    return Scene(f"settling_sphere_{seed}", x, np.zeros_like(x), xb, p, np.zeros(3), box)


def small_block(counts=(8, 8, 8), radius=0.025, seed: int = 7, box=(0.8, 0.8, 0.8), corner=None,
                jitter=0.01, viscosity=False, velocity=None) -> Scene:
    """A small jittered block in a closed box, for parity tests."""
    p = SPHParams(particleRadius=radius, viscosityMethod=6 if viscosity else 0)
    rng = np.random.default_rng(seed)
    sp = 2 * radius
    if corner is None:
        corner = (2 * sp, 2 * sp, 2 * sp)
    x = fluid_block(counts, sp, corner, radius, rng, jitter=jitter)
    v = np.zeros_like(x)
    if velocity is not None:
        v[:] = velocity
    xb = box_walls((0, 0, 0), box, sp)
    return Scene(f"small_{counts[0]}x{counts[1]}x{counts[2]}", x, v, xb, p, np.zeros(3), np.asarray(box, float))


CONFIGS = {
    "dambreak_8k": dambreak_8k,
    "dambreak_1m": dambreak_1m,
    "precision_4m": precision_4m,
    "learned_2m": learned_2m,
}
