"""Host-side mirror of the reference's DFSPH plugin interface over the C ABI.

Names follow the reference so that code written against pySPlisHSPlasH reads
the same: ``TimeStepDFSPH.step()`` (TimeStepDFSPH.cpp:117), ``getNumIterations``
(TimeStepDFSPH.h:73), the DFSPH parameter names (TimeStepDFSPH.cpp:77-114),
``FluidModel.getFieldBuffer`` (pySPlisHSPlasH/FluidModelModule.cpp:86-118) and the
Weiler2018 parameter names (Viscosity_Weiler2018.cpp:47-73).  Every call goes
through libsphgb300.so; there is no CPU path.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import native
from .scenes import Scene, SPHParams

# parameter name -> SPHParams attribute (reference names, scene-file keys)
PARAMETERS = {
    # TimeStepDFSPH (TimeStepDFSPH.cpp:77-114)
    "minIterations": "minIterations",
    "maxIterations": "maxIterations",
    "maxError": "maxError",
    "maxIterationsV": "maxIterationsV",
    "maxErrorV": "maxErrorV",
    "enableDivergenceSolver": "enableDivergenceSolver",
    # Simulation (Simulation.cpp:163-277)
    "particleRadius": "particleRadius",
    "gravitation": "gravitation",
    "cflMethod": "cflMethod",
    "cflFactor": "cflFactor",
    "cflMinTimeStepSize": "cflMinTimeStepSize",
    "cflMaxTimeStepSize": "cflMaxTimeStepSize",
    "timeStepSize": "timeStepSize",
    # FluidModel / XSPH / Weiler2018
    "density0": "density0",
    "xsph": "xsph",
    "xsphBoundary": "xsphBoundary",
    "viscosityMethod": "viscosityMethod",
    "viscosity": "viscosity",
    "viscosityBoundary": "viscosityBoundary",
    "viscoMaxIter": "viscoMaxIter",
    "viscoMaxError": "viscoMaxError",
}


class FluidModel:
    """Field access in particle-id order (the host std::vector order)."""

    def __init__(self, ts: "TimeStepDFSPH"):
        self._ts = ts

    def numActiveParticles(self) -> int:
        return self._ts.ctx.num_particles()[0]

    def numParticles(self) -> int:
        return self.numActiveParticles()

    def getFieldBuffer(self, name: str, dtype=np.float64) -> np.ndarray:
        return self._ts.ctx.download(name, dtype)

    def setFieldBuffer(self, name: str, values) -> None:
        self._ts.ctx.upload_field(name, values)

    def getDensity0(self) -> float:
        return self._ts.params.density0

    def getVolume(self, i: int = 0) -> float:
        return self._ts.params.volume

    def getMass(self, i: int = 0) -> float:
        return self._ts.params.volume * self._ts.params.density0


class TimeStepDFSPH:
    """GPU DFSPH time step with Akinci2012 boundaries, XSPH and Weiler2018 viscosity."""

    METHOD_NAME = "DFSPH"

    def __init__(self, scene: Scene, precision: str = "fp32", use_graph: bool = True, device: int = 0,
                 max_fluid_neighbors: int = 0, max_boundary_neighbors: int = 0):
        self.params: SPHParams = dataclasses.replace(scene.params)
        self.ctx = native.Context(precision=precision, device=device, use_graph=use_graph,
                                  max_fluid_neighbors=max_fluid_neighbors,
                                  max_boundary_neighbors=max_boundary_neighbors)
        self.ctx.set_params(self.params)
        self.ctx.upload_boundary(scene.xb)
        self.ctx.upload_fluid(scene.x, scene.v)
        self.ctx.set_time_step(self.params.timeStepSize)
        self.model = FluidModel(self)
        self.last = None

    # --- reference interface ------------------------------------------------
    def getMethodName(self) -> str:
        return self.METHOD_NAME

    def step(self):
        self.last = self.ctx.step(wait=True)
        return self.last

    def step_async(self):
        self.ctx.step(wait=False)

    def sync(self):
        self.last = self.ctx.sync()
        return self.last

    def getNumIterations(self) -> int:
        return 0 if self.last is None else int(self.last["iterations"])

    def getValue(self, name: str):
        if name == "iterations":
            return self.getNumIterations()
        if name == "iterationsV":
            return 0 if self.last is None else int(self.last["iterations_v"])
        if name == "viscoIterations":
            return 0 if self.last is None else int(self.last["visco_iterations"])
        return getattr(self.params, PARAMETERS[name])

    def setValue(self, name: str, value) -> None:
        if name in ("iterations", "iterationsV", "viscoIterations"):
            raise AttributeError(f"parameter {name!r} is read-only")
        setattr(self.params, PARAMETERS[name], value)
        if name == "timeStepSize":
            self.ctx.set_time_step(value)
        else:
            self.ctx.set_params(self.params)

    def getFluidModel(self, i: int = 0) -> FluidModel:
        if i != 0:
            raise IndexError("one fluid model per context")
        return self.model

    def getTimeStepSize(self) -> float:
        return self.ctx.get_time_step()

    def setTimeStepSize(self, dt: float) -> None:
        self.ctx.set_time_step(dt)

    def close(self):
        self.ctx.close()


class BatchedTimeStepDFSPH:
    """Many independent scenes advanced together by one context: every kernel launch of a
    step covers all scenes, each scene keeps its own CFL step size and solver decisions, and
    with use_graph a step of the whole batch is one graph launch.  The scenes share the
    parameter block (that of the first scene).  No reference counterpart: the reference runs
    one scene per process (Simulation.cpp:112-119)."""

    def __init__(self, scene_list, precision: str = "fp32", use_graph: bool = True, device: int = 0,
                 max_fluid_neighbors: int = 0, max_boundary_neighbors: int = 0):
        if not scene_list:
            raise ValueError("empty batch")
        self.params: SPHParams = dataclasses.replace(scene_list[0].params)
        self.ctx = native.Context(precision=precision, device=device, use_graph=use_graph,
                                  max_fluid_neighbors=max_fluid_neighbors,
                                  max_boundary_neighbors=max_boundary_neighbors)
        self.ctx.set_params(self.params)
        self.ctx.upload_scenes([s.x for s in scene_list], [s.v for s in scene_list], [s.xb for s in scene_list])
        self.ctx.set_time_step(self.params.timeStepSize)
        self.sizes = np.array([s.n for s in scene_list], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        self.last = None

    @property
    def num_scenes(self) -> int:
        return int(self.sizes.size)

    def step(self):
        """One step of every scene; returns the batch statistics (maxima over the scenes)."""
        self.last = self.ctx.step(wait=True)
        return self.last

    def step_async(self):
        self.ctx.step(wait=False)

    def sync(self):
        self.last = self.ctx.sync()
        return self.last

    def scene_stats(self):
        return self.ctx.scene_stats()

    def getFieldBuffer(self, name: str, dtype=np.float64):
        """A field of all scenes, split per scene (list of arrays in each scene's particle order)."""
        a = self.ctx.download(name, dtype)
        return [a[self.offsets[k]:self.offsets[k + 1]] for k in range(self.num_scenes)]

    def close(self):
        self.ctx.close()
