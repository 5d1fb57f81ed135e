"""Precision study (the 4,194,304-particle configuration): FP32 bulk arithmetic with FP64
reductions and positions, against an all-FP64 device run and the FP64 CPU oracle, over the
first 3 steps from an identical state.  Per field (density, alpha, kappa, velocity) the max
and mean relative error are reported after every step, by particle id, with the floors
rho0*1e-6 (density), median|alpha| (alpha), 1e-3*max|kappa| (kappa), 1e-3 m/s (velocity).

Default size is a 64x64x64 block in the same 11x3x11 m box (CI speed);
SPH_PRECISION_FULL=1 runs the full 256x64x256 block.  SPH_REPORT_DIR=<dir> writes
precision_study.json there.
"""
import json
import os

import numpy as np
import pytest

import oracle
from splishsplash_gb300 import scenes
from splishsplash_gb300.dfsph import TimeStepDFSPH

pytestmark = pytest.mark.gpu

FIELDS = [("density", "density"), ("alpha", "factor raw"), ("kappa", "p / rho^2"), ("velocity", "velocity")]


def errors(gpu, ref, floor):
    g = np.asarray(gpu, np.float64)
    r = np.asarray(ref, np.float64)
    if g.ndim == 2:
        d = np.linalg.norm(g - r, axis=1)
        den = np.maximum(np.linalg.norm(r, axis=1), floor)
    else:
        d = np.abs(g - r)
        den = np.maximum(np.abs(r), floor)
    e = d / den
    return float(e.max()), float(e.mean())


def floors(sim):
    return {"density": 1000.0 * 1e-6, "alpha": float(np.median(np.abs(sim.factor_raw))) or 1e-30,
            "kappa": max(1e-3 * float(np.max(np.abs(sim.kappa))), 1e-30), "velocity": 1e-3}


def test_precision_study_first_three_steps():
    full = os.environ.get("SPH_PRECISION_FULL") == "1"
    sc = scenes.precision_4m(counts=(256, 64, 256) if full else (64, 64, 64)).as_float32()
    sim = oracle.OracleSim(sc)
    g32 = TimeStepDFSPH(sc, precision="fp32", use_graph=True)
    g64 = TimeStepDFSPH(sc, precision="fp64", use_graph=True)
    report = {"workload": f"{sc.name}: {sc.n} fluid + {sc.nb} boundary", "steps": []}
    for step in range(3):
        s32 = g32.step()
        s64 = g64.step()
        sim.step()
        so = sim.stats()
        fl = floors(sim)
        row = {"step": step + 1,
               "iterations": {"oracle": [so["iterations"], so["iterations_v"], so["visco_iterations"]],
                              "fp32": [s32["iterations"], s32["iterations_v"], s32["visco_iterations"]],
                              "fp64": [s64["iterations"], s64["iterations_v"], s64["visco_iterations"]]},
               "fp32_vs_oracle": {}, "fp64_vs_oracle": {}, "fp32_vs_fp64": {}}
        for name, field in FIELDS:
            ref = {"density": sim.density, "alpha": sim.factor_raw, "kappa": sim.kappa, "velocity": sim.v}[name]
            a = g32.getFluidModel().getFieldBuffer(field)
            b = g64.getFluidModel().getFieldBuffer(field)
            row["fp32_vs_oracle"][name] = errors(a, ref, fl[name])
            row["fp64_vs_oracle"][name] = errors(b, ref, fl[name])
            row["fp32_vs_fp64"][name] = errors(a, b, fl[name])
        report["steps"].append(row)
    out = os.environ.get("SPH_REPORT_DIR")
    if out:
        os.makedirs(out, exist_ok=True)
        with open(os.path.join(out, "precision_study.json"), "w") as f:
            json.dump(report, f, indent=1)
    first = report["steps"][0]
    # one step from the identical state: spec bars
    assert first["fp32_vs_oracle"]["density"][0] < 1e-5
    assert first["fp32_vs_oracle"]["velocity"][0] < 1e-4
    for row in report["steps"]:
        assert row["iterations"]["fp64"] == row["iterations"]["oracle"]
        for name, _ in FIELDS:
            assert row["fp64_vs_oracle"][name][0] < 1e-8, (row["step"], name, row["fp64_vs_oracle"][name])
        assert row["fp32_vs_oracle"]["density"][0] < 1e-4
    g32.close()
    g64.close()
