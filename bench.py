#!/usr/bin/env python
"""Benchmark: DFSPH particle-steps/s on the 1M-particle dam break (one GB300).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (single-GPU configuration of the headline metric): 128x64x128 =
1,048,576 fluid particles, r = 0.01 m, jitter +/-0.01 r, in a 6x3x3 m box of
625,002 Akinci2012 boundary particles; DFSPH with the divergence solver, XSPH
0.01, Weiler2018 viscosity nu = 0.01 (CG tol 1e-3), CFL (factor 1, dt in
[1e-4, 5e-3]).  Synthetic seeded input; nothing is skipped inside a step.

One JSON line on stdout.  `value` = fluid particles x timed steps / summed
device time of the steps (CUDA events on the library's own stream, L2 flushed
between steps), inputs resident in HBM.  `e2e` = the same metric through the
C-ABI with host buffers, on a second context over the same warm-up and step
range (the solver's iteration counts change with the phase of the dam break):
each step uploads positions/velocities from pinned host memory, steps, and
downloads positions, velocities, density and both pressure warm starts.
`roofline` = the dominant kernel (by event-timed share of a profiled run)
against the measured HBM copy bandwidth.  `cpu_baseline` = the CPU
restatement (FP32 build, OpenMP over all host cores) timed for a bounded
sample from the GPU's state.  `learned_warmstart` = the metric's second part:
the 2,097,152-lattice sphere scene for 300 steps with the classic and with the
learned warm start (committed network), iterations and device time per step at
the same tolerance.  `ensemble` = 256 independent dam breaks advanced by one
batched context (one launch per kernel, one graph per step).

--impl reference times the CPU implementation of the reference's step on the same
workload and step window, all host threads: the reference's own FP32 AVX build
(oracle/_ref/libref_f32.so, compiled from its sources by oracle/build_ref.sh) where
it is present, else the FP32 build of the CPU restatement (oracle/sph_oracle.c) --
the reference's sources are not on every host, and its AVX path is x86-64 only.

--gpus N > 1 (torchrun): independent replicas, one per GPU (the step does not
shard); value = total particle-steps / max time over ranks.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DFSPH particle-steps/s at 1M; learned vs plain warm start at 0.01% rho error"
UNIT = "particle-steps/s"
WORKLOAD = "dambreak_1m"


def baseline_metric():
    try:
        with open(os.path.join(ROOT, "BASELINE.json")) as f:
            return json.load(f)["metric"]
    except Exception:
        return METRIC


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload_config(scene):
    p = scene.params
    return {
        "workload": f"{WORKLOAD}: {scene.n} fluid + {scene.nb} Akinci2012 boundary particles, r={p.particleRadius}, "
                    f"Weiler2018 nu={p.viscosity}, XSPH {p.xsph}, DFSPH maxError {p.maxError}% / maxErrorV "
                    f"{p.maxErrorV}%, CFL factor {p.cflFactor} dt in [{p.cflMinTimeStepSize}, {p.cflMaxTimeStepSize}]",
        "fluid_particles": scene.n,
        "boundary_particles": scene.nb,
        "precision": "fp32 bulk, fp64 reductions/dt/time/positions",
        "l2": "flushed between timed steps (256 MB device write)",
    }


class Clocks:
    """nvidia-smi sampling every 50 ms, started before the warm-up; the samples whose timestamps
    fall in the timed region (mark() to stop()) are kept, or the one just before a region shorter
    than the period."""

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.index = index
        self.t0 = None

    def start(self):
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def mark(self):
        """The timed region starts."""
        self.t0 = time.time()

    def stop(self):
        t1 = time.time()
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = []
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(parts[2]), float(parts[3]), parts[6:10]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        t0 = self.t0 if self.t0 is not None else t1
        keep = [r for r in rows if t0 - 0.01 <= r[0] <= t1 + 0.01]
        if not keep:
            keep = [r for r in rows if r[0] < t0][-1:]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = {nm for r in keep for nm, val in zip(names, r[3]) if val.lower().startswith("active")}
        sm = [r[1] for r in keep]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max((r[2] for r in keep), default=None),
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_stepper(scene, threads, state=None, prefer="auto"):
    """The CPU implementation of the reference's step for the CPU legs: the reference's own FP32
    AVX build (oracle/_ref/libref_f32.so, from its sources; x86-64 hosts with the reference tree)
    when it is present, else the FP32 build of the CPU restatement (oracle/sph_oracle.c).
    Returns (step function, close function, kind, description, the RefSim or None)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refsim
    if prefer == "reference" and not refsim.available("f32"):
        raise RuntimeError("the reference's FP32 build (oracle/_ref/libref_f32.so) is not present")
    if prefer != "port" and refsim.available("f32"):
        import dataclasses
        sc = scene if state is None else dataclasses.replace(scene, x=state["x"], v=state["v"])
        r = refsim.RefSim(sc, precision="f32", analytic_kernel=False, num_threads=threads)
        if state is not None:
            r.set("p / rho^2", state["kappa"])
            r.set("p_v / rho^2", state["kappa_v"])
            if scene.params.viscosityMethod == 6:
                r.set("velocity difference", state["vdiff"])
            r.set_time_step(state["dt"])
        r.ns_ms = lambda: r.timing("neighborhood_search")[0]
        return (lambda: r.step(), r.close, "reference",
                "the reference's TimeStepDFSPH built from its sources, FP32 AVX with precomputeValues, OpenMP; "
                "its neighbour search is this project's stand-in for CompactNSearch", r)
    import oracle  # CPU baseline only
    sim = oracle.OracleSim(scene, precision="f32", num_threads=threads)
    if state is not None:
        sim.x[:] = state["x"]
        sim.v[:] = state["v"]
        sim.kappa[:] = state["kappa"]
        sim.kappa_v[:] = state["kappa_v"]
        sim.vdiff[:] = state["vdiff"]
        sim.dt = state["dt"]

    def step():
        sim.step()
        return sim.stats()
    return (step, lambda: None, "port",
            "FP32 build of the CPU restatement of the reference's step (oracle/sph_oracle.c), OpenMP; the "
            "reference's own build needs its source tree, which this host does not hold", None)


def run_oracle_sample(scene, state, budget_s, threads, prefer="auto"):
    """CPU leg from `state`: at least one step, then as many as fit in budget_s."""
    step, close, kind, desc, _ = cpu_stepper(scene, threads, state, prefer)
    t0 = time.perf_counter()
    steps = 0
    iters = []
    while True:
        st = step()
        steps += 1
        iters.append((st["iterations"], st["iterations_v"], st["visco_iterations"]))
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    close()
    return scene.n * steps / dt, steps, dt, iters, kind, desc


def max_over_ranks(x: float, dist, device) -> float:
    """The largest x over the ranks (the slowest replica's time); x itself without a process
    group.  device: the tensor's device for the group's backend (cuda for NCCL, cpu for gloo)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, n: int, steps: int, seconds: float) -> float:
    """Whole-job particle-steps/s of `world` replicas, each advancing n particles `steps` times,
    timed by the slowest replica's `seconds` (replicas only: no data-path collective)."""
    return world * n * steps / seconds


def run_reference(args):
    """The reference arm: the CPU implementation of the step on all host threads, on this
    benchmark's workload and step window (warm-up steps, then the timed steps)."""
    from splishsplash_gb300 import scenes

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene = scenes.dambreak_1m()
    threads = cpu_cores()
    step, close, kind, desc, ref = cpu_stepper(scene, threads, prefer=args.cpu_impl)
    t_w = time.perf_counter()
    warm_done = 0
    for _ in range(args.warmup):
        step()
        warm_done += 1
        if time.perf_counter() - t_w > args.ref_budget:
            break
    ns0 = ref.ns_ms() if ref is not None else 0.0
    t0 = time.perf_counter()
    steps = 0
    for _ in range(args.steps):
        step()
        steps += 1
        if time.perf_counter() - t0 > args.ref_budget:
            break
    el = time.perf_counter() - t0
    ns_s = (ref.ns_ms() - ns0) * 1e-3 if ref is not None else None
    close()
    value = scene.n * steps / el
    sample = (f"{steps} of {args.steps} requested steps after {warm_done} of {args.warmup} warm-up steps of the full "
              f"{scene.n}-particle scene from rest (the timed window of the GPU arm)")
    line = {
        "impl": "reference", "metric": baseline_metric(), "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm_done, "ms_per_step": 1e3 * el / max(steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam break)",
        "config": workload_config(scene),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": desc,
    }
    if ns_s is not None:
        line["without_neighbor_search"] = {"value": scene.n * steps / max(el - ns_s, 1e-9), "unit": UNIT,
                                           "neighbor_search_s": ns_s}
    print(json.dumps(line), flush=True)


def config_table(args):
    """Config 0 (the 8k dam break, 500 steps) on the GPU and on the host cores, and config 3
    (the 256-scene ensemble) stepped scene by scene on the host cores, as the reference would
    run it (one Simulation per process).  CPU legs: the FP32 build of the CPU restatement."""
    import torch

    from splishsplash_gb300 import scenes
    from splishsplash_gb300.dfsph import TimeStepDFSPH

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = cpu_cores()
    sc = scenes.dambreak_8k()
    ts = TimeStepDFSPH(sc, use_graph=True)
    ts.step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(499):
        ts.step()
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    ts.close()
    # the same steps queued without a host read per step (sphgb_step(ctx, NULL)), one wait at the end
    ts = TimeStepDFSPH(sc, use_graph=True)
    ts.step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(499):
        ts.ctx.step(wait=False)
    last = ts.ctx.sync()
    gpu_q_s = time.perf_counter() - t0
    ts.close()
    sim = oracle.OracleSim(sc, precision="f32", num_threads=threads)
    t0 = time.perf_counter()
    cpu_steps = 0
    while cpu_steps < 500 and time.perf_counter() - t0 < args.cpu_budget:
        sim.step()
        cpu_steps += 1
    cpu_s = time.perf_counter() - t0
    ens = scenes.ensemble(num_scenes=256)
    t0 = time.perf_counter()
    done, parts = 0, 0
    for e in ens:
        s1 = oracle.OracleSim(e, precision="f32", num_threads=threads)
        s1.step()
        parts += e.n
        done += 1
        if time.perf_counter() - t0 > 3 * args.cpu_budget:
            break
    ens_s = time.perf_counter() - t0
    return {
        "config0": {"workload": f"{sc.name}: {sc.n} fluid + {sc.nb} boundary particles",
                    "gpu": {"value": sc.n * 499 / gpu_s, "unit": UNIT, "steps": 499,
                            "timing": "wall clock over steps 2..500, one graph launch and a statistics read per step"},
                    "gpu_queued": {"value": sc.n * 499 / gpu_q_s, "unit": UNIT, "steps": 499,
                                   "time_after": last["time"],
                                   "timing": "wall clock over steps 2..500 queued without a host read per step, "
                                             "one wait at the end"},
                    "cpu": {"value": sc.n * cpu_steps / cpu_s, "unit": UNIT, "steps": cpu_steps, "cores": threads,
                            "kind": "port"}},
        "config3_cpu_sequential": {"value": parts / ens_s, "unit": UNIT, "cores": threads, "kind": "port",
                                   "sample": f"first step of {done} of 256 scenes, one after the other, including "
                                             f"each scene's set-up ({ens_s:.1f} s)"},
    }


def learned_line(steps):
    """The 2,097,152-lattice sphere scene with the classic and the learned warm start, the
    latter with the library's default gate (1 divergence / 4 pressure Jacobi sweeps of both
    candidates) and with the initial-residual gate (1 / 1).  Iterations are reported as the
    solves count them and booked: with the losing candidate's gate sweeps added."""
    from splishsplash_gb300 import learned, scenes

    sc = scenes.learned_2m()
    net = learned.load()
    res = learned.evaluate(sc, net, steps=steps, strict=True)
    net.close()
    keep = ("pressure_iterations_mean", "divergence_iterations_mean", "solver_iterations_total",
            "solver_iterations_total_booked", "gate_sweeps", "ms_per_step", "final_avg_density_error_percent",
            "max_avg_density_error_percent", "learned_used_pressure_fraction", "learned_used_div_fraction")
    return {"workload": f"{sc.name}: {sc.n} fluid + {sc.nb} boundary particles, r=0.01, unit-sphere obstacle, "
                        f"{steps} steps from rest, maxError 0.01%",
            "plain": {k: res["plain"][k] for k in keep}, "learned": {k: res["learned"][k] for k in keep},
            "learned_initial_residual_gate": {k: res["learned_initial_residual_gate"][k] for k in keep},
            "iteration_reduction": res["gain"]["iteration_reduction"],
            "iteration_reduction_booked": res["gain"]["iteration_reduction_booked"],
            "time_per_step_reduction": res["gain"]["time_per_step_reduction"],
            "initial_residual_gate": res["gain_initial_residual_gate"],
            "gate": "default: 1 divergence / 4 pressure Jacobi sweeps of both candidates; initial-residual gate: 1 / 1",
            "network": "splishsplash_gb300/data/warmstart_mlp.npz (python -m splishsplash_gb300.learned)"}


def bender2019_line(steps, device):
    """The 1M dam break with its 6x3x3 m container given as a Bender2019 volume map (the
    reference's default boundary handling) instead of 625,002 boundary particles: map
    construction time and particle-steps/s over `steps` steps after 10 warm-up steps."""
    import torch

    from splishsplash_gb300 import native, scenes
    from splishsplash_gb300.dfsph import TimeStepDFSPH

    sc = scenes.dambreak_1m()
    sc.xb = np.zeros((0, 3))
    h = 4 * sc.params.particleRadius
    # cells of about 2 h over the map box (the container grown by 8 h on every side)
    ext = np.array([6.0, 3.0, 3.0]) + 16 * h
    res = np.maximum(1, np.round(ext / (2 * h))).astype(np.uint32)
    ts = TimeStepDFSPH(sc, use_graph=True, device=device)
    v, f = scenes.box_mesh((0, 0, 0), (6.0, 3.0, 3.0))
    t0 = time.perf_counter()
    ts.ctx.add_volume_map(v, f, res, invert=True)
    build_s = time.perf_counter() - t0
    ts.ctx.set_boundary_method(2)
    for _ in range(10):
        ts.step()
    ext_s = torch.cuda.ExternalStream(ts.ctx.stream())
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    its = []
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(ext_s):
            evs[k][0].record(ext_s)
        st = ts.step()
        with torch.cuda.stream(ext_s):
            evs[k][1].record(ext_s)
        its.append((st["iterations"], st["iterations_v"]))
    torch.cuda.synchronize()
    dev_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    ts.close()
    it = np.array(its)
    return {"workload": f"dambreak_1m fluid ({sc.n} particles) in a volume-mapped 6x3x3 m box, map {res.tolist()} cells",
            "value": sc.n * steps / dev_s, "unit": UNIT, "steps": steps, "warmup": 10,
            "ms_per_step": 1e3 * dev_s / steps, "map_build_s": build_s,
            "map_nodes": int(native.Context.volume_map_nodes(res)),
            "iterations_mean": {"pressure": float(it[:, 0].mean()), "divergence": float(it[:, 1].mean())}}


def ensemble_line(steps, device, use_graph=True):
    """256 independent dam breaks (N_i log-uniform in [2000, 60000]) in one batched context:
    particle-steps/s over `steps` steps after 10 warm-up steps (inputs far larger than L2)."""
    import torch

    from splishsplash_gb300 import scenes
    from splishsplash_gb300.dfsph import BatchedTimeStepDFSPH

    ens = scenes.ensemble(num_scenes=256)
    b = BatchedTimeStepDFSPH(ens, use_graph=use_graph, device=device)
    for _ in range(10):
        b.step()
    ext = torch.cuda.ExternalStream(b.ctx.stream())
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    it = []
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(ext):
            evs[k][0].record(ext)
        st = b.step()
        with torch.cuda.stream(ext):
            evs[k][1].record(ext)
        per = b.scene_stats()
        it.append((st["iterations"], float(np.mean([p["iterations"] for p in per])),
                   st["iterations_v"], float(np.mean([p["iterations_v"] for p in per]))))
    torch.cuda.synchronize()
    dev_s = sum(a.elapsed_time(c) for a, c in evs) / 1e3
    n = int(b.sizes.sum())
    b.close()
    it = np.array(it)
    return {"workload": f"256 dam-break scenes, {n} fluid particles in total, r=0.025, per-scene CFL dt",
            "value": n * steps / dev_s, "unit": UNIT, "steps": steps, "warmup": 10,
            "ms_per_step": 1e3 * dev_s / steps,
            "pressure_iterations": {"batch_loop_mean": float(it[:, 0].mean()), "scene_mean": float(it[:, 1].mean())},
            "divergence_iterations": {"batch_loop_mean": float(it[:, 2].mean()),
                                      "scene_mean": float(it[:, 3].mean())}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=190)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: as many as --steps")
    ap.add_argument("--profile-steps", type=int, default=4)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--cpu-impl", default="auto", choices=["auto", "reference", "port"],
                    help="CPU legs: the reference's own FP32 build (where present; auto) or the CPU restatement")
    ap.add_argument("--ref-budget", type=float, default=900.0,
                    help="--impl reference: seconds after which the warm-up or the timed steps stop early")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nz", type=int, default=128,
                    help="fluid block depth (128 = the 1M workload; smaller for multi-pass profiler captures)")
    ap.add_argument("--host-loops", action="store_true",
                    help="host-driven solver loops instead of the captured graph (kernels visible to ncu)")
    ap.add_argument("--only-timed", action="store_true",
                    help="run warm-up and the device-resident timed steps only (profiling captures)")
    ap.add_argument("--no-extras", action="store_true", help="skip the learned-warm-start and ensemble lines")
    ap.add_argument("--lanes", type=int, default=0, choices=[0, 1, 2, 4],
                    help="lanes per particle of the neighbour passes (0: the library's autotuner)")
    ap.add_argument("--staging", type=int, default=0, choices=[0, 1, 2],
                    help="shared-memory staging of the solver passes: 0 autotuned, 1 off, 2 on")
    ap.add_argument("--config-table", action="store_true",
                    help="print configs 0 and 3 (GPU and host cores) as one JSON line and exit")
    ap.add_argument("--learned-steps", type=int, default=300)
    ap.add_argument("--ensemble-steps", type=int, default=60)
    ap.add_argument("--bender-steps", type=int, default=60)
    ap.add_argument("--only-bender", action="store_true", help="print the volume-map boundary line alone and exit")
    ap.add_argument("--only-ensemble", action="store_true",
                    help="print the 256-scene ensemble line alone and exit (with --host-loops: host-driven solver "
                         "loops, so that a profiler sees every kernel)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return
    if args.config_table:
        print(json.dumps({"config_table": config_table(args)}), flush=True)
        return
    if args.only_bender:
        print(json.dumps({"boundary_bender2019": bender2019_line(args.bender_steps, 0)}), flush=True)
        return
    if args.only_ensemble:
        print(json.dumps({"ensemble": ensemble_line(args.ensemble_steps, 0, use_graph=not args.host_loops)}),
              flush=True)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from splishsplash_gb300 import bytes_model, scenes
    from splishsplash_gb300.dfsph import TimeStepDFSPH

    scene = scenes.dambreak_1m(nz=args.nz)
    ts = TimeStepDFSPH(scene, precision="fp32", use_graph=not args.host_loops, device=local)
    ts.ctx.set_lanes_per_particle(args.lanes)
    ts.ctx.set_neighbor_staging(args.staging)
    ext = torch.cuda.ExternalStream(ts.ctx.stream())
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    clocks = Clocks(local)
    clocks.start()   # sampling from before the warm-up; mark() keeps the timed region's samples
    for _ in range(args.warmup):
        ts.step()

    # ---------------- device-resident timed region ----------------
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    iters = []
    launches = 0
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks.mark()
    t_wall = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            evs[k][0].record(ext)
        st = ts.step()
        with torch.cuda.stream(ext):
            evs[k][1].record(ext)
        iters.append((st["iterations"], st["iterations_v"], st["visco_iterations"]))
        launches += int(st["kernel_launches"])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    dev_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    t_max = max_over_ranks(dev_s, dist, f"cuda:{local}")
    if dist:
        dist.barrier()
    value = replica_rate(world, scene.n, args.steps, t_max)
    lanes, trial_ms = ts.ctx.lanes_per_particle()
    staged, staged_frac, staged_trial_ms = ts.ctx.neighbor_staging()
    block_threads, block_trial_ms = ts.ctx.solver_block_threads()
    if args.only_timed:
        if rank == 0:
            print(json.dumps({"metric": baseline_metric(), "value": value, "unit": UNIT, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
                              "lanes_per_particle": lanes, "staged": staged, "staged_block_fraction": staged_frac,
                              "solver_block_threads": block_threads, "note": "timed steps only"}), flush=True)
        ts.close()
        return

    # ---------------- end-to-end through the C ABI with host buffers ----------------
    # A second context over the same warm-up and step range as the device-resident run.
    n = scene.n
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    hx, hv = pin((n, 3), torch.float32), pin((n, 3), torch.float32)
    hrho, hk, hkv = pin((n,), torch.float32), pin((n,), torch.float32), pin((n,), torch.float32)
    te = TimeStepDFSPH(scene, precision="fp32", use_graph=not args.host_loops, device=local)
    te.ctx.set_lanes_per_particle(args.lanes)
    te.ctx.set_neighbor_staging(args.staging)
    for _ in range(args.warmup):
        te.step()
    te.ctx.download("position", out=hx)
    te.ctx.download("velocity", out=hv)
    torch.cuda.synchronize()
    e2e_steps = args.steps if args.e2e_steps <= 0 else min(args.e2e_steps, args.steps)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    inputs = {"position": hx, "velocity": hv}
    outputs = {"position": hx, "velocity": hv, "density": hrho, "p / rho^2": hk, "p_v / rho^2": hkv}
    for _ in range(e2e_steps):
        # as the reference-side plugin steps: the step is queued, the download waits for it and
        # its fields, then the step's statistics are read on the host
        te.ctx.upload_fields(inputs)
        te.ctx.step(wait=False)
        te.ctx.download_fields(outputs)
        te.ctx.sync()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    te.close()
    e2e_s = max_over_ranks(e2e_s, dist, f"cuda:{local}")
    e2e = {"value": replica_rate(world, n, e2e_steps, e2e_s), "unit": UNIT, "h2d_bytes_per_step": 2 * n * 3 * 4,
           "d2h_bytes_per_step": 2 * n * 3 * 4 + 3 * n * 4, "steps": e2e_steps,
           "region": f"steps {args.warmup + 1}..{args.warmup + e2e_steps} of a fresh context (same as the timed run)"}

    # ---------------- per-kernel event timing (roofline) ----------------
    ts.ctx.profile(True)
    ts.ctx.profile_reset()
    for _ in range(max(1, args.profile_steps)):
        ts.step()
    prof = ts.ctx.profile_read()
    ts.ctx.profile(False)
    nf = float(np.mean(ts.ctx.download("fluid neighbors")))
    nb = float(np.mean(ts.ctx.download("boundary neighbors")))
    total_ms = sum(ms for _, ms in prof.values())
    kernels = {}
    for name, (cnt, ms) in prof.items():
        if cnt == 0:
            continue
        avg = ms / cnt
        byts = bytes_model.per_launch(name, n, nf, nb)
        kernels[name] = {"launches": cnt, "avg_ms": avg, "share": ms / total_ms if total_ms else 0.0,
                         "algorithmic_bytes": byts, "gbs": byts / (avg * 1e-3) / 1e9 if avg > 0 else 0.0}
    dom = max(kernels, key=lambda k: kernels[k]["share"])
    peak, peak_kind = peaks()
    traffic = None
    tf = os.path.join(ROOT, "profiles", f"dram_bytes_{dom}.txt")
    if os.path.exists(tf):
        try:
            traffic = float(open(tf).read().split()[0])
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": kernels[dom]["gbs"], "peak": peak, "unit": "GB/s",
                "frac": kernels[dom]["gbs"] / peak, "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": kernels[dom]["algorithmic_bytes"],
                "avg_launch_ms": kernels[dom]["avg_ms"], "share_of_step": kernels[dom]["share"],
                "mean_neighbors": {"fluid": nf, "boundary": nb}}

    # ---------------- CPU baseline (rank 0, N = 1) ----------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        state = {k: ts.ctx.download(f) for k, f in (("x", "position"), ("v", "velocity"), ("kappa", "p / rho^2"),
                                                     ("kappa_v", "p_v / rho^2"), ("vdiff", "velocity difference"))}
        state["dt"] = ts.getTimeStepSize()
        threads = cpu_cores()
        v_cpu, s_cpu, t_cpu, it_cpu, kind, desc = run_oracle_sample(scene, state, args.cpu_budget, threads,
                                                                    args.cpu_impl)
        cpu = {"value": v_cpu, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"{s_cpu} step(s) of the full scene from the GPU state after the timed region, {t_cpu:.1f} s "
                         f"({desc}); solver iterations {it_cpu}"}

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        extras["learned_warmstart"] = learned_line(args.learned_steps)
        extras["ensemble"] = ensemble_line(args.ensemble_steps, local)
        extras["boundary_bender2019"] = bender2019_line(args.bender_steps, local)

    if rank == 0:
        it = np.array(iters)
        line = {
            "metric": baseline_metric(), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam break)",
            "config": {**workload_config(scene), "lanes_per_particle": lanes,
                       "lanes_autotune_trial_ms": dict(zip(("1", "2", "4"), trial_ms)) if args.lanes == 0 else None,
                       "staged_solver_passes": staged, "staged_block_fraction": round(staged_frac, 4),
                       "staged_autotune_trial_ms": staged_trial_ms or None,
                       "solver_block_threads": block_threads,
                       "block_threads_autotune_trial_ms": dict(zip(("128", "256", "512"), block_trial_ms))
                       if args.lanes == 0 else None},
            "e2e": e2e, "gpu_launches": launches,
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "wall_ms_per_step": 1e3 * wall / args.steps,
            "solver_iterations_mean": {"pressure": float(it[:, 0].mean()), "divergence": float(it[:, 1].mean()),
                                       "viscosity_cg": float(it[:, 2].mean())},
            "kernels": kernels,
            **extras,
        }
        print(json.dumps(line), flush=True)
    ts.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
