"""Learned warm start: data collection, training and evaluation.

The network predicts, per particle, the multiplier that the divergence and the pressure
warm start apply to the previous step's stored kappa_v and kappa (the classic warm start
uses 0.5, TimeStepDFSPH.cpp:449-453 and :293-296).  Features and targets are dimensionless,
so scenes of different particle size, depth and step size train one network.

Pipeline (all GPU work goes through libsphgb300.so):
  1. collect(): run the plain solver (classic warm start) on batches of independent scenes
     (BatchedTimeStepDFSPH: all scenes of a batch in one launch per kernel) and record, per
     step, each particle's network inputs at the start of the step (SPHGB_FIELD_FEATURES)
     and the ratio of the converged stored warm start after the step to the stored value
     before it ("p_v / rho^2", "p / rho^2").  Each sample's loss weight is its previous kappa
     squared relative to its scene's mean square, so the loss is the squared error of the
     predicted kappa in the scene's own scale; samples whose classic warm start is masked
     out (zero) weigh nothing.
  2. train(): Adam (lr 1e-3) with the library's own BF16 tensor-core forward and FP32
     backward kernels.
  3. evaluate(): the same scene with the classic warm start and with the network; both
     iterate to the same tolerances.  Per step and solver both candidates run the gate's
     Jacobi iterations (sphgb_set_warmstart_gate; default 1 divergence, 4 pressure) and the
     prediction is kept only if its error after them is lower, otherwise the classic warm
     start continues.  Also reported: the network judged by the initial residuals alone
     (gate 1).  Reports iterations, device time per step and the final average density
     error.

    python -m splishsplash_gb300.learned --out <dir>   # full pipeline, writes weights + report
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import time

import numpy as np

from . import native, scenes
from .dfsph import BatchedTimeStepDFSPH, TimeStepDFSPH

SCALE_V = 1.0      # network output x SCALE_V = divergence warm-start multiplier
SCALE_P = 1.0      # network output x SCALE_P = pressure warm-start multiplier
MAX_MULT = 4.0     # the device limits the multiplier to [0, 4]
MAX_WEIGHT = 25.0
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart_mlp.npz")


def _group_by_params(scene_list):
    groups = {}
    for s in scene_list:
        groups.setdefault(repr(dataclasses.astuple(s.params)), []).append(s)
    return list(groups.values())


def targets(k_prev, k_new, mask, offsets):
    """Multiplier targets k_new / k_prev (limited to [0, MAX_MULT]) and loss weights
    (k_prev / rms_scene(k_prev))^2 (limited to MAX_WEIGHT) where mask and k_prev > 0."""
    ok = mask & (k_prev > 0)
    t = np.where(ok, k_new / np.where(ok, k_prev, 1.0), 0.0)
    t = np.clip(t, 0.0, MAX_MULT)
    w = np.zeros_like(k_prev)
    for a, b in zip(offsets[:-1], offsets[1:]):
        sel = ok[a:b]
        if not sel.any():
            continue
        kp = k_prev[a:b]
        s2 = np.mean(kp[sel] ** 2)
        w[a:b][sel] = np.minimum(kp[sel] ** 2 / s2, MAX_WEIGHT)
    return t.astype(np.float32), w.astype(np.float32)


def collect(scene_list, steps=80, warmup=10, stride=4, frac=0.25, seed=0, log=None):
    """(X, T, W) from plain-solver runs of the scenes, batched per parameter block:
    X n x 10 features, T n x 2 multiplier targets (divergence, pressure), W n x 2 weights."""
    rng = np.random.default_rng(seed)
    xs, ts_, ws = [], [], []
    for group in _group_by_params(scene_list):
        b = BatchedTimeStepDFSPH(group, use_graph=True)
        b.ctx.set_feature_output(True)
        off = b.offsets
        kp_prev = b.ctx.download("p / rho^2", np.float64)
        kv_prev = b.ctx.download("p_v / rho^2", np.float64)
        t0 = time.time()
        for k in range(warmup + steps):
            b.step()
            kp = b.ctx.download("p / rho^2", np.float64)
            kv = b.ctx.download("p_v / rho^2", np.float64)
            if k >= warmup and (k - warmup) % stride == 0:
                X = b.ctx.download("features", np.float32)
                dadv = b.ctx.download("advected density", np.float64)
                # classic warm starts are non-zero only where these masks hold
                mask_v = (X[:, 1] > 0) & (X[:, 2] >= -0.5)
                mask_p = dadv > 1.0
                tv, wv = targets(kv_prev, kv, mask_v, off)
                tp, wp = targets(kp_prev, kp, mask_p, off)
                pick = (rng.uniform(size=X.shape[0]) < frac) & ((wv > 0) | (wp > 0))
                xs.append(X[pick])
                ts_.append(np.stack([tv[pick], tp[pick]], 1))
                ws.append(np.stack([wv[pick], wp[pick]], 1))
            kp_prev, kv_prev = kp, kv
        if log is not None:
            log.append({"scenes": len(group), "particles": int(off[-1]), "steps": warmup + steps,
                        "seconds": time.time() - t0})
        b.close()
    return np.concatenate(xs), np.concatenate(ts_), np.concatenate(ws)


def train(X, T, W, epochs=40, lr=1e-3, batch=2048, seed=1):
    net = native.Mlp(seed=seed)
    net.set_output_scale(SCALE_V, SCALE_P)
    losses = net.train(X, T, W, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, losses


def save(net, path=WEIGHTS):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    sv, sp = net.output_scale()
    np.savez(path, params=net.params(), scale_v=sv, scale_p=sp)


def load(path=WEIGHTS, device=0):
    d = np.load(path)
    net = native.Mlp(device=device)
    net.set_params(d["params"])
    net.set_output_scale(float(d["scale_v"]), float(d["scale_p"]))
    return net


def run(scene, steps, net=None, warmup=0, use_graph=True, gate=(0, 0)):
    """Advance `scene` with the classic warm start (net=None) or the network (with the given
    per-solver gate, sphgb_set_warmstart_gate); per-step stats and device time per step
    (CUDA events on the library stream)."""
    import torch

    ts = TimeStepDFSPH(scene, use_graph=use_graph)
    if net is not None:
        ts.ctx.set_warmstart_mlp(net)
        ts.ctx.set_warmstart_gate(*gate)
    ext = torch.cuda.ExternalStream(ts.ctx.stream())
    for _ in range(warmup):
        ts.step()
    stats, times = [], []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            a.record(ext)
        st = ts.step()
        with torch.cuda.stream(ext):
            b.record(ext)
        stats.append(st)
        times.append((a, b))
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in times]
    rho = ts.getFluidModel().getFieldBuffer("density")
    ts.close()
    return stats, ms, rho


def summarize(stats, ms, rho, rho0=1000.0, gate=None):
    """Per-run summary.  gate = (divergence, pressure) Jacobi sweeps that the network's warm-start
    selection runs for both candidates, or None for the classic warm start: the losing
    candidate's sweeps are work the GPU did, and `solver_iterations_total_booked` adds them
    (gate sweeps per gated solve) to the iterations of the solves themselves."""
    it = np.array([[s["iterations"], s["iterations_v"]] for s in stats], float)
    used = np.array([s["learned_used"] for s in stats])
    rc = np.array([s["ws_residual_classic"] for s in stats], float)
    rl = np.array([s["ws_residual_learned"] for s in stats], float)
    ratio = np.where(rc > 0, rl / np.maximum(rc, 1e-300), 1.0)
    return {
        "gate_error_ratio_learned_over_classic_median": [float(np.median(ratio[:, 0])),
                                                                float(np.median(ratio[:, 1]))],
        "pressure_iterations_mean": float(it[:, 0].mean()),
        "divergence_iterations_mean": float(it[:, 1].mean()),
        "solver_iterations_total": float(it.sum()),
        "solver_iterations_total_booked": float(it.sum() + (0 if gate is None else len(stats) * (gate[0] + gate[1]))),
        "gate_sweeps": None if gate is None else list(gate),
        "ms_per_step": float(np.mean(ms)),
        "final_avg_density_error_percent": float(stats[-1]["avg_density_err"] / rho0 * 100.0),
        "max_avg_density_error_percent": float(max(s["avg_density_err"] for s in stats) / rho0 * 100.0),
        "learned_used_div_fraction": float(np.mean((used & 1) > 0)),
        "learned_used_pressure_fraction": float(np.mean((used & 2) > 0)),
        "final_density_max": float(rho.max()),
    }


def _gain(plain, learned):
    return {
        "iteration_reduction": 1.0 - learned["solver_iterations_total"] / max(plain["solver_iterations_total"], 1.0),
        "iteration_reduction_booked": 1.0 - learned["solver_iterations_total_booked"] /
        max(plain["solver_iterations_total_booked"], 1.0),
        "time_per_step_reduction": 1.0 - learned["ms_per_step"] / plain["ms_per_step"],
    }


def default_gate(params):
    """The gate sweeps sphgb_set_warmstart_gate(0, 0) selects: 1 for the divergence solve,
    max(minIterations, 4) for the pressure solve, never more than the solvers' caps."""
    return (min(1, params.maxIterationsV) if params.enableDivergenceSolver else 0,
            min(max(4, params.minIterations), params.maxIterations))


def evaluate(scene, net, steps=300, warmup=0, strict=True):
    """Plain vs learned (default gate); with strict=True also the learned warm start judged
    by the candidates' initial residuals alone (gate 1 for both solvers)."""
    sp, mp, rp = run(scene, steps, None, warmup)
    sl, ml, rl = run(scene, steps, net, warmup)
    plain, learned = summarize(sp, mp, rp), summarize(sl, ml, rl, gate=default_gate(scene.params))
    out = {"plain": plain, "learned": learned, "gain": _gain(plain, learned)}
    if strict:
        ss, ms, rs = run(scene, steps, net, warmup, gate=(1, 1))
        strict_gate = (1 if scene.params.enableDivergenceSolver else 0, 1)
        out["learned_initial_residual_gate"] = summarize(ss, ms, rs, gate=strict_gate)
        out["gain_initial_residual_gate"] = _gain(plain, out["learned_initial_residual_gate"])
    return out


def training_scenes(num_ensemble=256, settling=3):
    """The ensemble of independent dam breaks (r = 0.025) and small settling columns around a
    sphere (r = 0.01, the evaluation scene's kind with other seeds and proportions)."""
    ens = scenes.ensemble(num_scenes=num_ensemble)
    settle = [scenes.settling_sphere(counts=c, box=b, sphere_radius=r, seed=2000 + k)
              for k, (c, b, r) in enumerate([((48, 48, 48), (2.4, 1.6, 2.4), 0.4), ((64, 56, 64), (3.0, 2.0, 3.0), 0.5),
                                             ((40, 64, 56), (2.2, 2.0, 2.6), 0.45)][:settling])]
    return ens, settle


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None, help="directory for the report (weights go to the package data dir)")
    ap.add_argument("--ensemble", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=1000)
    ap.add_argument("--ensemble-stride", type=int, default=10)
    ap.add_argument("--ensemble-frac", type=float, default=0.01)
    ap.add_argument("--settling", type=int, default=3)
    ap.add_argument("--settling-steps", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--eval-steps", type=int, default=300)
    ap.add_argument("--eval-scene", default="learned_2m")
    args = ap.parse_args()
    t0 = time.time()
    ens, settle = training_scenes(args.ensemble, args.settling)
    log = []
    X1, T1, W1 = collect(ens, steps=args.ensemble_steps, warmup=10, stride=args.ensemble_stride,
                         frac=args.ensemble_frac, seed=0, log=log)
    X2, T2, W2 = collect(settle, steps=args.settling_steps, warmup=10, stride=4, frac=0.2, seed=1, log=log)
    X, T, W = np.concatenate([X1, X2]), np.concatenate([T1, T2]), np.concatenate([W1, W2])
    t_collect = time.time() - t0
    net, losses = train(X, T, W, epochs=args.epochs)
    t_train = time.time() - t0 - t_collect
    save(net)
    sc = scenes.learned_2m() if args.eval_scene == "learned_2m" else scenes.dambreak_1m()
    res = evaluate(sc, net, steps=args.eval_steps)
    report = {"training": {"batches": log, "samples": int(X.shape[0]), "samples_ensemble": int(X1.shape[0]),
                           "samples_settling": int(X2.shape[0]), "epochs": args.epochs,
                           "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
                           "collect_s": t_collect, "train_s": t_train},
              "evaluation_scene": f"{sc.name}: {sc.n} fluid + {sc.nb} boundary", **res}
    print(json.dumps(report, indent=1))
    if args.out:
        os.makedirs(args.out, exist_ok=True)
        with open(os.path.join(args.out, "learned_warmstart.json"), "w") as f:
            json.dump(report, f, indent=1)


if __name__ == "__main__":
    main()
