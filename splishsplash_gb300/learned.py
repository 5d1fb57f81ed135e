"""Learned warm start: data collection, training and evaluation.

Pipeline (all GPU work goes through libsphgb300.so):
  1. collect(): run the plain solver (classic warm start) on independent dam breaks of
     the ensemble configuration and record, per step, each particle's network inputs at
     the start of the step (SPHGB_FIELD_FEATURES) and the converged, stored warm starts
     after it (kappa_v*dt and kappa*dt^2, the "p_v / rho^2" and "p / rho^2" fields)
     divided by the output scales.
  2. train(): Adam (lr 1e-3) with the library's own BF16 tensor-core forward and
     FP32 backward kernels.
  3. evaluate(): the same scene with the classic warm start and with the network
     (which is used per solver and step only where it lowers the initial residual);
     both iterate to the same tolerances.  Reports iterations, device time per step
     and the final average density error.

    python -m splishsplash_gb300.learned --out <dir>   # full pipeline, writes weights + report
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import native, scenes
from .dfsph import TimeStepDFSPH

SCALE_V = 1.0e-2   # kMlpDefaultScaleV: output 0 x SCALE_V = stored kappa_v * dt
SCALE_P = 1.0e-4   # kMlpDefaultScaleP: output 1 x SCALE_P = stored kappa * dt^2
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart_mlp.npz")


def collect(scene_list, steps=80, warmup=10, stride=4, frac=0.25, seed=0):
    """(X, Y) pairs from plain-solver runs: X n x 10 features, Y n x 2 scaled targets."""
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    for sc in scene_list:
        ts = TimeStepDFSPH(sc, use_graph=True)
        ts.ctx.set_feature_output(True)
        for k in range(warmup + steps):
            ts.step()
            if k < warmup or (k - warmup) % stride:
                continue
            X = ts.ctx.download("features", np.float32)
            kv = ts.ctx.download("p_v / rho^2", np.float32)
            kp = ts.ctx.download("p / rho^2", np.float32)
            pick = rng.uniform(size=X.shape[0]) < frac
            xs.append(X[pick])
            ys.append(np.stack([kv[pick] / SCALE_V, kp[pick] / SCALE_P], 1))
        ts.close()
    return np.concatenate(xs).astype(np.float32), np.concatenate(ys).astype(np.float32)


def train(X, Y, epochs=40, lr=1e-3, batch=2048, seed=1):
    net = native.Mlp(seed=seed)
    net.set_output_scale(SCALE_V, SCALE_P)
    losses = net.train(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)
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


def run(scene, steps, net=None, warmup=0, use_graph=True):
    """Advance `scene` with the classic warm start (net=None) or the network; per-step stats
    and device time per step (CUDA events on the library stream)."""
    import torch

    ts = TimeStepDFSPH(scene, use_graph=use_graph)
    if net is not None:
        ts.ctx.set_warmstart_mlp(net)
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


def summarize(stats, ms, rho, rho0=1000.0):
    it = np.array([[s["iterations"], s["iterations_v"]] for s in stats], float)
    used = np.array([s["learned_used"] for s in stats])
    rc = np.array([s["ws_residual_classic"] for s in stats], float)
    rl = np.array([s["ws_residual_learned"] for s in stats], float)
    ratio = np.where(rc > 0, rl / np.maximum(rc, 1e-300), 1.0)
    return {
        "initial_residual_ratio_learned_over_classic_median": [float(np.median(ratio[:, 0])),
                                                                float(np.median(ratio[:, 1]))],
        "pressure_iterations_mean": float(it[:, 0].mean()),
        "divergence_iterations_mean": float(it[:, 1].mean()),
        "solver_iterations_total": float(it.sum()),
        "ms_per_step": float(np.mean(ms)),
        "final_avg_density_error_percent": float(stats[-1]["avg_density_err"] / rho0 * 100.0),
        "max_avg_density_error_percent": float(max(s["avg_density_err"] for s in stats) / rho0 * 100.0),
        "learned_used_div_fraction": float(np.mean((used & 1) > 0)),
        "learned_used_pressure_fraction": float(np.mean((used & 2) > 0)),
        "final_density_max": float(rho.max()),
    }


def evaluate(scene, net, steps=300, warmup=0):
    sp, mp, rp = run(scene, steps, None, warmup)
    sl, ml, rl = run(scene, steps, net, warmup)
    plain, learned = summarize(sp, mp, rp), summarize(sl, ml, rl)
    gain = {
        "iteration_reduction": 1.0 - learned["solver_iterations_total"] / max(plain["solver_iterations_total"], 1.0),
        "time_per_step_reduction": 1.0 - learned["ms_per_step"] / plain["ms_per_step"],
    }
    return {"plain": plain, "learned": learned, "gain": gain}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None, help="directory for the report (weights go to the package data dir)")
    ap.add_argument("--scenes", type=int, default=12)
    ap.add_argument("--settling", type=int, default=3)
    ap.add_argument("--steps", type=int, default=120)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--eval-steps", type=int, default=300)
    ap.add_argument("--eval-scene", default="learned_2m")
    args = ap.parse_args()
    t0 = time.time()
    ens = scenes.ensemble(num_scenes=256)
    # ensemble dam breaks plus settling columns around a sphere (the evaluation scene's kind,
    # smaller and with other seeds and proportions)
    settle = [scenes.settling_sphere(counts=c, box=b, sphere_radius=r, seed=2000 + k)
              for k, (c, b, r) in enumerate([((48, 48, 48), (2.4, 1.6, 2.4), 0.4), ((64, 56, 64), (3.0, 2.0, 3.0), 0.5),
                                             ((40, 64, 56), (2.2, 2.0, 2.6), 0.45)][: args.settling])]
    train_scenes = ens[: args.scenes] + settle
    X, Y = collect(train_scenes, steps=args.steps)
    t_collect = time.time() - t0
    net, losses = train(X, Y, epochs=args.epochs)
    t_train = time.time() - t0 - t_collect
    save(net)
    sc = scenes.learned_2m() if args.eval_scene == "learned_2m" else scenes.dambreak_1m()
    res = evaluate(sc, net, steps=args.eval_steps)
    report = {"training": {"scenes": [s.name for s in train_scenes], "samples": int(X.shape[0]), "epochs": args.epochs,
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
