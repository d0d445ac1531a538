#!/usr/bin/env python3
"""Train the warm-start MLP of the batched solver on converged solutions.

For each training scene (the 60-tree forest family at a new seed, with a
random sun, random leaf/soil optics ramps and random sky/beam levels) the
hemisphere view-factor graph is built, the 64-band system is solved to
convergence in FP64, and facetcu_mlp_samples_device turns the solution into
one sample per facet side: 12 features from the first Jacobi sweep and the
local geometry, 64 targets (B - B1) / (sky + beam) per band.  All samples
stay on the device; facetcu_mlp_train_device runs Adam over them.

The trained weights are then evaluated on unseen seeds against the cold
start: iterations to the stop rule and the final error against FP64.

    python -m streamsim_gb300.train_mlp --scenes 40 --eval 10 --out weights.npy
"""
import argparse
import json
import time

import numpy as np


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--scenes", type=int, default=40)
    p.add_argument("--eval", type=int, default=10)
    p.add_argument("--steps", type=int, default=20000)
    p.add_argument("--batch", type=int, default=65536)
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--rays", type=int, default=512)
    p.add_argument("--top-k", type=int, default=256)
    p.add_argument("--tolerance", type=float, default=1e-6)
    p.add_argument("--small", action="store_true", help="config-1 scenes (2,048 leaves)")
    p.add_argument("--out", default=None, help="where to write the weights (.npy)")
    p.add_argument("--report", default=None, help="where to write the evaluation (.json)")
    p.add_argument("--weights", default=None,
                   help="evaluate these weights (.npy) instead of training")
    return p.parse_args(argv)


def random_optics(rng):
    return dict(leaf=(rng.uniform(0.02, 0.08), rng.uniform(0.35, 0.55)),
                soil=(rng.uniform(0.08, 0.16), rng.uniform(0.20, 0.35)),
                leaf_tau_ratio=rng.uniform(0.3, 0.5), sky=rng.uniform(50.0, 200.0),
                beam=rng.uniform(400.0, 1000.0), zenith=rng.uniform(10.0, 60.0),
                azimuth=rng.uniform(0.0, 360.0))


def fixed_optics():
    """The benchmark's optics and sun."""
    return dict(leaf=(0.04, 0.48), soil=(0.12, 0.30), leaf_tau_ratio=0.4, sky=100.0, beam=800.0,
                zenith=30.0, azimuth=135.0)


def make_case(fc, scenes, seed, optics, args):
    """One scene with its view-factor graph and 64-band inputs (host arrays)."""
    sc = scenes.config1(seed=seed, leaves=2048, grid=32) if args.small else scenes.config2(seed)
    m = fc.FacetrtCuda()
    m.initialize(256, 256, 64)
    m.setGeometry(sc.vertices)
    uv, dirs = scenes.hemisphere_samples(args.rays, 32, seed=7)
    m.buildHemisphereGraph(uv, dirs, args.rays, args.top_k, 32)
    sun = scenes.sun_direction(optics["zenith"], optics["azimuth"])
    suv, _ = scenes.hemisphere_samples(256, 32, seed=8)
    lit = m.hemisphereSunlit(sun, suv, 256, 32)
    rho, tau = scenes.band_optics(sc, 64, optics["leaf"], optics["soil"], optics["leaf_tau_ratio"])
    case = dict(scene=sc, model=m, rho=rho, tau=tau,
                dgeo=scenes.direct_geometry(sc, lit, sun)[None, :],
                sky=np.full(64, optics["sky"], np.float32),
                beam=np.full(64, optics["beam"], np.float32))
    return case


def solve_truth(fc, case):
    truth, _ = case["model"].solveBatched(case["rho"], case["tau"], case["sky"], case["beam"],
                                          case["dgeo"], precision=fc.PRECISION_FP64,
                                          tolerance=1e-12, maximum_iterations=4000)
    return truth


def samples(fc, torch, case, truth):
    """Features and targets of one case, as device tensors."""
    S = case["scene"].surface_count
    dev = torch.device("cuda")
    t = {k: torch.from_numpy(np.ascontiguousarray(case[k])).to(dev)
         for k in ("rho", "tau", "sky", "beam", "dgeo")}
    conv = torch.from_numpy(truth).to(dev)
    x = torch.empty((S, fc.MLP_INPUTS), dtype=torch.float32, device=dev)
    y = torch.empty((S, fc.MLP_OUTPUTS), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    cfg = fc.BatchConfig(64, 1, fc.PRECISION_FP32, fc.WARM_NONE, 1, 0.0, 0, 0)
    case["model"].mlpSamplesDevice(cfg, t["rho"].data_ptr(), t["tau"].data_ptr(), None,
                                   t["sky"].data_ptr(), t["beam"].data_ptr(), t["dgeo"].data_ptr(),
                                   conv.data_ptr(), x.data_ptr(), y.data_ptr())
    return x, y


def evaluate(fc, case, truth, params, tolerance):
    """Cold vs MLP warm start on one case: iterations, seconds, error."""
    m = case["model"]
    m.mlpSetParameters(params)
    scale = np.maximum(np.abs(truth), 1e-6 * np.abs(truth).max())
    row = {}
    for name, warm in (("cold", fc.WARM_NONE), ("mlp", fc.WARM_MLP)):
        args = (case["rho"], case["tau"], case["sky"], case["beam"], case["dgeo"])
        m.solveBatched(*args, precision=fc.PRECISION_MIXED, tolerance=tolerance,
                       maximum_iterations=2000, warm_start=warm)
        out, res = m.solveBatched(*args, precision=fc.PRECISION_MIXED, tolerance=tolerance,
                                  maximum_iterations=2000, warm_start=warm)
        row[name] = dict(iterations=int(res["iterations"]), seconds=float(res["seconds"]),
                         max_rel_err=float(np.max(np.abs(out - truth) / scale)))
    return row


def evaluate_only(fc, scenes, args, params, rng):
    """Cold vs learned start on args.eval unseen seeds (the benchmark's
    optics on the first, random optics and suns on the rest)."""
    for _ in range(args.scenes):  # the optics draws of the training scenes
        random_optics(rng)
    rows = []
    for i in range(args.eval):
        optics = fixed_optics() if i == 0 else random_optics(rng)
        case = make_case(fc, scenes, 10000 + i, optics, args)
        truth = solve_truth(fc, case)
        row = evaluate(fc, case, truth, params, args.tolerance)
        row["seed"] = 10000 + i
        rows.append(row)
        case["model"].close()
    report = dict(evaluation=rows, tolerance=args.tolerance,
                  mean_iterations_cold=float(np.mean([r["cold"]["iterations"] for r in rows])),
                  mean_iterations_mlp=float(np.mean([r["mlp"]["iterations"] for r in rows])),
                  mean_ms_cold=float(np.mean([r["cold"]["seconds"] for r in rows]) * 1e3),
                  mean_ms_mlp=float(np.mean([r["mlp"]["seconds"] for r in rows]) * 1e3),
                  max_err_cold=float(max(r["cold"]["max_rel_err"] for r in rows)),
                  max_err_mlp=float(max(r["mlp"]["max_rel_err"] for r in rows)))
    print(json.dumps(report))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    return report


def main(argv=None):
    import torch

    from streamsim_gb300 import facetcu as fc
    from streamsim_gb300 import scenes

    args = parse(argv)
    rng = np.random.default_rng(20240)
    if args.weights:
        return evaluate_only(fc, scenes, args, np.load(args.weights), rng)
    xs, ys = [], []
    t0 = time.perf_counter()
    for i in range(args.scenes):
        case = make_case(fc, scenes, 100 + i, random_optics(rng), args)
        truth = solve_truth(fc, case)
        x, y = samples(fc, torch, case, truth)
        xs.append(x)
        ys.append(y)
        case["model"].close()
    X = torch.cat(xs)
    Y = torch.cat(ys)
    del xs, ys
    gen_s = time.perf_counter() - t0

    trainer = fc.FacetrtCuda()
    trainer.initialize(16, 16, 8)
    trainer.mlpReset(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = []
    chunk = max(1, args.steps // 10)
    done = 0
    while done < args.steps:
        k = min(chunk, args.steps - done)
        losses.append(trainer.mlpTrainDevice(X.data_ptr(), Y.data_ptr(), X.shape[0], k,
                                             args.batch, args.lr, 1 + done))
        done += k
    train_s = time.perf_counter() - t0
    params = trainer.mlpParameters()
    trainer.close()
    target_var = float(Y.var().item())
    n_samples = int(X.shape[0])
    del X, Y
    if args.out:
        np.save(args.out, params.astype(np.float32))

    rows = []
    for i in range(args.eval):
        optics = fixed_optics() if i == 0 else random_optics(rng)
        case = make_case(fc, scenes, 10000 + i, optics, args)
        truth = solve_truth(fc, case)
        row = evaluate(fc, case, truth, params, args.tolerance)
        row["seed"] = 10000 + i
        rows.append(row)
        case["model"].close()
    report = dict(training_scenes=args.scenes, samples=n_samples,
                  steps=args.steps, batch=args.batch, learning_rate=args.lr,
                  generation_s=gen_s, training_s=train_s, loss_curve=losses,
                  target_variance=target_var, evaluation=rows,
                  mean_iterations_cold=float(np.mean([r["cold"]["iterations"] for r in rows])),
                  mean_iterations_mlp=float(np.mean([r["mlp"]["iterations"] for r in rows])))
    print(json.dumps(report))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
