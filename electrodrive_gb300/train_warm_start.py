"""Train the point-cloud warm-start network on solves of the plain method.

    python -m electrodrive_gb300.train_warm_start --out weights.npz [--train 2000] [--test 100]

Data: random spheres, ellipsoids (semi-axes U[0.5, 2]), tori (R U[0.8, 1.5],
r/R U[0.15, 0.45]) and sphere dimers (radii U[0.5, 1.5], gap U[0.1, 1]),
each with a random potential per conductor and a point charge q U[-1, 1]
outside it, meshed with about ``--panels`` panels and solved to a 1e-10
relative residual (dense FP64 Jacobi GMRES up to 8,000 panels, the FP64 FMM
operator in two-float arithmetic refined around FP32 FMM GMRES above).
Training and held-out sets use disjoint seeds.  Training runs the library's
own forward, backward and Adam kernels on the GPU, one geometry per step.
The held-out report gives, for the cold start (b / I_self), the base guess
(b / A(1)) and the learned start: the start's error, Jacobi GMRES
iterations and time to a 1e-6 true residual, and the mixed FP32/FP64
refinement solve to 1e-6 (steps, time).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch


def summarize(evals):
    """Means over held-out geometries of compare_starts() results."""
    out = {}
    for k in evals[0]:
        e = [x[k] for x in evals]
        d = {"mean_iters": float(np.mean([r["iters"] for r in e])),
             "mean_seconds": float(np.mean([r["seconds"] for r in e])),
             "mean_start_error": float(np.mean([r["start_error"] for r in e])),
             "mean_start_seconds": float(np.mean([r["start_seconds"] for r in e])),
             "all_converged": bool(all(r["code"] == 0 for r in e))}
        if all("mixed" in r for r in e):
            d["mixed"] = {"mean_seconds": float(np.mean([r["mixed"]["seconds"] for r in e])),
                          "mean_outer": float(np.mean([r["mixed"]["outer"] for r in e])),
                          "mean_inner_iters": float(np.mean([r["mixed"]["inner_iters"] for r in e])),
                          "mean_fp64_matvecs": float(np.mean([r["mixed"]["fp64_matvecs"] for r in e])),
                          "all_converged": bool(all(r["mixed"]["code"] == 0 for r in e))}
        out[k] = d
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--report", default=None)
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--test", type=int, default=100)
    ap.add_argument("--panels", default="10000:50000")
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--init", default=None, help="start from these weights (fine-tuning)")
    args = ap.parse_args(argv)

    from .core.warm_start import KINDS, PointCloudNet, compare_starts, make_sample, random_case, train

    lo, hi = (int(x) for x in args.panels.split(":"))
    t0 = time.perf_counter()
    rng = np.random.default_rng(1000 + args.seed)
    train_set = []
    for i in range(args.train):
        mesh, spec = random_case(rng, KINDS[i % len(KINDS)], int(rng.integers(lo, hi + 1)))
        s = make_sample(mesh, spec, keep_ops=False, operator="fmm")
        s["mesh"] = None  # training reads the device copies only
        train_set.append(s)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = PointCloudNet.load(args.init) if args.init else PointCloudNet(seed=args.seed)
    t1 = time.perf_counter()
    hist = train(net, train_set, epochs=args.epochs, lr=args.lr, seed=args.seed, log_every=5)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    panels_total = int(sum(int(s["areas"].shape[0]) for s in train_set))
    del train_set
    evals = []
    rng = np.random.default_rng(2000 + args.seed)
    for i in range(args.test):
        mesh, spec = random_case(rng, KINDS[i % len(KINDS)], int(rng.integers(lo, hi + 1)))
        evals.append(compare_starts(net, make_sample(mesh, spec, operator="fmm")))
    report = {"train_geometries": args.train, "test_geometries": args.test, "panels": [lo, hi],
              "epochs": args.epochs, "lr": args.lr, "seconds_data": t_data, "seconds_train": t_train,
              "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1], "held_out": summarize(evals),
              "train_panels_total": panels_total}
    net.save(args.out, loss_history=np.asarray(hist), report=json.dumps(report))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
