"""Train the point-cloud warm-start network on solves of the plain method.

    python -m electrodrive_gb300.train_warm_start --out weights.npz [--train 320] [--test 64]

Data: random spheres, ellipsoids (semi-axes U[0.5, 2]), tori (R U[0.8, 1.5],
r/R U[0.15, 0.45]) and sphere dimers (radii U[0.5, 1.5], gap U[0.1, 1]),
each with a random potential per conductor and a point charge q U[-1, 1]
outside it, meshed with ``--panels`` panels and solved by the plain method
(dense FP64 operator, Jacobi GMRES to 1e-10).  Training and held-out sets
use disjoint seeds.  Training runs the library's own forward, backward and
Adam kernels on the GPU, one geometry per step.  The held-out report gives
GMRES iterations and time to a 1e-6 true residual from the cold start
(b / I_self), the base guess (b / A(1)) and the learned start.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--report", default=None)
    ap.add_argument("--train", type=int, default=320)
    ap.add_argument("--test", type=int, default=64)
    ap.add_argument("--panels", default="1500:6000")
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)

    from .core.warm_start import KINDS, PointCloudNet, compare_starts, make_sample, random_case, train

    lo, hi = (int(x) for x in args.panels.split(":"))
    t0 = time.perf_counter()

    def build(n, seed):
        rng = np.random.default_rng(seed)
        out = []
        for i in range(n):
            out.append(make_sample(*random_case(rng, KINDS[i % len(KINDS)], int(rng.integers(lo, hi + 1)))))
        return out

    train_set = build(args.train, 1000 + args.seed)
    test_set = build(args.test, 2000 + args.seed)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = PointCloudNet(seed=args.seed)
    t1 = time.perf_counter()
    hist = train(net, train_set, epochs=args.epochs, lr=args.lr, seed=args.seed, log_every=10)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    evals = [compare_starts(net, s) for s in test_set]
    summary = {}
    for k in ("cold", "base", "learned"):
        summary[k] = {"mean_iters": float(np.mean([e[k]["iters"] for e in evals])),
                      "mean_seconds": float(np.mean([e[k]["seconds"] for e in evals])),
                      "mean_start_error": float(np.mean([e[k]["start_error"] for e in evals])),
                      "all_converged": bool(all(e[k]["code"] == 0 for e in evals))}
    report = {"train_geometries": args.train, "test_geometries": args.test, "panels": [lo, hi],
              "epochs": args.epochs, "lr": args.lr, "seconds_data": t_data, "seconds_train": t_train,
              "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1], "held_out": summary,
              "train_panels_total": int(sum(s["mesh"].n_panels for s in train_set))}
    net.save(args.out, loss_history=np.asarray(hist), report=json.dumps(report))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
