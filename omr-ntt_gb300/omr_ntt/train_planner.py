"""Collect autotuner timings, train the learned plan selector, report regret.

    python -m omr_ntt.train_planner --points 2000 --train 1500 --out DIR

Writes DIR/planner_dataset.npz (features, per-class median ms, exhaustive
best ms, the points), DIR/planner_mlp.npz (network parameters + metadata),
DIR/planner_mlp.bin (the weight file the library loads) and
prints one JSON summary: mean / median / p90 regret on the held-out points for
the network, for the built-in heuristic, and the share of points within 5%.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import planner as P


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=2000)
    ap.add_argument("--train", type=int, default=1500)
    ap.add_argument("--seed", type=int, default=2025)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data"))
    ap.add_argument("--dataset", default=None, help="reuse a collected dataset")
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    pts = P.planning_points(a.seed, a.points)
    t0 = time.time()
    if a.dataset:
        z = np.load(a.dataset)
        ds = {"X": z["X"], "T": z["T"], "best": z["best"]}
    else:
        ds = P.collect(pts, reps=a.reps, progress=100)
        np.savez_compressed(os.path.join(a.out, "planner_dataset.npz"), X=ds["X"], T=ds["T"].astype(np.float32),
                 best=ds["best"].astype(np.float32), points=json.dumps(pts))
    t_collect = time.time() - t0
    X, T, best = ds["X"], ds["T"].astype(np.float64), ds["best"].astype(np.float64)
    Y, M = P.targets(T)
    tr, te = slice(0, a.train), slice(a.train, len(pts))
    mlp = P.Mlp(seed=a.seed)
    t1 = time.time()
    hist = mlp.fit(X[tr], Y[tr], M[tr], epochs=a.epochs, batch=64, lr=a.lr, seed=a.seed)
    t_train = time.time() - t1
    pred = mlp.forward(X[te])
    ch = P.choose(pred, T[te])
    r_mlp = P.regret(T[te], best[te], ch)
    hc = np.array([P.heuristic_class(p) for p in pts[te]])
    r_heur = P.regret(T[te], best[te], hc)
    cb = np.nanmin(T[te], axis=1)
    r_classbest = cb / best[te] - 1.0

    def stats(r):
        return {"mean": float(np.mean(r)), "median": float(np.median(r)), "p90": float(np.quantile(r, 0.9)),
                "within_5pct": float(np.mean(r <= 0.05))}

    summary = {
        "points": len(pts), "train": a.train, "held_out": len(pts) - a.train,
        "classes": int(T.shape[1]), "mean_applicable_classes": float(np.isfinite(T).sum(1).mean()),
        "final_train_loss": float(hist[-1]), "collect_s": round(t_collect, 1), "train_s": round(t_train, 2),
        "regret_mlp": stats(r_mlp), "regret_heuristic": stats(r_heur),
        "regret_best_class": stats(r_classbest),
    }
    P.save_model(os.path.join(a.out, "planner_mlp.npz"), mlp,
                 {"seed": a.seed, "epochs": a.epochs, "lr": a.lr, "summary": summary})
    P.save_weight_file(os.path.join(a.out, "planner_mlp.bin"), mlp.params())
    print(json.dumps(summary), flush=True)


if __name__ == "__main__":
    main()
