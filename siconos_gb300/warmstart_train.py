"""Train the learned warm start on solutions the GPU solver generates.

    python -m siconos_gb300.warmstart_train --scenes 2000 --out siconos_gb300/data/warmstart_mlp.npz

Training pairs (features -> reaction) come from the lattice generator with
dims drawn uniformly in [lo, hi]^3 and mu ~ U(0.1, 0.9) per scene.  Each
scene gives two solves, one scene at a time on the whole GPU:
  step 0  from r = 0 (the previous-reaction features are 0),
  step 1  after a velocity random-walk step (v0 += N(0, 0.01^2) per degree
          of freedom, contacts kept), warm-started from step 0's reaction
          (which becomes the previous-reaction features).
Solves use the FP32 sweeps + FP64 polish to the tolerance `tol` (default
1e-3, the tolerance the time-stepping and benchmark solves work to) within
1,500 sweeps, and only scenes whose FP64 fc3d_compute_error reached it give
pairs.  With --residual the targets are the change of the reaction from the
previous-step reaction (features 13-15; zero on a first step), and the warm
start adds the output to that reaction.  Up to `per_scene` contacts per scene
and step are kept, so large scenes do not dominate.  The network is then
trained with Adam on the GPU (minibatches of 4096, cosine learning-rate
decay) and saved with its statistics and training record.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from .device import DeviceSolver
from .learned import WarmStartMLP, host_features, init_params, make_stats
from .scene import lattice


def generate(n_scenes: int, seed: int = 1000, lo=(5, 5, 5), hi=(30, 30, 30), per_scene: int = 2048,
             max_iter: int = 1500, walk_std: float = 0.01, device: int = 0, log=None, tol: float = 1e-3,
             residual: bool = False, log_every: int = 100):
    """Training pairs from solves of one scene at a time on the whole GPU (the
    dataflow FP32 sweep, then the FP64 check and polish): a batched launch
    gives each scene one block, and the FP64 polish of a scene of tens of
    thousands of contacts on one block takes seconds a sweep."""
    rng = np.random.default_rng(seed)
    Xs, Ts = [], []
    summary = {"scenes": 0, "contacts": 0, "solves": 0, "sweeps": 0, "errors_step0": [], "errors_step1": [],
               "kept_step0": 0, "kept_step1": 0}
    d = DeviceSolver(device)
    d.autotune(0)  # one structure per scene: the dataflow sweep's defaults, untimed
    kw = dict(tol=tol, max_iter=max_iter)
    try:
        for k in range(n_scenes):
            dims = [int(v) for v in rng.integers(lo, np.asarray(hi) + 1)]
            sc = lattice(*dims, seed=seed * 1000003 + k, mu=float(rng.uniform(0.1, 0.9)))
            d.load(sc)
            o1 = d.solve(**kw)
            r1, _ = d.get()
            if o1["info"] == 0:  # FP64 error at most tol: the solve gives pairs
                X = host_features(sc.nc, sc.rowptr, sc.colidx, sc.blocks, sc.q, sc.mu, None, sc.gap)
                sel = rng.permutation(sc.nc)[:per_scene]
                Xs.append(X[sel])
                Ts.append(r1.reshape(-1, 3)[sel].astype(np.float32))
                summary["kept_step0"] += 1
            sc.perturb(seed * 7919 + k, walk_std)
            d.set_q_mu(sc.q, sc.mu)
            d.set_r(r1)
            o2 = d.solve(**kw)
            r2, _ = d.get()
            if o1["info"] == 0 and o2["info"] == 0:
                X = host_features(sc.nc, sc.rowptr, sc.colidx, sc.blocks, sc.q, sc.mu, r1, sc.gap)
                sel = rng.permutation(sc.nc)[:per_scene]
                Xs.append(X[sel])
                t = r2.reshape(-1, 3)[sel] - (r1.reshape(-1, 3)[sel] if residual else 0.0)
                Ts.append(t.astype(np.float32))
                summary["kept_step1"] += 1
            summary["scenes"] += 1
            summary["contacts"] += sc.nc
            summary["solves"] += 2
            summary["sweeps"] += o1["sweeps32"] + o1["sweeps64"] + o2["sweeps32"] + o2["sweeps64"]
            summary["errors_step0"].append(o1["error"])
            summary["errors_step1"].append(o2["error"])
            if log and (k + 1) % log_every == 0:
                log({"scenes": summary["scenes"], "samples": int(sum(len(x) for x in Xs)),
                     "kept_step0": summary["kept_step0"], "kept_step1": summary["kept_step1"]})
            del sc
    finally:
        d.close()
    X = np.concatenate(Xs)
    T = np.concatenate(Ts)
    for key in ("errors_step0", "errors_step1"):
        e = np.asarray(summary.pop(key))
        summary[key.replace("errors", "median_error")] = float(np.median(e))
        summary[key.replace("errors", "max_error")] = float(e.max())
    return X, T, summary


def train(X, T, epochs: int = 20, batch: int = 4096, lr: float = 2e-3, wd: float = 1e-4, seed: int = 0,
          device: int = 0, log=None, residual: bool = False):
    rng = np.random.default_rng(seed)
    val = rng.choice(len(X), max(1, len(X) // 50), replace=False)
    m = WarmStartMLP(device)
    m.residual(residual)
    m.set_params(init_params(seed), make_stats(X, T))
    m.set_data(X, T)
    t = time.perf_counter()
    hist = m.train(epochs, batch=batch, lr=lr, wd=wd, seed=seed, val_idx=val, log=log)
    return m, hist, time.perf_counter() - t


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--lo", type=int, default=5)
    ap.add_argument("--hi", type=int, default=30)
    ap.add_argument("--per-scene", type=int, default=2048)
    ap.add_argument("--max-iter", type=int, default=1500)
    ap.add_argument("--tol", type=float, default=1e-3)
    ap.add_argument("--residual", action="store_true", help="targets: change of the reaction from the previous step")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)

    def log(row):
        print(json.dumps(row), flush=True)

    t0 = time.perf_counter()
    X, T, summary = generate(a.scenes, a.seed, (a.lo,) * 3, (a.hi,) * 3, a.per_scene, a.max_iter, log=log,
                             tol=a.tol, residual=a.residual)
    t_gen = time.perf_counter() - t0
    m, hist, t_train = train(X, T, a.epochs, a.batch, a.lr, log=log, residual=a.residual)
    cfg = dict({k: v for k, v in vars(a).items() if k != "out"}, samples=len(X), generate_s=t_gen,
               train_s=t_train, **summary)
    log({"config": cfg, "final": hist[-1]})
    if a.out:
        m.save(a.out, config=json.dumps(cfg), history=json.dumps(hist))
    m.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
