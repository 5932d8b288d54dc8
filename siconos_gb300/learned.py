"""Learned warm start for the GPU NSGS solver (include/fc3dgpu_mlp.h).

A per-contact MLP (17 -> 128 -> 128 -> 128 -> 3, ReLU, BF16 weights, FP32
accumulation) proposes each contact's reaction in its local frame from its
diagonal Delassus block, q_i, mu_i, the previous-step reaction and the normal
gap.  Training, inference and the warm start itself run in the library's
CUDA kernels; this module holds the host side: parameter initialisation,
statistics, the training loop, training-set generation with the GPU solver
on the lattice generator, and the evaluation of what the proposal saves.

Plain NSGS stays the fallback and the arbiter: the context keeps its current
reaction (zero or the previous step's) whenever the proposal's
fc3d_compute_error is not smaller.
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

import numpy as np

from . import numerics as sn

NF, NO, NSTATS = 17, 3, 40
DATA = Path(__file__).resolve().parent / "data"
DEFAULT_WEIGHTS = DATA / "warmstart_mlp.npz"
_SHAPES = [(32, 128), (128, 128), (128, 128), (128, 16)]
_FAN_IN = [NF, 128, 128, 128]


def host_features(nc, rowptr, colidx, blocks, q, mu, r_prev=None, gap=None) -> np.ndarray:
    """The 17 features of every contact (float32, nc x 17), as the device
    forms them: diagonal block (column-major), q_i, mu_i, previous r_i, gap_i."""
    rowptr = np.asarray(rowptr, np.int64)
    colidx = np.asarray(colidx, np.int64)
    blocks = np.asarray(blocks, np.float64).reshape(-1, 9)
    rows = np.repeat(np.arange(nc), np.diff(rowptr))
    diag = np.full(nc, -1, np.int64)
    sel = np.nonzero(colidx == rows)[0]
    diag[rows[sel]] = sel
    if (diag < 0).any():
        raise ValueError("every contact needs its diagonal block")
    X = np.zeros((nc, NF), np.float32)
    X[:, 0:9] = blocks[diag].astype(np.float32)
    X[:, 9:12] = np.asarray(q, np.float64).reshape(nc, 3).astype(np.float32)
    X[:, 12] = np.asarray(mu, np.float64).astype(np.float32)
    if r_prev is not None:
        X[:, 13:16] = np.asarray(r_prev, np.float64).reshape(nc, 3).astype(np.float32)
    if gap is not None:
        X[:, 16] = np.asarray(gap, np.float64).astype(np.float32)
    return X


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights on the real fan-in, zero biases, padding zero."""
    g = np.random.default_rng(seed)
    parts = []
    for l, ((k, n), fan) in enumerate(zip(_SHAPES, _FAN_IN)):
        W = np.zeros((k, n), np.float32)
        kk = NF if l == 0 else k
        nn = NO if l == 3 else n
        W[:kk, :nn] = g.standard_normal((kk, nn)) * np.sqrt(2.0 / fan)
        parts += [W.reshape(-1), np.zeros(n, np.float32)]
    return np.concatenate(parts).astype(np.float32)


def make_stats(X, T) -> np.ndarray:
    """Feature and target mean / standard deviation (a constant column gets
    standard deviation 1)."""
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    sx = X.std(axis=0)
    st = T.std(axis=0)
    sx[sx < 1e-12] = 1.0
    st[st < 1e-12] = 1.0
    return np.concatenate([X.mean(axis=0), sx, T.mean(axis=0), st]).astype(np.float32)


class WarmStartMLP:
    """The network on one GPU (fc3dgpu_mlp)."""

    def __init__(self, device: int = 0):
        self.L = sn.lib()
        self.h = self.L.fc3dgpu_mlp_create(device)
        if not self.h:
            raise RuntimeError(sn.last_error())
        self.nparams = int(self.L.fc3dgpu_mlp_nparams())
        self.ndata = 0

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc}): {sn.last_error()}")

    def tensor_path(self, tcgen05: bool) -> bool:
        """Products on tcgen05 (True) or on the mma.sync reference path
        (False); returns the previous setting."""
        return bool(self.L.fc3dgpu_mlp_set_tensor_path(self.h, int(tcgen05)))

    def set_params(self, params, stats):
        params = np.ascontiguousarray(params, np.float32)
        stats = np.ascontiguousarray(stats, np.float32)
        assert params.size == self.nparams and stats.size == NSTATS
        self._check(self.L.fc3dgpu_mlp_set_params(self.h, params.ctypes.data, stats.ctypes.data), "set_params")

    def get_params(self):
        p = np.zeros(self.nparams, np.float32)
        s = np.zeros(NSTATS, np.float32)
        self._check(self.L.fc3dgpu_mlp_get_params(self.h, p.ctypes.data, s.ctypes.data), "get_params")
        return p, s

    def set_data(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        assert X.shape[1] == NF and T.shape[1] == NO and len(X) == len(T)
        self._check(self.L.fc3dgpu_mlp_set_data(self.h, len(X), X.ctypes.data, T.ctypes.data), "set_data")
        self.ndata = len(X)

    def grad(self, idx):
        """Gradient and loss on the samples idx (no update)."""
        idx = np.ascontiguousarray(idx, np.int32)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        self._check(self.L.fc3dgpu_mlp_train_step(self.h, len(idx), idx.ctypes.data, 0.0, 0.0, g.ctypes.data,
                                                  C.byref(loss), 0), "train_step")
        return g, float(loss.value)

    def step(self, idx, lr: float, wd: float = 0.0, want_loss: bool = True):
        idx = np.ascontiguousarray(idx, np.int32)
        loss = C.c_float()
        self._check(self.L.fc3dgpu_mlp_train_step(self.h, len(idx), idx.ctypes.data, lr, wd, None,
                                                  C.byref(loss) if want_loss else None, 1), "train_step")
        return float(loss.value) if want_loss else None

    def infer(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((len(X), NO), np.float32)
        self._check(self.L.fc3dgpu_mlp_infer(self.h, len(X), X.ctypes.data, Y.ctypes.data, 0), "infer")
        return Y

    def train(self, epochs: int, batch: int = 4096, lr: float = 2e-3, wd: float = 1e-4, seed: int = 0,
              val_idx=None, log=None):
        """Adam over shuffled minibatches with a cosine learning-rate decay.
        Returns the per-epoch mean training loss (and validation loss)."""
        g = np.random.default_rng(seed)
        n = self.ndata
        train = np.arange(n) if val_idx is None else np.setdiff1d(np.arange(n), val_idx)
        steps_per_epoch = max(1, len(train) // batch)
        total = epochs * steps_per_epoch
        hist = []
        k = 0
        for ep in range(epochs):
            perm = g.permutation(train)
            ls = []
            for s in range(steps_per_epoch):
                rate = lr * 0.5 * (1.0 + np.cos(np.pi * k / total))
                want = (s % 16) == 0
                l = self.step(perm[s * batch:(s + 1) * batch], rate, wd, want_loss=want)
                if want:
                    ls.append(l)
                k += 1
            row = {"epoch": ep, "train_loss": float(np.mean(ls))}
            if val_idx is not None:
                row["val_loss"] = self.loss(val_idx)
            hist.append(row)
            if log:
                log(row)
        return hist

    def loss(self, idx, chunk: int = 65536) -> float:
        tot, n = 0.0, 0
        for s in range(0, len(idx), chunk):
            part = np.asarray(idx[s:s + chunk])
            _, l = self.grad(part)
            tot += l * len(part)
            n += len(part)
        return tot / max(1, n)

    def residual(self, on: bool) -> bool:
        """Outputs are the change of the reaction (True) or the reaction
        (False); returns the previous setting."""
        return bool(self.L.fc3dgpu_mlp_set_residual(self.h, int(on)))

    def save(self, path, **meta):
        p, s = self.get_params()
        np.savez(path, params=p, stats=s, residual=np.int32(self.L.fc3dgpu_mlp_residual(self.h)), **meta)

    def load(self, path=DEFAULT_WEIGHTS):
        z = np.load(path)
        self.set_params(z["params"], z["stats"])
        self.residual(bool(int(z["residual"])) if "residual" in z.files else False)
        return {k: z[k] for k in z.files if k not in ("params", "stats", "residual")}

    def close(self):
        if getattr(self, "h", None):
            self.L.fc3dgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def warm_start(solver, mlp: WarmStartMLP, gap=None) -> dict:
    """Learned warm start of a DeviceSolver context (its current reaction is
    the fallback).  Returns the two initial errors and whether the proposal
    was taken."""
    out = np.zeros(3)
    g = None if gap is None else np.ascontiguousarray(gap, np.float64)
    rc = solver.L.fc3dgpu_ctx_warm_start(solver.ctx, mlp.h, None if g is None else g.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"warm start failed ({rc}): {sn.last_error()}")
    return {"error_fallback": float(out[0]), "error_proposal": float(out[1]), "taken": bool(out[2])}


def device_features(solver, gap=None) -> np.ndarray:
    X = np.zeros((solver.nc, NF), np.float32)
    g = None if gap is None else np.ascontiguousarray(gap, np.float64)
    rc = solver.L.fc3dgpu_ctx_features(solver.ctx, None if g is None else g.ctypes.data, X.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"features failed ({rc}): {sn.last_error()}")
    return X


def _timed_solve(solver, **kw):
    t = time.perf_counter()
    st = solver.solve(**kw)
    st["wall_ms"] = 1e3 * (time.perf_counter() - t)
    return st


def evaluate(mlp: WarmStartMLP, dims=(60, 60, 30), seed: int = 424242, mu: float = 0.5, tol: float = 1e-8,
             max_iter: int = 2000, walk_std: float = 0.01, device: int = 0, **solve_kw) -> dict:
    """Sweeps and time to `tol` (within `max_iter` sweeps) on a held-out
    lattice, per warm start:
      step 0 (fresh scene): zero start, learned start (fallback zero);
      step 1 (after one velocity random-walk step): zero start, previous-step
      start, learned start (fallback previous step).
    The learned rows include the warm start's own time (features,
    inference, two error evaluations)."""
    from .device import DeviceSolver
    from .scene import lattice
    sc = lattice(*dims, seed=seed, mu=mu)
    d = DeviceSolver(device)
    kw = dict(tol=tol, max_iter=max_iter, **solve_kw)
    out = {"scene": {"dims": list(dims), "seed": seed, "contacts": sc.nc, "blocks": sc.nnzb}, "tol": tol,
           "max_iter": max_iter}
    try:
        d.load(sc)
        d.solve(tol=tol, max_iter=2)  # warm the kernels and the autotuned launch shape
        res = {}
        d.zero_r()
        res["zero"] = _timed_solve(d, **kw)
        r0, _ = d.get()
        d.zero_r()
        t = time.perf_counter()
        ws = warm_start(d, mlp, sc.gap)
        t_ws = 1e3 * (time.perf_counter() - t)
        st = _timed_solve(d, **kw)
        st.update(ws, warm_start_ms=t_ws)
        st["wall_ms"] += t_ws
        res["learned"] = st
        out["step0"] = res
        sc.perturb(seed + 1, walk_std)
        d.set_q_mu(sc.q, sc.mu)
        res = {}
        d.zero_r()
        res["zero"] = _timed_solve(d, **kw)
        d.set_r(r0)
        res["previous"] = _timed_solve(d, **kw)
        d.set_r(r0)
        t = time.perf_counter()
        ws = warm_start(d, mlp, sc.gap)
        t_ws = 1e3 * (time.perf_counter() - t)
        st = _timed_solve(d, **kw)
        st.update(ws, warm_start_ms=t_ws)
        st["wall_ms"] += t_ws
        res["learned"] = st
        out["step1"] = res
    finally:
        d.close()
    return out
