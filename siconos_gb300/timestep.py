"""Time-stepping sequence on the GPU solver: consecutive FC3D solves of one
lattice with the contacts (and W) kept and q following a random walk
(v0 += N(0, walk_std^2) per degree of freedom between steps).

W is assembled and coloured once.  With `assembly="host"` the scene
generator forms each step's q on the host and uploads it; with
`assembly="device"` W and q are assembled on the GPU from the contact
geometry and the velocity random walk runs there too, so a step moves no
array between host and device.  Each step starts from the previous step's
reaction (`warm="previous"`), from the learned proposal with that reaction as
its fallback (`warm="learned"`), or from zero (`warm="zero"`).
`checker(scene, r, q)` (optional) is called on every `check_every`-th step
with the step's reaction and q, and its value is recorded as `check_error`,
e.g. an independent FP64 fc3d_compute_error.
"""
from __future__ import annotations

import time

import numpy as np

from .device import DeviceSolver
from .scene import lattice


def run_sequence(dims=(80, 80, 40), steps: int = 200, seed: int = 5, mu: float = 0.5, walk_std: float = 0.01,
                 tol: float = 1e-3, max_iter: int = 1000, warm: str = "learned", mlp=None, check_every: int = 10,
                 checker=None, device: int = 0, log=None, assembly: str = "host", h: float = 1e-3):
    if warm not in ("learned", "previous", "zero"):
        raise ValueError(f"unknown warm start {warm!r}")
    if assembly not in ("host", "device"):
        raise ValueError(f"unknown assembly {assembly!r}")
    if warm == "learned" and mlp is None:
        raise ValueError("the learned warm start needs a trained network")
    from .learned import warm_start
    sc = lattice(*dims, seed=seed, mu=mu)
    d = DeviceSolver(device)
    recs = []
    try:
        if assembly == "device":
            geo = sc.contacts()
            d.set_contacts(geo)
            d.set_mu(sc.mu)
            d.set_velocities(geo["vel"], h)
            d.zero_r()
        else:
            d.load(sc)
        d.solve(tol=tol, max_iter=2)  # kernels loaded, launch shape tuned
        d.zero_r()
        for k in range(steps):
            t0 = time.perf_counter()
            if k > 0:
                if assembly == "device":
                    d.random_walk(seed * 7919 + k, walk_std)
                else:
                    sc.perturb(seed * 7919 + k, walk_std)
                    d.set_q_mu(sc.q, sc.mu)
            t1 = time.perf_counter()
            if warm == "zero":
                d.zero_r()
            ws = warm_start(d, mlp, sc.gap) if warm == "learned" else None
            t2 = time.perf_counter()
            st = d.solve(tol=tol, max_iter=max_iter)
            t3 = time.perf_counter()
            rec = {"step": k, "info": st["info"], "sweeps32": st["sweeps32"], "sweeps64": st["sweeps64"],
                   "error": st["error"], "solve_ms": st["ms_total"], "q_update_ms": 1e3 * (t1 - t0),
                   "warm_ms": 1e3 * (t2 - t1), "wall_ms": 1e3 * (t3 - t0)}
            if ws is not None:
                rec["proposal_taken"] = ws["taken"]
                rec["error_fallback"] = ws["error_fallback"]
                rec["error_proposal"] = ws["error_proposal"]
            if checker is not None and k % check_every == 0:
                r, _ = d.get()
                q = d.get_q() if assembly == "device" else sc.q
                rec["check_error"] = float(checker(sc, r, q))
            recs.append(rec)
            if log:
                log(rec)
    finally:
        d.close()
    return {"scene": {"dims": list(dims), "seed": seed, "contacts": sc.nc, "blocks": sc.nnzb}, "steps": recs}


def summarise(run: dict) -> dict:
    s = run["steps"]
    sw = np.array([r["sweeps32"] + r["sweeps64"] for r in s])
    out = {"steps": len(s), "converged": int(sum(r["info"] == 0 for r in s)), "sweeps_mean": float(sw.mean()),
           "sweeps_max": int(sw.max()), "solve_ms_mean": float(np.mean([r["solve_ms"] for r in s])),
           "wall_ms_mean": float(np.mean([r["wall_ms"] for r in s])),
           "error_max": float(max(r["error"] for r in s))}
    if any("proposal_taken" in r for r in s):
        out["proposals_taken"] = int(sum(r.get("proposal_taken", False) for r in s))
    chk = [(r["error"], r["check_error"]) for r in s if "check_error" in r]
    if chk:
        out["checked_steps"] = len(chk)
        out["check_rel_diff_max"] = float(max(abs(a - b) / max(abs(b), 1e-300) for a, b in chk))
    return out
