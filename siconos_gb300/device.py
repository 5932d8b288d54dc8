"""Device-resident solver handle over the ``fc3dgpu_ctx_*`` C-ABI: upload a
problem once, solve many times with inputs already in HBM."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import numerics as sn


class DeviceSolver:
    def __init__(self, device: int = 0):
        self.L = sn.lib()
        self.ctx = self.L.fc3dgpu_ctx_create(device)
        if not self.ctx:
            raise RuntimeError("fc3dgpu_ctx_create failed: " + sn.last_error())
        self.nc = 0

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc}): {sn.last_error()}")

    def set_W(self, nc, rowptr, colidx, blocks, colouring: int = sn.FC3DGPU_COLOURING_DEFAULT):
        self._check(self.L.fc3dgpu_ctx_set_W(self.ctx, nc, np.ascontiguousarray(rowptr, np.int64),
                                             np.ascontiguousarray(colidx, np.int64),
                                             np.ascontiguousarray(blocks, np.float64).reshape(-1), colouring),
                    "set_W")
        self.nc = nc

    def set_q_mu(self, q, mu):
        self._check(self.L.fc3dgpu_ctx_set_q_mu(self.ctx, np.ascontiguousarray(q, np.float64),
                                                np.ascontiguousarray(mu, np.float64)), "set_q_mu")

    def set_r(self, r):
        self._check(self.L.fc3dgpu_ctx_set_r(self.ctx, np.ascontiguousarray(r, np.float64)), "set_r")

    def load(self, scene, colouring: int = sn.FC3DGPU_COLOURING_DEFAULT, r0=None):
        self.set_W(scene.nc, scene.rowptr, scene.colidx, scene.blocks, colouring)
        self.set_q_mu(scene.q, scene.mu)
        self.set_r(np.zeros(3 * scene.nc) if r0 is None else r0)

    @staticmethod
    def params(**kw) -> sn.FC3DGPUParams:
        p = sn.FC3DGPUParams()
        sn.lib().fc3dgpu_params_default(C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def solve(self, **kw) -> dict:
        p = self.params(**kw)
        st = sn.FC3DGPUStats()
        rc = self.L.fc3dgpu_ctx_solve(self.ctx, C.byref(p), C.byref(st))
        self._check(rc, "solve")
        return st.as_dict()

    def timeline(self, sweep: int = 0, cap: int = 1 << 20):
        """Arm the phase timeline for `sweep` of the next solves and return
        the previous record as an array (colour, block, [start, end])."""
        out = np.zeros(cap, np.uint64)
        n = self.L.fc3dgpu_ctx_timeline(self.ctx, sweep, out.ctypes.data, cap)
        return out[:max(n, 0)]

    def sync(self, neighbourhood: bool) -> bool:
        """Neighbourhood (True) or grid-wide (False) synchronisation between
        colours; returns the previous setting."""
        return bool(self.L.fc3dgpu_ctx_sync(self.ctx, int(neighbourhood)))

    def staging(self, on: bool) -> bool:
        return bool(self.L.fc3dgpu_ctx_staging(self.ctx, int(on)))

    def spin_limit(self, polls: int) -> int:
        """Polls before a device wait gives up (0 = default); returns the
        previous setting."""
        return int(self.L.fc3dgpu_ctx_spin_limit(self.ctx, polls))

    def flow(self, on: bool) -> bool:
        """Slab-dataflow FP32 sweeps (True) or the coloured kernel (False);
        returns the previous setting."""
        return bool(self.L.fc3dgpu_ctx_flow(self.ctx, int(on)))

    def flow_warps(self, nw: int) -> int:
        """Warps per block of the dataflow sweep (8, 10, 12; 0 = default);
        returns the previous request."""
        rc = int(self.L.fc3dgpu_ctx_flow_warps(self.ctx, nw))
        if rc < 0:
            raise RuntimeError(sn.last_error())
        return rc

    def autotune(self, mode: int) -> int:
        """Autotuner mode (0 off, 1 result-preserving variants, 2 all);
        returns the previous mode."""
        rc = int(self.L.fc3dgpu_ctx_autotune(self.ctx, mode))
        if rc < 0:
            raise RuntimeError(sn.last_error())
        return rc

    def tuning(self):
        """The autotuner's choice for the current structure, or None."""
        ch = np.zeros(4, np.int32)
        ms = np.zeros(11, np.float32)
        if self.L.fc3dgpu_ctx_tuning(self.ctx, ch.ctypes.data, ms.ctypes.data) != 0:
            return None
        return {"flow": bool(ch[0]), "flow_warps": int(ch[1]), "lanes32": int(ch[2]), "lanes64": int(ch[3]),
                "ms_sweep32": {"flow8": float(ms[0]), "flow10": float(ms[1]), "flow12": float(ms[2]),
                               "lanes1": float(ms[3]), "lanes2": float(ms[4]), "lanes4": float(ms[5]),
                               "lanes8": float(ms[6])},
                "ms_sweep64": {"lanes1": float(ms[7]), "lanes2": float(ms[8]), "lanes4": float(ms[9]),
                               "lanes8": float(ms[10])}}

    # ---- batched problems -------------------------------------------------
    def set_contacts(self, geo: dict, colouring: int = sn.FC3DGPU_COLOURING_DEFAULT):
        """Assemble W on the device from contact geometry (see
        LatticeScene.contacts)."""
        nc, nb = len(geo["bodyA"]), len(geo["body_mass"])
        arr = {k: np.ascontiguousarray(geo[k], np.int32 if k.startswith("body") and k[4] in "AB" else np.float64)
               for k in ("bodyA", "bodyB", "frame", "point", "body_pos", "body_mass", "body_inertia")}
        self._check(self.L.fc3dgpu_ctx_set_contacts(self.ctx, nb, nc, *(arr[k].ctypes.data for k in
                                                                         ("bodyA", "bodyB", "frame", "point",
                                                                          "body_pos", "body_mass", "body_inertia")),
                                                    colouring), "set_contacts")
        self.nc, self.nb = nc, nb

    def set_mu(self, mu):
        m = np.ascontiguousarray(mu, np.float64)
        self._check(self.L.fc3dgpu_ctx_set_mu(self.ctx, m.ctypes.data), "set_mu")

    def set_velocities(self, vel, h: float = 1e-3):
        v = np.ascontiguousarray(vel, np.float64)
        self._check(self.L.fc3dgpu_ctx_set_velocities(self.ctx, v.ctypes.data, h), "set_velocities")

    def random_walk(self, seed: int, std: float = 0.01):
        self._check(self.L.fc3dgpu_ctx_random_walk(self.ctx, seed, std), "random_walk")

    def get_q(self) -> np.ndarray:
        q = np.zeros(3 * self.nc)
        self._check(self.L.fc3dgpu_ctx_get_q(self.ctx, q.ctypes.data), "get_q")
        return q

    def get_velocities(self) -> np.ndarray:
        v = np.zeros(6 * self.nb)
        self._check(self.L.fc3dgpu_ctx_get_velocities(self.ctx, v.ctypes.data), "get_velocities")
        return v

    def sizes(self):
        nc, nnzb, ncol = C.c_int(), C.c_longlong(), C.c_int()
        self._check(self.L.fc3dgpu_ctx_sizes(self.ctx, C.byref(nc), C.byref(nnzb), C.byref(ncol)), "sizes")
        return nc.value, nnzb.value, ncol.value

    def get_W(self):
        nc, nnzb, _ = self.sizes()
        rp = np.zeros(nc + 1, np.int64)
        ci = np.zeros(nnzb, np.int64)
        bl = np.zeros(9 * nnzb)
        self._check(self.L.fc3dgpu_ctx_get_W(self.ctx, rp.ctypes.data, ci.ctypes.data, bl.ctypes.data), "get_W")
        return rp, ci, bl.reshape(nnzb, 9)

    def load_batch(self, scenes, colouring: int = sn.FC3DGPU_COLOURING_DEFAULT):
        """Upload independent problems (objects with nc, rowptr, colidx,
        blocks, q, mu) as one batch; r starts at zero."""
        ncs = np.array([sc.nc for sc in scenes], np.int32)
        offs = np.concatenate([[0], np.cumsum(ncs)]).astype(np.int64)
        boffs = np.concatenate([[0], np.cumsum([sc.rowptr[-1] for sc in scenes])]).astype(np.int64)
        rowptr = np.concatenate([sc.rowptr[:-1] + b for sc, b in zip(scenes, boffs[:-1])] + [[boffs[-1]]])
        colidx = np.concatenate([sc.colidx + o for sc, o in zip(scenes, offs[:-1])])
        blocks = np.concatenate([np.asarray(sc.blocks).reshape(-1, 9) for sc in scenes])
        self._check(self.L.fc3dgpu_ctx_set_W_batch(self.ctx, len(scenes), ncs, np.ascontiguousarray(rowptr, np.int64),
                                                   np.ascontiguousarray(colidx, np.int64),
                                                   np.ascontiguousarray(blocks).reshape(-1), colouring), "set_W_batch")
        self.nc = int(offs[-1])
        self.batch_offsets = offs
        self.set_q_mu(np.concatenate([sc.q for sc in scenes]), np.concatenate([sc.mu for sc in scenes]))
        self.set_r(np.zeros(3 * self.nc))

    def solve_batch(self, **kw) -> dict:
        n = len(self.batch_offsets) - 1
        p = self.params(**kw)
        s32 = np.zeros(n, np.int32)
        s64 = np.zeros(n, np.int32)
        err = np.zeros(n)
        info = np.zeros(n, np.int32)
        ms = C.c_double()
        self._check(self.L.fc3dgpu_ctx_solve_batch(self.ctx, C.byref(p), s32.ctypes.data, s64.ctypes.data,
                                                   err.ctypes.data, info.ctypes.data, C.byref(ms)), "solve_batch")
        return {"sweeps32": s32, "sweeps64": s64, "error": err, "info": info, "ms": ms.value}

    def get_batch(self):
        r, u = self.get()
        o = self.batch_offsets
        return [r[3 * o[k]:3 * o[k + 1]] for k in range(len(o) - 1)], [u[3 * o[k]:3 * o[k + 1]] for k in range(len(o) - 1)]

    def zero_r(self):
        self._check(self.L.fc3dgpu_ctx_zero_r(self.ctx), "zero_r")

    def stream(self) -> int:
        return int(self.L.fc3dgpu_ctx_stream(self.ctx) or 0)

    def launches(self) -> int:
        return int(self.L.fc3dgpu_ctx_launches(self.ctx))

    def get(self):
        r = np.zeros(3 * self.nc)
        u = np.zeros(3 * self.nc)
        self._check(self.L.fc3dgpu_ctx_get_r_u(self.ctx, r.ctypes.data, u.ctypes.data), "get_r_u")
        return r, u

    def compute_error(self) -> float:
        e = C.c_double()
        self._check(self.L.fc3dgpu_ctx_compute_error(self.ctx, C.byref(e)), "compute_error")
        return e.value

    def trace(self, cap: int = 100000) -> np.ndarray:
        out = np.zeros(cap)
        n = self.L.fc3dgpu_ctx_trace(self.ctx, out, cap)
        return out[:max(n, 0)].copy()

    def counters(self, enable: bool = True) -> dict:
        out = np.zeros(8, np.uint64)
        self._check(self.L.fc3dgpu_ctx_counters(self.ctx, int(enable), out.ctypes.data), "counters")
        return dict(zip(["newton", "pli", "line_search", "solves", "max_newton", "unit_cycles", "max_unit_cycles",
                         "units"], (int(v) for v in out)))

    def colours(self) -> np.ndarray:
        out = np.zeros(self.nc, np.int32)
        self.L.fc3dgpu_ctx_colours(self.ctx, out)
        return out

    def close(self):
        if self.ctx:
            self.L.fc3dgpu_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
