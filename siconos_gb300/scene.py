"""Seeded sphere-lattice scenes (include/fc3dgpu_scene.h) as friction-contact
problems, and the batch / time-stepping workloads built from them."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import numerics as sn


@dataclass
class LatticeScene:
    dims: tuple
    seed: int
    nc: int
    nbodies: int
    rowptr: np.ndarray
    colidx: np.ndarray
    blocks: np.ndarray  # nnzb x 9, column-major 3x3
    q: np.ndarray
    mu: np.ndarray
    gap: np.ndarray
    handle: object = None

    @property
    def nnzb(self) -> int:
        return int(self.rowptr[-1])

    def problem(self) -> sn.FrictionContactProblem:
        W = sn.SparseBlockMatrix(self.nc, self.rowptr, self.colidx, self.blocks)
        return sn.FrictionContactProblem(3, self.nc, W, self.q, self.mu)

    def contacts(self) -> dict:
        """Geometry for a device assembly of W and q: contact bodies, frames,
        points; body centres, masses, inertias, velocities."""
        L = sn.lib()
        A = np.zeros(self.nc, np.int32)
        B = np.zeros(self.nc, np.int32)
        L.fc3dgpu_lattice_fill_geometry(self.handle, None, A.ctypes.data, B.ctypes.data)
        out = {"bodyA": A, "bodyB": B, "frame": np.zeros(9 * self.nc), "point": np.zeros(3 * self.nc),
               "body_pos": np.zeros(3 * self.nbodies), "body_mass": np.zeros(self.nbodies),
               "body_inertia": np.zeros(self.nbodies), "vel": np.zeros(6 * self.nbodies)}
        L.fc3dgpu_lattice_fill_contacts(self.handle, *(out[k].ctypes.data for k in
                                                       ("frame", "point", "body_pos", "body_mass", "body_inertia",
                                                        "vel")))
        return out

    def perturb(self, seed: int, std: float = 0.01, h: float = 1e-3):
        """v0 += N(0, std^2) per degree of freedom; q recomputed, contacts kept."""
        L = sn.lib()
        L.fc3dgpu_lattice_perturb_velocities(self.handle, seed, std)
        L.fc3dgpu_lattice_fill_q(self.handle, h, self.q)

    def __del__(self):
        try:
            if self.handle:
                sn.lib().fc3dgpu_lattice_free(self.handle)
                self.handle = None
        except Exception:
            pass


def lattice(nx: int, ny: int, nz: int, seed: int = 1, mu: float = 0.5, jitter_std: float = 1e-3,
            v0_std: float = 0.1, h: float = 1e-3) -> LatticeScene:
    L = sn.lib()
    hdl = L.fc3dgpu_lattice_create(nx, ny, nz, seed, jitter_std, v0_std)
    if not hdl:
        raise ValueError("bad lattice size")
    nb, nc, nnzb = C.c_int(), C.c_int(), C.c_int64()
    L.fc3dgpu_lattice_sizes(hdl, C.byref(nb), C.byref(nc), C.byref(nnzb))
    n, k = nc.value, nnzb.value
    rp = np.zeros(n + 1, np.int64)
    ci = np.zeros(k, np.int64)
    bl = np.zeros(9 * k)
    q = np.zeros(3 * n)
    gap = np.zeros(n)
    L.fc3dgpu_lattice_fill_W(hdl, rp, ci, bl)
    L.fc3dgpu_lattice_fill_q(hdl, h, q)
    L.fc3dgpu_lattice_fill_geometry(hdl, gap.ctypes.data, None, None)
    return LatticeScene((nx, ny, nz), seed, n, nb.value, rp, ci, bl.reshape(k, 9), q, np.full(n, float(mu)), gap, hdl)


def lattice_global(nx: int, ny: int, nz: int, seed: int = 1, mu: float = 0.5, jitter_std: float = 1e-3,
                   v0_std: float = 0.1, h: float = 1e-3, mass_scale: float = 10.0):
    """The scene in the global form of the reference's
    GlobalFrictionContactProblem (M v = q + H r, u = H^T v + b, 6 dofs per
    body): a namespace with n, nc and the CSR arrays Mp, Mi, Mx, Hp, Hi, Hx
    and q, b, mu (see include/fc3dgpu_scene.h)."""
    from types import SimpleNamespace
    L = sn.lib()
    hdl = L.fc3dgpu_lattice_create(nx, ny, nz, seed, jitter_std, v0_std)
    if not hdl:
        raise ValueError("bad lattice size")
    try:
        nb, nc, nnzb = C.c_int(), C.c_int(), C.c_int64()
        L.fc3dgpu_lattice_sizes(hdl, C.byref(nb), C.byref(nc), C.byref(nnzb))
        n, nh = C.c_int64(), C.c_int64()
        L.fc3dgpu_lattice_global_sizes(hdl, C.byref(n), C.byref(nh))
        Mp, Mi, Mx = np.zeros(n.value + 1, np.int64), np.zeros(n.value, np.int64), np.zeros(n.value)
        Hp, Hi, Hx = np.zeros(n.value + 1, np.int64), np.zeros(nh.value, np.int64), np.zeros(nh.value)
        q, b = np.zeros(n.value), np.zeros(3 * nc.value)
        L.fc3dgpu_lattice_fill_global(hdl, h, mass_scale, Mp, Mi, Mx, Hp, Hi, Hx, q, b)
    finally:
        L.fc3dgpu_lattice_free(hdl)
    return SimpleNamespace(dims=(nx, ny, nz), seed=seed, n=n.value, nc=nc.value, nbodies=nb.value, Mp=Mp, Mi=Mi,
                           Mx=Mx, Hp=Hp, Hi=Hi, Hx=Hx, q=q, b=b, mu=np.full(nc.value, float(mu)))


def batch_specs(count: int = 512, seed: int = 7, lo=(3, 3, 2), hi=(20, 20, 10), mu_range=(0.1, 0.9)):
    """(dims, seed, mu) of each scene of the batch: dims drawn uniformly in
    [lo, hi] per axis, mu ~ U(mu_range) per scene."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        d = tuple(int(rng.integers(lo[a], hi[a] + 1)) for a in range(3))
        m = float(rng.uniform(*mu_range))
        out.append((d, seed * 100003 + k, m))
    return out


def batch_scenes(count: int = 512, seed: int = 7, lo=(3, 3, 2), hi=(20, 20, 10), mu_range=(0.1, 0.9)):
    """Independent scenes of batch_specs."""
    return [lattice(*d, seed=sd, mu=m) for d, sd, m in batch_specs(count, seed, lo, hi, mu_range)]
