"""The oracle -- TEST INFRASTRUCTURE ONLY.

Two CPU implementations of the reference's FC3D NSGS path, used only by
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg as
checkers:

* ``port``: this project's C restatement (``fc3d_oracle.c``,
  ``colour_oracle.c``), built by ``oracle/build.py``; it runs anywhere;
* ``ref``: the reference's own numerics C sources compiled by
  ``oracle/build_ref.py`` into ``oracle/_ref`` (only where the reference
  checkout is present).

Problems are passed as plain block-CSR numpy arrays: ``rowptr`` (int64,
nc+1), ``colidx`` (int64, nnzb), ``blocks`` (float64, nnzb x 9, each 3x3 block
column-major), ``q`` (3 nc), ``mu`` (nc).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_F64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


@dataclass
class Problem:
    """A friction-contact problem (3D unless dim says 2) in block-CSR form
    (host arrays)."""

    nc: int
    rowptr: np.ndarray
    colidx: np.ndarray
    blocks: np.ndarray
    q: np.ndarray
    mu: np.ndarray
    dim: int = 3

    @property
    def nnzb(self) -> int:
        return int(self.rowptr[-1])


@dataclass
class Result:
    info: int
    iterations: int
    error: float
    r: np.ndarray
    u: np.ndarray
    trace: np.ndarray


_port = None
_ref = None


def port():
    """ctypes handle on the oracle's C restatement (built on first use)."""
    global _port
    if _port is None:
        from . import build as _b
        lib = C.CDLL(str(_b.build()))
        lib.oracle_fc3d_nsgs.restype = C.c_int
        lib.oracle_fc3d_nsgs.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double, C.c_int,
                                         C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                         C.POINTER(C.c_int)]
        lib.oracle_fc2d_nsgs.restype = C.c_int
        lib.oracle_fc2d_nsgs.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double, C.c_int,
                                         C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                         C.POINTER(C.c_int)]
        lib.oracle_rfc3d_nsgs.restype = C.c_int
        lib.oracle_rfc3d_nsgs.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, _F64, C.c_double,
                                          C.c_int, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        lib.oracle_rfc3d_compute_error.restype = C.c_double
        lib.oracle_rfc3d_compute_error.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, _F64,
                                                   C.c_double]
        lib.oracle_rfc3d_max_eig.restype = C.c_double
        lib.oracle_rfc3d_max_eig.argtypes = [_F64]
        lib.oracle_fc2d_sweeps_f32.restype = C.c_int
        lib.oracle_fc2d_sweeps_f32.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, C.c_int, C.c_void_p]
        lib.oracle_fc2d_compute_error.restype = C.c_double
        lib.oracle_fc2d_compute_error.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double]
        lib.oracle_fc3d_compute_error.restype = C.c_double
        lib.oracle_fc3d_compute_error.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double]
        lib.oracle_ac_std.restype = None
        lib.oracle_ac_std.argtypes = [_F64, _F64, C.c_double, _F64, _F64, C.c_void_p, C.c_void_p]
        lib.oracle_solve_3x3_gepp.restype = C.c_int
        lib.oracle_solve_3x3_gepp.argtypes = [_F64, _F64]
        lib.oracle_projection_on_cone.restype = C.c_uint
        lib.oracle_projection_on_cone.argtypes = [_F64, C.c_double]
        lib.oracle_local_solve.restype = C.c_double
        lib.oracle_local_solve.argtypes = [_F64, _F64, C.c_double, _F64, _F64, C.c_double]
        lib.fc3dgpu_lattice_create.restype = C.c_void_p
        lib.fc3dgpu_lattice_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double, C.c_double]
        lib.fc3dgpu_lattice_free.argtypes = [C.c_void_p]
        lib.fc3dgpu_lattice_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                              C.POINTER(C.c_int64)]
        lib.fc3dgpu_lattice_fill_W.argtypes = [C.c_void_p, _I64, _I64, _F64]
        lib.fc3dgpu_lattice_fill_q.argtypes = [C.c_void_p, C.c_double, _F64]
        if hasattr(lib, "oracle_colour_greedy"):
            lib.oracle_colour_greedy.restype = C.c_int
            lib.oracle_colour_greedy.argtypes = [C.c_int, _I64, _I64, C.c_int, _I32]
            lib.oracle_colour_check.restype = C.c_int
            lib.oracle_colour_check.argtypes = [C.c_int, _I64, _I64, _I32]
            lib.oracle_colour_priority.restype = C.c_uint32
            lib.oracle_colour_priority.argtypes = [C.c_uint32, C.c_int, C.c_uint32]
        _port = lib
    return _port


def lattice(nx: int, ny: int, nz: int, seed: int = 1, mu: float = 0.5, jitter_std: float = 1e-3,
            v0_std: float = 0.1, h: float = 1e-3) -> Problem:
    """The seeded sphere-lattice scene as a Problem, from the generator
    compiled into the oracle library (the same source and results as
    ``siconos_gb300.scene.lattice``), for CPU-only measurements that must not
    load the solver library."""
    L = port()
    hdl = L.fc3dgpu_lattice_create(nx, ny, nz, seed, jitter_std, v0_std)
    if not hdl:
        raise ValueError("bad lattice size")
    try:
        nb, nc, nnzb = C.c_int(), C.c_int(), C.c_int64()
        L.fc3dgpu_lattice_sizes(hdl, C.byref(nb), C.byref(nc), C.byref(nnzb))
        n, k = nc.value, nnzb.value
        rp = np.zeros(n + 1, np.int64)
        ci = np.zeros(k, np.int64)
        bl = np.zeros(9 * k)
        q = np.zeros(3 * n)
        L.fc3dgpu_lattice_fill_W(hdl, rp, ci, bl)
        L.fc3dgpu_lattice_fill_q(hdl, h, q)
    finally:
        L.fc3dgpu_lattice_free(hdl)
    return Problem(n, rp, ci, bl.reshape(k, 9), q, np.full(n, float(mu)))


def ref_available() -> bool:
    from . import build_ref as _br
    return _br.LIB.exists()


def ref():
    """ctypes handle on the reference's own numerics (oracle/_ref), or None."""
    global _ref
    if _ref is None:
        from . import build_ref as _br
        if not _br.LIB.exists():
            return None
        lib = C.CDLL(str(_br.LIB))
        lib.ref_fc3d_nsgs.restype = C.c_int
        lib.ref_fc3d_nsgs.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double, C.c_int,
                                      C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                      C.POINTER(C.c_int)]
        lib.ref_fc3d_compute_error.restype = C.c_double
        lib.ref_fc3d_compute_error.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64]
        lib.ref_dat_open.restype = C.c_void_p
        lib.ref_dat_open.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int64), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]
        lib.ref_dat_get.restype = C.c_int
        lib.ref_dat_get.argtypes = [C.c_void_p, _I64, _I64, _F64, _F64, _F64]
        lib.ref_dat_close.argtypes = [C.c_void_p]
        lib.ref_fc2d_nsgs.restype = C.c_int
        lib.ref_fc2d_nsgs.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double, C.c_int,
                                      C.POINTER(C.c_int), C.POINTER(C.c_double)]
        lib.ref_fc2d_compute_error.restype = C.c_double
        lib.ref_fc2d_compute_error.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64]
        lib.ref_dat_write.restype = C.c_int
        lib.ref_dat_write.argtypes = [C.c_char_p, C.c_int, C.c_int, _I64, _I64, _F64, _F64, _F64, C.c_int]
        lib.ref_rfc3d_nsgs.restype = C.c_int
        lib.ref_rfc3d_nsgs.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, _F64, C.c_double,
                                       C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                       C.POINTER(C.c_int)]
        lib.ref_rfc3d_compute_error.restype = C.c_double
        lib.ref_rfc3d_compute_error.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, _F64]
        lib.ref_rfc3d_max_eig.restype = C.c_double
        lib.ref_rfc3d_max_eig.argtypes = [_F64]
        lib.ref_rfc3d_dat_open.restype = C.c_void_p
        lib.ref_rfc3d_dat_open.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int)]
        lib.ref_rfc3d_dat_get.restype = C.c_int
        lib.ref_rfc3d_dat_get.argtypes = [C.c_void_p, _I64, _I64, _F64, _F64, _F64, _F64]
        lib.ref_rfc3d_dat_close.argtypes = [C.c_void_p]
        lib.computeAlartCurnierSTD.restype = None
        lib.computeAlartCurnierSTD.argtypes = [_F64, _F64, C.c_double, _F64, _F64, C.c_void_p, C.c_void_p]
        lib.ref_solve_3x3_gepp.restype = C.c_int
        lib.ref_solve_3x3_gepp.argtypes = [_F64, _F64]
        lib.ref_projection_on_cone.restype = C.c_uint
        lib.ref_projection_on_cone.argtypes = [_F64, C.c_double]
        _ref = lib
    return _ref


def write_dat_ref(P: Problem, path: str | Path, dense: bool = False) -> None:
    """Write a problem with the reference's own writer."""
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    rc = lib.ref_dat_write(str(path).encode(), P.dim, P.nc, np.ascontiguousarray(P.rowptr, np.int64),
                           np.ascontiguousarray(P.colidx, np.int64),
                           np.ascontiguousarray(P.blocks, np.float64).reshape(-1),
                           np.ascontiguousarray(P.q, np.float64), np.ascontiguousarray(P.mu, np.float64),
                           1 if dense else 0)
    if rc != 0:
        raise IOError(f"reference writer failed on {path} ({rc})")


def read_dat(path: str | Path) -> Problem:
    """Read a reference ``.dat`` fixture with the reference's own reader."""
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    nc, nnzb, st, dm = C.c_int(), C.c_int64(), C.c_int(), C.c_int()
    h = lib.ref_dat_open(str(path).encode(), C.byref(nc), C.byref(nnzb), C.byref(st), C.byref(dm))
    if not h:
        raise IOError(f"cannot read {path}")
    n, nb, d = nc.value, nnzb.value, dm.value
    rp = np.zeros(n + 1, np.int64)
    ci = np.zeros(max(nb, 1), np.int64)
    bl = np.zeros(d * d * max(nb, 1))
    q = np.zeros(d * n)
    mu = np.zeros(n)
    rc = lib.ref_dat_get(h, rp, ci, bl, q, mu)
    lib.ref_dat_close(h)
    if rc != 0:
        raise IOError(f"unsupported storage in {path}")
    return Problem(n, rp, ci[:nb].copy(), bl[: d * d * nb].reshape(nb, d * d).copy(), q, mu, d)


def _solve(fn, P: Problem, r0, tol, maxiter, order, trace_cap, is_port):
    r = np.zeros(3 * P.nc) if r0 is None else np.ascontiguousarray(r0, dtype=np.float64).copy()
    u = np.zeros(3 * P.nc)
    it, err, tl = C.c_int(), C.c_double(), C.c_int()
    tr = np.zeros(max(trace_cap, 1))
    blocks = np.ascontiguousarray(P.blocks, dtype=np.float64).reshape(-1)
    order_arr = None if order is None else np.ascontiguousarray(order, np.int32)
    args = [P.nc, P.rowptr, P.colidx, blocks, P.q, P.mu, r, u, tol, maxiter]
    if is_port:
        args.append(None if order_arr is None else order_arr.ctypes.data)
    args += [C.byref(it), C.byref(err), tr.ctypes.data if trace_cap else None, trace_cap, C.byref(tl)]
    info = fn(*args)
    return Result(info, it.value, err.value, r, u, tr[: min(tl.value, trace_cap)].copy())


def nsgs_port(P: Problem, r0=None, tol=1e-8, maxiter=10000, order=None, trace_cap=0) -> Result:
    return _solve(port().oracle_fc3d_nsgs, P, r0, tol, maxiter, order, trace_cap, True)


def nsgs_ref(P: Problem, r0=None, tol=1e-8, maxiter=10000, trace_cap=0) -> Result:
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    return _solve(lib.ref_fc3d_nsgs, P, r0, tol, maxiter, None, trace_cap, False)


def compute_error_port(P: Problem, r) -> tuple[float, np.ndarray]:
    u = np.zeros(3 * P.nc)
    nq = float(np.sqrt(np.sum(P.q * P.q)))
    blocks = np.ascontiguousarray(P.blocks, dtype=np.float64).reshape(-1)
    e = port().oracle_fc3d_compute_error(P.nc, P.rowptr, P.colidx, blocks, P.q, P.mu,
                                         np.ascontiguousarray(r, np.float64), u, nq)
    return e, u


def compute_error_ref(P: Problem, r) -> tuple[float, np.ndarray]:
    u = np.zeros(3 * P.nc)
    blocks = np.ascontiguousarray(P.blocks, dtype=np.float64).reshape(-1)
    e = ref().ref_fc3d_compute_error(P.nc, P.rowptr, P.colidx, blocks, P.q, P.mu,
                                     np.ascontiguousarray(r, np.float64), u)
    return e, u


# ---- 2D friction contact (dim = 2, blocks 2x2) --------------------------------
def fc2d_nsgs_port(P: Problem, r0=None, tol=1e-5, maxiter=10000, order=None, trace_cap=0) -> Result:
    """The restatement of fc2d_nsgs (oracle/fc2d_oracle.c)."""
    r = np.zeros(2 * P.nc) if r0 is None else np.ascontiguousarray(r0, dtype=np.float64).copy()
    u = np.zeros(2 * P.nc)
    it, err, tl = C.c_int(), C.c_double(), C.c_int()
    tr = np.zeros(max(trace_cap, 1))
    order_arr = None if order is None else np.ascontiguousarray(order, np.int32)
    info = port().oracle_fc2d_nsgs(P.nc, np.ascontiguousarray(P.rowptr, np.int64),
                                   np.ascontiguousarray(P.colidx, np.int64),
                                   np.ascontiguousarray(P.blocks, np.float64).reshape(-1),
                                   np.ascontiguousarray(P.q, np.float64), np.ascontiguousarray(P.mu, np.float64),
                                   r, u, tol, maxiter, None if order_arr is None else order_arr.ctypes.data,
                                   C.byref(it), C.byref(err), tr.ctypes.data if trace_cap else None, trace_cap,
                                   C.byref(tl))
    return Result(info, it.value, err.value, r, u, tr[: min(tl.value, trace_cap)].copy())


def fc2d_nsgs_ref(P: Problem, r0=None, tol=1e-5, maxiter=10000) -> Result:
    """The reference's own fc2d_nsgs through fc2d_driver."""
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    r = np.zeros(2 * P.nc) if r0 is None else np.ascontiguousarray(r0, dtype=np.float64).copy()
    u = np.zeros(2 * P.nc)
    it, err = C.c_int(), C.c_double()
    info = lib.ref_fc2d_nsgs(P.nc, np.ascontiguousarray(P.rowptr, np.int64),
                             np.ascontiguousarray(P.colidx, np.int64),
                             np.ascontiguousarray(P.blocks, np.float64).reshape(-1),
                             np.ascontiguousarray(P.q, np.float64), np.ascontiguousarray(P.mu, np.float64), r, u,
                             tol, maxiter, C.byref(it), C.byref(err))
    return Result(info, it.value, err.value, r, u, np.zeros(0))


def fc2d_sweeps_f32_port(P: Problem, r0, nsweeps: int, order=None) -> np.ndarray:
    """`nsweeps` single-precision sweeps from r0 (the FP32 phase of the GPU
    solver's mixed mode, oracle/fc2d_oracle.c); the reaction widened to
    double."""
    r = np.ascontiguousarray(r0, dtype=np.float64).copy()
    order_arr = None if order is None else np.ascontiguousarray(order, np.int32)
    rc = port().oracle_fc2d_sweeps_f32(P.nc, np.ascontiguousarray(P.rowptr, np.int64),
                                       np.ascontiguousarray(P.colidx, np.int64),
                                       np.ascontiguousarray(P.blocks, np.float64).reshape(-1),
                                       np.ascontiguousarray(P.q, np.float64), np.ascontiguousarray(P.mu, np.float64),
                                       r, nsweeps, None if order_arr is None else order_arr.ctypes.data)
    if rc != 0:
        raise ValueError("a contact has no diagonal block")
    return r


def fc2d_compute_error_port(P: Problem, r) -> tuple[float, np.ndarray]:
    u = np.zeros(2 * P.nc)
    q = np.ascontiguousarray(P.q, np.float64)
    nq = float(np.sqrt(np.sum(q * q)))
    e = port().oracle_fc2d_compute_error(P.nc, np.ascontiguousarray(P.rowptr, np.int64),
                                         np.ascontiguousarray(P.colidx, np.int64),
                                         np.ascontiguousarray(P.blocks, np.float64).reshape(-1), q,
                                         np.ascontiguousarray(P.mu, np.float64),
                                         np.ascontiguousarray(r, np.float64), u, nq)
    return e, u


def fc2d_compute_error_ref(P: Problem, r) -> tuple[float, np.ndarray]:
    u = np.zeros(2 * P.nc)
    e = ref().ref_fc2d_compute_error(P.nc, np.ascontiguousarray(P.rowptr, np.int64),
                                     np.ascontiguousarray(P.colidx, np.int64),
                                     np.ascontiguousarray(P.blocks, np.float64).reshape(-1),
                                     np.ascontiguousarray(P.q, np.float64), np.ascontiguousarray(P.mu, np.float64),
                                     np.ascontiguousarray(r, np.float64), u)
    return e, u


# ---- 3D rolling friction (5 components per contact) -------------------------
@dataclass
class RollingProblem:
    """A rolling-friction problem: W as block-CSR of 5x5 column-major blocks,
    q[5 nc], mu and mu_r per contact."""

    nc: int
    rowptr: np.ndarray
    colidx: np.ndarray
    blocks: np.ndarray
    q: np.ndarray
    mu: np.ndarray
    mur: np.ndarray

    @property
    def nnzb(self) -> int:
        return int(self.rowptr[-1])

    def arrays(self):
        return (self.nc, np.ascontiguousarray(self.rowptr, np.int64), np.ascontiguousarray(self.colidx, np.int64),
                np.ascontiguousarray(self.blocks, np.float64).reshape(-1), np.ascontiguousarray(self.q, np.float64),
                np.ascontiguousarray(self.mu, np.float64), np.ascontiguousarray(self.mur, np.float64))


def read_rfc3d_dat(path: str | Path) -> RollingProblem:
    """A rolling-friction ``.dat`` fixture read by the reference's own reader."""
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    nc, nnzb, st = C.c_int(), C.c_int64(), C.c_int()
    h = lib.ref_rfc3d_dat_open(str(path).encode(), C.byref(nc), C.byref(nnzb), C.byref(st))
    if not h:
        raise IOError(f"cannot read {path}")
    n, nb = nc.value, nnzb.value
    rp = np.zeros(n + 1, np.int64)
    ci = np.zeros(max(nb, 1), np.int64)
    bl = np.zeros(25 * max(nb, 1))
    q, mu, mur = np.zeros(5 * n), np.zeros(n), np.zeros(n)
    rc = lib.ref_rfc3d_dat_get(h, rp, ci, bl, q, mu, mur)
    lib.ref_rfc3d_dat_close(h)
    if rc != 0:
        raise IOError(f"unsupported storage in {path}")
    return RollingProblem(n, rp, ci[:nb].copy(), bl[: 25 * nb].reshape(nb, 25).copy(), q, mu, mur)


def _rfc3d_solve(fn, P: RollingProblem, r0, tol, maxiter, order, trace_cap, is_port):
    r = np.zeros(5 * P.nc) if r0 is None else np.ascontiguousarray(r0, dtype=np.float64).copy()
    u = np.zeros(5 * P.nc)
    it, err, tl = C.c_int(), C.c_double(), C.c_int()
    tr = np.zeros(max(trace_cap, 1))
    order_arr = None if order is None else np.ascontiguousarray(order, np.int32)
    args = [*P.arrays(), r, u, tol, maxiter]
    if is_port:
        args.append(None if order_arr is None else order_arr.ctypes.data)
    args += [C.byref(it), C.byref(err), tr.ctypes.data if trace_cap else None, trace_cap, C.byref(tl)]
    info = fn(*args)
    return Result(info, it.value, err.value, r, u, tr[: min(tl.value, trace_cap)].copy())


def rfc3d_nsgs_port(P: RollingProblem, r0=None, tol=1e-8, maxiter=10000, order=None, trace_cap=0) -> Result:
    """The restatement of rolling_friction_3d_nsgs (oracle/rfc3d_oracle.c)."""
    return _rfc3d_solve(port().oracle_rfc3d_nsgs, P, r0, tol, maxiter, order, trace_cap, True)


def rfc3d_nsgs_ref(P: RollingProblem, r0=None, tol=1e-8, maxiter=10000, trace_cap=0) -> Result:
    """The reference's own rolling_friction_3d_nsgs through its driver."""
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    return _rfc3d_solve(lib.ref_rfc3d_nsgs, P, r0, tol, maxiter, None, trace_cap, False)


def rfc3d_compute_error_port(P: RollingProblem, r) -> tuple[float, np.ndarray]:
    u = np.zeros(5 * P.nc)
    a = P.arrays()
    nq = float(np.sqrt(np.sum(a[4] * a[4])))
    e = port().oracle_rfc3d_compute_error(*a, np.ascontiguousarray(r, np.float64), u, nq)
    return e, u


def rfc3d_compute_error_ref(P: RollingProblem, r) -> tuple[float, np.ndarray]:
    u = np.zeros(5 * P.nc)
    e = ref().ref_rfc3d_compute_error(*P.arrays(), np.ascontiguousarray(r, np.float64), u)
    return e, u
