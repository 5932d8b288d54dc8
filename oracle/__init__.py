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
        lib.oracle_fc3d_nsgs_opts.restype = C.c_int
        lib.oracle_fc3d_nsgs_opts.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double,
                                              C.c_int, C.c_void_p, _I32, _F64, C.POINTER(C.c_int),
                                              C.POINTER(C.c_double), C.c_void_p, C.c_int, C.POINTER(C.c_int),
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
        lib.ref_fc3d_nsgs_opts.restype = C.c_int
        lib.ref_fc3d_nsgs_opts.argtypes = [C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, _F64, C.c_double, C.c_int,
                                           _I32, _F64, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p,
                                           C.c_int, C.POINTER(C.c_int)]
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


# NSGS options beyond the defaults (fc3d_nsgs.c:711-900): error evaluation
# (0 FULL, 1 LIGHT, 2 LIGHT_WITH_FULL_FINAL, 3 ADAPTIVE), the full-error
# frequency of FULL, the local tolerance strategy (0 ADAPTIVE, 1 GIVEN_VALUE,
# 2 ADAPTIVE_N_CONTACT) and its ratio, relaxation (1 = on) with omega, the
# filter of local solutions (1 = on) and contact freezing (sweeps skipped).
DEFAULT_NSGS_OPTIONS = {"err_mode": 2, "freq": 0, "strategy": 1, "ratio": 10.0, "relax": 0, "omega": 1.0,
                        "filter": 0, "freeze": 0}


def _opts6(options):
    o = dict(DEFAULT_NSGS_OPTIONS, **(options or {}))
    return (np.array([o["err_mode"], o["freq"], o["strategy"], o["relax"], o["filter"], o["freeze"]], np.int32),
            np.array([o["ratio"], o["omega"]], np.float64))


def nsgs_port(P: Problem, r0=None, tol=1e-8, maxiter=10000, order=None, trace_cap=0, options=None,
              u0=None) -> Result:
    """The restatement of fc3d_nsgs.  With `options` (keys of
    DEFAULT_NSGS_OPTIONS) the general loop with those options; `u0` is the
    velocity on entry, which the LIGHT and ADAPTIVE evaluations leave as it
    is (the result's `u_written` tells)."""
    if options is None:
        return _solve(port().oracle_fc3d_nsgs, P, r0, tol, maxiter, order, trace_cap, True)
    return _solve_opts(port().oracle_fc3d_nsgs_opts, P, r0, tol, maxiter, order, trace_cap, options, u0, True)


def nsgs_ref(P: Problem, r0=None, tol=1e-8, maxiter=10000, trace_cap=0, options=None, u0=None) -> Result:
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    if options is None:
        return _solve(lib.ref_fc3d_nsgs, P, r0, tol, maxiter, None, trace_cap, False)
    return _solve_opts(lib.ref_fc3d_nsgs_opts, P, r0, tol, maxiter, None, trace_cap, options, u0, False)


def _solve_opts(fn, P: Problem, r0, tol, maxiter, order, trace_cap, options, u0, is_port):
    r = np.zeros(3 * P.nc) if r0 is None else np.ascontiguousarray(r0, dtype=np.float64).copy()
    u = np.zeros(3 * P.nc) if u0 is None else np.ascontiguousarray(u0, dtype=np.float64).copy()
    it, err, tl, uw = C.c_int(), C.c_double(), C.c_int(), C.c_int()
    tr = np.zeros(max(trace_cap, 1))
    blocks = np.ascontiguousarray(P.blocks, dtype=np.float64).reshape(-1)
    o6, d2 = _opts6(options)
    args = [P.nc, P.rowptr, P.colidx, blocks, P.q, P.mu, r, u, tol, maxiter]
    if is_port:
        args.append(None if order is None else np.ascontiguousarray(order, np.int32).ctypes.data)
    args += [o6, d2, C.byref(it), C.byref(err), tr.ctypes.data if trace_cap else None, trace_cap, C.byref(tl)]
    if is_port:
        args.append(C.byref(uw))
    info = fn(*args)
    res = Result(info, it.value, err.value, r, u, tr[: min(tl.value, trace_cap)].copy())
    res.u_written = bool(uw.value) if is_port else None
    return res


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


# ---- global 3D friction contact (M v = q + H r, u = H^T v + b) --------------
@dataclass
class GlobalProblem:
    """A global friction-contact problem: M (n x n) and H (n x 3 nc) as CSR
    (row pointers, ascending column indices, values), q[n], b[3 nc], mu[nc]."""

    n: int
    nc: int
    Mp: np.ndarray
    Mi: np.ndarray
    Mx: np.ndarray
    Hp: np.ndarray
    Hi: np.ndarray
    Hx: np.ndarray
    q: np.ndarray
    b: np.ndarray
    mu: np.ndarray

    @staticmethod
    def from_dense(M, H, q, b, mu) -> "GlobalProblem":
        M = np.asarray(M, np.float64)
        H = np.asarray(H, np.float64)
        n = M.shape[0]
        nc = H.shape[1] // 3

        def csr(A):
            p = np.zeros(A.shape[0] + 1, np.int64)
            rows, cols = np.nonzero(A)
            np.add.at(p, rows + 1, 1)
            return np.cumsum(p), cols.astype(np.int64), A[rows, cols].astype(np.float64)

        return GlobalProblem(n, nc, *csr(M), *csr(H), np.ascontiguousarray(q, np.float64),
                             np.ascontiguousarray(b, np.float64), np.ascontiguousarray(mu, np.float64))

    def dense(self):
        M = np.zeros((self.n, self.n))
        H = np.zeros((self.n, 3 * self.nc))
        for i in range(self.n):
            M[i, self.Mi[self.Mp[i]:self.Mp[i + 1]]] = self.Mx[self.Mp[i]:self.Mp[i + 1]]
            H[i, self.Hi[self.Hp[i]:self.Hp[i + 1]]] = self.Hx[self.Hp[i]:self.Hp[i + 1]]
        return M, H

    def arrays(self):
        c = np.ascontiguousarray
        return (self.n, self.nc, c(self.Mp, np.int64), c(self.Mi, np.int64), c(self.Mx, np.float64),
                c(self.Hp, np.int64), c(self.Hi, np.int64), c(self.Hx, np.float64), c(self.q, np.float64),
                c(self.b, np.float64), c(self.mu, np.float64))


@dataclass
class GlobalResult:
    info: int
    iterations: int  # -1 where the solver does not report it (the reference's)
    error: float
    r: np.ndarray
    u: np.ndarray
    v: np.ndarray
    trace: np.ndarray


def _gport():
    lib = port()
    if not getattr(lib, "_gfc3d_typed", False):
        lib.oracle_gfc3d_nsgs.restype = C.c_int
        lib.oracle_gfc3d_nsgs.argtypes = [C.c_int64, C.c_int, _I64, _I64, _F64, _I64, _I64, _F64, _F64, _F64, _F64,
                                          _F64, _F64, _F64, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int),
                                          C.POINTER(C.c_double), C.c_void_p, C.c_int]
        lib.oracle_gfc3d_compute_error.restype = C.c_double
        lib.oracle_gfc3d_compute_error.argtypes = [C.c_int64, C.c_int, _I64, _I64, _F64, _I64, _I64, _F64, _F64,
                                                   _F64, _F64, _F64, _F64, _F64]
        lib.oracle_gfc3d_components.restype = C.c_int
        lib.oracle_gfc3d_components.argtypes = [C.c_int64, _I64, _I64, _I64]
        lib._gfc3d_typed = True
    return lib


def _gref():
    lib = ref()
    if lib is None:
        raise RuntimeError("oracle/_ref is not built")
    if not getattr(lib, "_gfc3d_typed", False):
        lib.ref_gfc3d_dat_open.restype = C.c_void_p
        lib.ref_gfc3d_dat_open.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_int)]
        lib.ref_gfc3d_dat_get.restype = C.c_int
        lib.ref_gfc3d_dat_get.argtypes = [C.c_void_p, _F64, _F64, _F64, _F64, _F64]
        lib.ref_gfc3d_dat_close.argtypes = [C.c_void_p]
        lib.ref_gfc3d_nsgs.restype = C.c_int
        lib.ref_gfc3d_nsgs.argtypes = [C.c_int, C.c_int, _F64, _F64, _F64, _F64, _F64, _F64, _F64, _F64, C.c_double,
                                       C.c_int, C.c_int, C.POINTER(C.c_double)]
        lib.ref_gfc3d_compute_error.restype = C.c_double
        lib.ref_gfc3d_compute_error.argtypes = [C.c_int, C.c_int, _F64, _F64, _F64, _F64, _F64, _F64, _F64, _F64]
        lib._gfc3d_typed = True
    return lib


def read_gfc3d_dat(path: str | Path) -> tuple[GlobalProblem, int, int]:
    """A GFC3D ``.dat`` fixture read by the reference's own reader; returns
    the problem and the storage types of M and H in the file."""
    lib = _gref()
    n, nc, ms, hs = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    h = lib.ref_gfc3d_dat_open(str(path).encode(), C.byref(n), C.byref(nc), C.byref(ms), C.byref(hs))
    if not h:
        raise IOError(f"cannot read {path}")
    M = np.zeros(n.value * n.value)
    H = np.zeros(max(n.value * 3 * nc.value, 1))
    q, b, mu = np.zeros(n.value), np.zeros(max(3 * nc.value, 1)), np.zeros(max(nc.value, 1))
    rc = lib.ref_gfc3d_dat_get(h, M, H, q, b, mu)
    lib.ref_gfc3d_dat_close(h)
    if rc != 0:
        raise IOError(f"unsupported problem in {path}")
    m = 3 * nc.value
    P = GlobalProblem.from_dense(M.reshape(n.value, n.value, order="F"),
                                 H[: n.value * m].reshape(n.value, m, order="F"), q, b[:m], mu[: nc.value])
    return P, ms.value, hs.value


def gfc3d_nsgs_port(P: GlobalProblem, r0=None, v0=None, tol=1e-8, maxiter=1000, freq=0,
                    trace_cap=0) -> GlobalResult:
    """The restatement of gfc3d_nsgs (oracle/gfc3d_oracle.c)."""
    r = np.zeros(3 * P.nc) if r0 is None else np.ascontiguousarray(r0, np.float64).copy()
    v = np.zeros(P.n) if v0 is None else np.ascontiguousarray(v0, np.float64).copy()
    u = np.zeros(3 * P.nc)
    it, err = C.c_int(), C.c_double()
    tr = np.zeros(max(trace_cap, 1))
    info = _gport().oracle_gfc3d_nsgs(*P.arrays(), r, u, v, tol, maxiter, freq, C.byref(it), C.byref(err),
                                      tr.ctypes.data if trace_cap else None, trace_cap)
    return GlobalResult(info, it.value, err.value, r, u, v, tr[: min(it.value, trace_cap)].copy())


def gfc3d_nsgs_ref(P: GlobalProblem, r0=None, v0=None, tol=1e-8, maxiter=1000, freq=0) -> GlobalResult:
    """The reference's own gfc3d_nsgs through gfc3d_driver, on dense M and H."""
    lib = _gref()
    M, H = P.dense()
    r = np.zeros(3 * P.nc) if r0 is None else np.ascontiguousarray(r0, np.float64).copy()
    v = np.zeros(P.n) if v0 is None else np.ascontiguousarray(v0, np.float64).copy()
    u = np.zeros(max(3 * P.nc, 1))
    err = C.c_double()
    info = lib.ref_gfc3d_nsgs(P.n, P.nc, np.asfortranarray(M).reshape(-1, order="F"),
                              np.ascontiguousarray(np.asfortranarray(H).reshape(-1, order="F")), P.q,
                              np.ascontiguousarray(P.b) if P.nc else np.zeros(1), P.mu if P.nc else np.zeros(1),
                              r if P.nc else np.zeros(1), u, v, tol, maxiter, freq, C.byref(err))
    return GlobalResult(info, -1, err.value, r, u[: 3 * P.nc], v, np.zeros(0))


def gfc3d_compute_error_port(P: GlobalProblem, r, v) -> tuple[float, np.ndarray]:
    u = np.zeros(3 * P.nc)
    e = _gport().oracle_gfc3d_compute_error(*P.arrays(), np.ascontiguousarray(r, np.float64),
                                            np.ascontiguousarray(v, np.float64), u)
    return e, u


def gfc3d_compute_error_ref(P: GlobalProblem, r, v) -> tuple[float, np.ndarray]:
    M, H = P.dense()
    u = np.zeros(3 * P.nc)
    e = _gref().ref_gfc3d_compute_error(P.n, P.nc, np.asfortranarray(M).reshape(-1, order="F"),
                                        np.ascontiguousarray(np.asfortranarray(H).reshape(-1, order="F")), P.q, P.b,
                                        P.mu, np.ascontiguousarray(r, np.float64),
                                        np.ascontiguousarray(v, np.float64), u)
    return e, u


def gfc3d_components(P: GlobalProblem) -> tuple[int, np.ndarray]:
    """Connected components of M's pattern (the blocks M is factorised by)."""
    comp = np.zeros(P.n, np.int64)
    k = _gport().oracle_gfc3d_components(P.n, np.ascontiguousarray(P.Mp, np.int64),
                                         np.ascontiguousarray(P.Mi, np.int64), comp)
    return k, comp


def lattice_global(nx: int, ny: int, nz: int, seed: int = 1, mu: float = 0.5, jitter_std: float = 1e-3,
                   v0_std: float = 0.1, h: float = 1e-3, mass_scale: float = 10.0) -> GlobalProblem:
    """The seeded sphere lattice in the global form (M v = q + H r,
    u = H^T v + b; 6 dofs per body), from the generator compiled into the
    oracle library (the same source as ``siconos_gb300.scene.lattice_global``)."""
    L = port()
    if not getattr(L, "_global_typed", False):
        L.fc3dgpu_lattice_global_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.fc3dgpu_lattice_fill_global.argtypes = [C.c_void_p, C.c_double, C.c_double, _I64, _I64, _F64, _I64, _I64, _F64, _F64,
                                                  _F64]
        L._global_typed = True
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
    return GlobalProblem(n.value, nc.value, Mp, Mi, Mx, Hp, Hi, Hx, q, b, np.full(nc.value, float(mu)))
