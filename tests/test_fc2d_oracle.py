"""The 2D friction-contact oracle against the golden fixtures, and the host
side of the GPU 2D solver (options, argument checks) without a GPU.

Fixtures whose ``results`` field is "reference" hold the reference's own
fc2d_nsgs outputs (tests/golden/make_golden.py); the restatement must
reproduce them bit for bit.  "oracle" fixtures (CSparse-stored problems the
reference build here cannot read) pin the restatement against itself across
platforms."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN

FC2D_CASES = sorted(p.stem for p in GOLDEN.glob("fc2d_*.npz"))


def load_fc2d(name):
    import oracle as O
    z = np.load(GOLDEN / f"{name}.npz")
    P = O.Problem(int(z["nc"]), z["rowptr"], z["colidx"], z["blocks"], z["q"], z["mu"], 2)
    return P, {k: z[k] for k in z.files}


def test_fixture_set():
    kinds = [str(load_fc2d(c)[1]["results"]) for c in FC2D_CASES]
    assert len(FC2D_CASES) == 11
    assert kinds.count("reference") == 8


@pytest.mark.parametrize("case", FC2D_CASES)
def test_port_reproduces_fixture(case):
    import oracle as O
    P, g = load_fc2d(case)
    if P.nc > 3000:
        pytest.skip("large case: covered on the GPU")
    for suffix, maxiter in (("", 10000), ("20", 20)):
        res = O.fc2d_nsgs_port(P, tol=1e-5, maxiter=maxiter)
        assert res.info == int(g["info" + suffix])
        assert res.iterations == int(g["iterations" + suffix])
        assert res.error == float(g["error" + suffix])
        np.testing.assert_array_equal(res.r, g["r" + suffix])
        np.testing.assert_array_equal(res.u, g["u" + suffix])


@pytest.mark.parametrize("case", [c for c in FC2D_CASES if "granular" not in c])
def test_port_compute_error_matches_reference_run(case):
    """fc2d_compute_error of the reference's final reaction gives the error
    and velocity it reported (norm_q summed in index order as the solver)."""
    import oracle as O
    P, g = load_fc2d(case)
    e, u = O.fc2d_compute_error_port(P, g["r"])
    np.testing.assert_array_equal(u, g["u"])
    assert e == pytest.approx(float(g["error"]), rel=1e-14, abs=0)


def test_port_order_permutes_sweep():
    """With a visiting order, the restatement is the sequential sweep in that
    order: a reversed order gives another iterate, the identity the same."""
    import oracle as O
    P, g = load_fc2d("fc2d_FC2D_SliderCrankLagrangian00000")
    a = O.fc2d_nsgs_port(P, tol=0.0, maxiter=7)
    b = O.fc2d_nsgs_port(P, tol=0.0, maxiter=7, order=np.arange(P.nc, dtype=np.int32))
    c = O.fc2d_nsgs_port(P, tol=0.0, maxiter=7, order=np.arange(P.nc, dtype=np.int32)[::-1].copy())
    np.testing.assert_array_equal(a.r, b.r)
    assert a.iterations == b.iterations == c.iterations == 7
    assert not np.array_equal(a.r, c.r)


def test_f32_sweeps_track_f64():
    """The single-precision restatement follows the FP64 sweep to FP32
    rounding (it is the checker of the GPU's FP32 phase)."""
    import oracle as O
    P, _ = load_fc2d("fc2d_FrictionContactProblem00071")
    r32 = O.fc2d_sweeps_f32_port(P, np.zeros(2 * P.nc), 30)
    ref = O.fc2d_nsgs_port(P, tol=0.0, maxiter=30)
    assert np.abs(r32 - ref.r).max() <= 1e-5 * np.abs(ref.r).max()
    assert not np.array_equal(r32, ref.r)
    again = O.fc2d_sweeps_f32_port(P, r32, 0)
    np.testing.assert_array_equal(again, r32)


def test_port_singular_diagonal_block():
    import oracle as O
    rowptr = np.array([0, 1, 2], np.int64)
    colidx = np.array([0, 1], np.int64)
    blocks = np.array([[1.0, 0.0, 0.0, 1.0], [1.0, 1.0, 1.0, 1.0]])  # second determinant 0
    P = O.Problem(2, rowptr, colidx, blocks, np.array([-1.0, 0.1, -1.0, 0.2]), np.array([0.3, 0.3]), 2)
    res = O.fc2d_nsgs_port(P)
    assert res.info == 1 and res.iterations == 0 and np.isinf(res.error)


# ----------------------------------------------------------------------------
# host side of the GPU solver (no device call)
# ----------------------------------------------------------------------------
def _problem2d(nc=3):
    import siconos_gb300.numerics as sn
    rowptr = np.arange(nc + 1, dtype=np.int64)
    colidx = np.arange(nc, dtype=np.int64)
    blocks = np.tile(np.array([2.0, 0.1, 0.1, 1.5]), (nc, 1))
    W = sn.SparseBlockMatrix(nc, rowptr, colidx, blocks, block_size=2)
    q = np.tile(np.array([-1.0, 0.2]), nc)
    mu = np.full(nc, 0.3)
    return sn.FrictionContactProblem(2, nc, W, q, mu)


def test_options_defaults(built_lib):
    import siconos_gb300.numerics as sn
    o = sn.SolverOptions(sn.SICONOS_FRICTION_2D_NSGS_GPU)
    assert o.solverId == sn.SICONOS_FRICTION_2D_NSGS_GPU == 412
    assert o.iparam[sn.SICONOS_IPARAM_MAX_ITER] == 1000
    assert o.dparam[sn.SICONOS_DPARAM_TOL] == 1e-4
    assert o.iparam[sn.SICONOS_IPARAM_NSGS_SHUFFLE] == 0
    assert o.iparam[sn.FC3DGPU_IPARAM_PRECISION] == 0  # FP32 sweeps + FP64 polish
    assert o.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] == \
        sn.SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL
    o.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] = sn.SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT
    built_lib.fc2dgpu_nsgs_set_default(o.ptr)
    assert o.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] == \
        sn.SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL
    with pytest.raises(ValueError):
        sn.SolverOptions(sn.SICONOS_FRICTION_2D_NSGS)


def test_driver_argument_checks(built_lib):
    """The fc2d_driver checks, all before any device work."""
    import siconos_gb300.numerics as sn
    P = _problem2d()
    r, u = np.zeros(6), np.zeros(6)
    o = sn.SolverOptions(sn.SICONOS_FRICTION_2D_NSGS_GPU)
    L = built_lib
    assert L.fc2dgpu_driver(None, r.ctypes.data_as(sn._DP), u.ctypes.data_as(sn._DP), o.ptr) == \
        sn.NUMERICS_ERR_NULL_POINTER
    assert L.fc2dgpu_driver(C.byref(P.c), r.ctypes.data_as(sn._DP), u.ctypes.data_as(sn._DP), None) == \
        sn.NUMERICS_ERR_INVALID_OPTION
    # a 3D problem is not a 2D one
    P3 = sn.FrictionContactProblem(3, 2, sn.SparseBlockMatrix(2, [0, 1, 2], [0, 1], np.eye(3).reshape(1, 9)
                                                              .repeat(2, 0)), np.ones(6), np.ones(2))
    assert L.fc2dgpu_driver(C.byref(P3.c), r.ctypes.data_as(sn._DP), u.ctypes.data_as(sn._DP), o.ptr) == \
        sn.NUMERICS_ERR_INVALID_ARGUMENT
    assert "expected 2" in sn.last_error()
    # a foreign solver id
    o3 = sn.SolverOptions(sn.SICONOS_FRICTION_3D_NSGS_GPU)
    assert sn.fc2d_driver(P, r, u, o3) == sn.NUMERICS_ERR_INVALID_SOLVER
    # contact freezing is not implemented by the coloured sweep
    o.iparam[sn.SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT] = 5
    assert sn.fc2d_nsgs_gpu(P, r, u, o) == sn.NUMERICS_ERR_NOT_IMPLEMENTED


def tiled2d(P, copies: int, seed: int):
    """`copies` independent copies of a 2D problem along W's diagonal, q of
    each copy scaled by a seeded factor in [0.9, 1.1]."""
    import oracle as O
    g = np.random.default_rng(seed)
    nc, nb = P.nc, P.nnzb
    rp = [0]
    for c in range(copies):
        rp.extend((P.rowptr[1:] + c * nb).tolist())
    return O.Problem(copies * nc, np.asarray(rp, np.int64),
                     np.concatenate([P.colidx + c * nc for c in range(copies)]).astype(np.int64),
                     np.tile(np.asarray(P.blocks).reshape(nb, 4), (copies, 1)),
                     np.tile(P.q, copies) * np.repeat(g.uniform(0.9, 1.1, copies), 2 * nc), np.tile(P.mu, copies), 2)


def test_tiled2d_copies_are_independent():
    import oracle as O
    P, _ = load_fc2d("fc2d_FrictionContactProblem00071")
    T = tiled2d(P, 3, 2)
    res = O.fc2d_nsgs_port(T, tol=0.0, maxiter=6)
    for c in range(3):
        Pc = O.Problem(P.nc, P.rowptr, P.colidx, P.blocks, T.q[2 * c * P.nc:2 * (c + 1) * P.nc], P.mu, 2)
        np.testing.assert_array_equal(res.r[2 * c * P.nc:2 * (c + 1) * P.nc], O.fc2d_nsgs_port(Pc, tol=0.0, maxiter=6).r)
