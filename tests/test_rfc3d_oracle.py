"""The 3D rolling-friction oracle (oracle/rfc3d_oracle.c) against the golden
fixtures, which hold the reference's own rolling_friction_3d_nsgs results
(tests/golden/make_golden.py --only=rfc3d): r, u, iterations, error and the
per-iteration error trace, bit for bit, for full and 20-iteration runs.
Where the reference library is built here, also against it directly."""
import numpy as np
import pytest

from conftest import GOLDEN

RFC3D_CASES = sorted(p.stem for p in GOLDEN.glob("rfc3d_*.npz"))


def load_rfc3d(name):
    import oracle as O
    z = np.load(GOLDEN / f"{name}.npz")
    P = O.RollingProblem(int(z["nc"]), z["rowptr"], z["colidx"], z["blocks"], z["q"], z["mu"], z["mur"])
    return P, {k: z[k] for k in z.files}


def test_fixture_set():
    assert len(RFC3D_CASES) == 6


@pytest.mark.parametrize("case", RFC3D_CASES)
def test_port_reproduces_reference(case):
    import oracle as O
    P, g = load_rfc3d(case)
    for suffix, maxiter in (("", 10000), ("20", 20)):
        res = O.rfc3d_nsgs_port(P, tol=1e-8, maxiter=maxiter, trace_cap=maxiter)
        assert res.info == int(g["info" + suffix])
        assert res.iterations == int(g["iterations" + suffix])
        assert res.error == float(g["error" + suffix])
        np.testing.assert_array_equal(res.r, g["r" + suffix])
        np.testing.assert_array_equal(res.u, g["u" + suffix])
        np.testing.assert_array_equal(res.trace, g["trace" + suffix])


@pytest.mark.parametrize("case", RFC3D_CASES)
def test_port_compute_error(case):
    import oracle as O
    P, g = load_rfc3d(case)
    e, u = O.rfc3d_compute_error_port(P, g["r"])
    np.testing.assert_array_equal(u, g["u"])
    assert e == pytest.approx(float(g["error"]), rel=1e-14, abs=0)


def test_port_order_is_a_permuted_sweep():
    import oracle as O
    P, _ = load_rfc3d("rfc3d_rockfall_21_54029")
    ident = np.arange(P.nc, dtype=np.int32)
    a = O.rfc3d_nsgs_port(P, tol=0.0, maxiter=15)
    b = O.rfc3d_nsgs_port(P, tol=0.0, maxiter=15, order=ident)
    c = O.rfc3d_nsgs_port(P, tol=0.0, maxiter=15, order=ident[::-1].copy())
    np.testing.assert_array_equal(a.r, b.r)
    assert not np.array_equal(a.r, c.r)


@pytest.mark.parametrize("case", ["rfc3d_rockfall_14_25792", "rfc3d_RFC3D_cube_1"])
def test_port_matches_reference_library(case):
    """Direct run of the reference library (when built here) from a nonzero
    start, with the same random reaction on both."""
    import oracle as O
    if not O.ref_available():
        pytest.skip("oracle/_ref is not built here")
    P, _ = load_rfc3d(case)
    r0 = np.abs(np.random.default_rng(5).standard_normal(5 * P.nc)) * 1e-3
    a = O.rfc3d_nsgs_ref(P, r0=r0, tol=1e-9, maxiter=300, trace_cap=300)
    b = O.rfc3d_nsgs_port(P, r0=r0, tol=1e-9, maxiter=300, trace_cap=300)
    assert (a.info, a.iterations, a.error) == (b.info, b.iterations, b.error)
    np.testing.assert_array_equal(a.r, b.r)
    np.testing.assert_array_equal(a.trace, b.trace)
    for k in range(P.nnzb):
        blk = np.ascontiguousarray(P.blocks[k])
        assert O.ref().ref_rfc3d_max_eig(blk) == O.port().oracle_rfc3d_max_eig(blk)


def tiled(P, copies: int, seed: int):
    """`copies` independent copies of a rolling problem along the diagonal of
    W, each with q scaled by a seeded factor in [0.9, 1.1] (a larger problem
    with the fixture's block structure)."""
    import oracle as O
    g = np.random.default_rng(seed)
    nc, nb = P.nc, P.nnzb
    rp = [0]
    for c in range(copies):
        rp.extend((P.rowptr[1:] + c * nb).tolist())
    rowptr = np.asarray(rp, np.int64)
    colidx = np.concatenate([P.colidx + c * nc for c in range(copies)]).astype(np.int64)
    blocks = np.tile(P.blocks, (copies, 1))
    scale = np.repeat(g.uniform(0.9, 1.1, copies), 5 * nc)
    q = np.tile(P.q, copies) * scale
    return O.RollingProblem(copies * nc, rowptr, colidx, blocks, q, np.tile(P.mu, copies), np.tile(P.mur, copies))


def test_tiled_problem_is_independent_copies():
    import oracle as O
    P, _ = load_rfc3d("rfc3d_rockfall_14_25792")
    T = tiled(P, 3, 1)
    assert T.nc == 3 * P.nc and T.nnzb == 3 * P.nnzb
    res = O.rfc3d_nsgs_port(T, tol=0.0, maxiter=5)
    for c in range(3):
        Pc = O.RollingProblem(P.nc, P.rowptr, P.colidx, P.blocks, T.q[5 * c * P.nc:5 * (c + 1) * P.nc], P.mu, P.mur)
        one = O.rfc3d_nsgs_port(Pc, tol=0.0, maxiter=5)
        np.testing.assert_array_equal(res.r[5 * c * P.nc:5 * (c + 1) * P.nc], one.r)


# ----------------------------------------------------------------------------
# host side of the GPU solver (no device call)
# ----------------------------------------------------------------------------
def test_options_defaults(built_lib):
    import siconos_gb300.numerics as sn
    o = sn.SolverOptions(sn.SICONOS_ROLLING_FRICTION_3D_NSGS_GPU)
    assert o.solverId == 3020
    assert o.iparam[0] == 1000 and o.dparam[0] == 1e-4
    assert o.iparam[13] == 2 and o.iparam[2] == 1 and o.dparam[11] == 10.0
    loc = o.internalSolvers[0]
    assert loc.solverId == sn.SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN
    assert loc.iparam[0] == 10 and loc.dparam[0] == 1e-12
    assert loc.iparam[9] == 1 and loc.iparam[10] == 4  # spectral-norm rho, natural map


def _rproblem(sn, q0=-1.0):
    W = sn.SparseBlockMatrix(1, [0, 1], [0], np.eye(5).reshape(1, 25), block_size=5)
    return sn.RollingFrictionContactProblem(5, 1, W, np.array([q0, 0.1, 0.0, 0.05, 0.0]), np.array([0.5]),
                                            np.array([0.1]))


def test_driver_checks_and_trivial_case(built_lib):
    import siconos_gb300.numerics as sn
    o = sn.SolverOptions(sn.SICONOS_ROLLING_FRICTION_3D_NSGS_GPU)
    P = _rproblem(sn, q0=0.2)
    r, u = np.ones(5), np.zeros(5)
    assert sn.rolling_friction_3d_driver(P, r, u, o) == 0
    np.testing.assert_array_equal(r, 0.0)
    np.testing.assert_array_equal(u, P._q)
    P = _rproblem(sn)
    o.iparam[11] = 1  # shuffle
    assert sn.rolling_friction_3d_driver(P, r, u, o) == sn.NUMERICS_ERR_NOT_IMPLEMENTED
    o3 = sn.SolverOptions(sn.SICONOS_FRICTION_3D_NSGS_GPU)
    assert sn.rolling_friction_3d_driver(P, r, u, o3) == sn.NUMERICS_ERR_INVALID_SOLVER
