"""GPU rolling-friction NSGS (SICONOS_ROLLING_FRICTION_3D_NSGS_GPU) against the
oracle.  The GPU visits contacts in colour order; the oracle run in that
order is the same sequential Gauss-Seidel, so reactions and velocities agree
bit for bit (FP64 without contraction, the reference's operation order; rho
from the same Jacobi eigenvalue iteration on the host).  Errors are sums over
contacts in another order: relative 1e-12."""
import numpy as np
import pytest

from test_rfc3d_oracle import RFC3D_CASES, load_rfc3d, tiled

pytestmark = pytest.mark.gpu
RTOL = 1e-12


@pytest.fixture(scope="module")
def sn(built_lib):
    import siconos_gb300.numerics as sn
    try:
        c = sn.RollingContext(1, [0, 1], [0], np.eye(5).reshape(-1), [-1.0, 0, 0, 0, 0], [0.5], [0.1])
    except (RuntimeError, ValueError) as e:
        pytest.fail(f"no usable CUDA device for a -m gpu run: {e}")
    c.close()
    return sn


def _ctx(sn, P):
    return sn.RollingContext(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu, P.mur)


def _order(colour):
    return np.argsort(colour, kind="stable").astype(np.int32)


@pytest.mark.parametrize("case", RFC3D_CASES)
def test_rho_and_fixed_sweeps_bit_exact(sn, case):
    import oracle as O
    P, _ = load_rfc3d(case)
    ctx = _ctx(sn, P)
    # rho = 1 / largest eigenvalue of each diagonal block, as the oracle
    rho = ctx.rho()
    for i in range(P.nc):
        k = [kk for kk in range(P.rowptr[i], P.rowptr[i + 1]) if P.colidx[kk] == i][0]
        assert rho[i] == 1.0 / O.port().oracle_rfc3d_max_eig(np.ascontiguousarray(P.blocks[k]))
    _, colour = ctx.colours()
    n = 15
    res = ctx.solve(0.0, n)
    r, u = ctx.get_r_u()
    ref = O.rfc3d_nsgs_port(P, tol=0.0, maxiter=n, order=_order(colour), trace_cap=n)
    assert res["iterations"] == ref.iterations == n
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    np.testing.assert_allclose(ctx.trace(n), ref.trace, rtol=RTOL, atol=0)
    ctx.close()


@pytest.mark.parametrize("case", RFC3D_CASES)
def test_converged_solve_matches_oracle(sn, case):
    import oracle as O
    P, g = load_rfc3d(case)
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    res = ctx.solve(1e-8, 10000)
    r, u = ctx.get_r_u()
    ref = O.rfc3d_nsgs_port(P, tol=1e-8, maxiter=10000, order=_order(colour))
    assert (res["info"], res["iterations"]) == (ref.info, ref.iterations)
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    assert res["info"] == int(g["info"])
    ctx.close()


@pytest.mark.parametrize("case", ["rfc3d_rockfall_14_25792", "rfc3d_RFC3D_cube_1"])
@pytest.mark.parametrize("storage", ["sbm", "dense"])
def test_driver_solves_fixture(sn, case, storage):
    """Through rolling_friction_3d_driver with its defaults (tol 1e-8), W
    sparse-block or dense; the result meets the tolerance the reference
    meets, and u is W r + q as the oracle forms it."""
    import oracle as O
    P, g = load_rfc3d(case)
    W = sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks, block_size=5)
    M = W if storage == "sbm" else W.todense()
    prob = sn.RollingFrictionContactProblem(5, P.nc, M, P.q.copy(), P.mu.copy(), P.mur.copy())
    o = sn.SolverOptions(sn.SICONOS_ROLLING_FRICTION_3D_NSGS_GPU)
    o.iparam[sn.SICONOS_IPARAM_MAX_ITER] = 10000
    o.dparam[sn.SICONOS_DPARAM_TOL] = 1e-8
    r, u = np.zeros(5 * P.nc), np.zeros(5 * P.nc)
    info = sn.rolling_friction_3d_driver(prob, r, u, o)
    assert info == int(g["info"]) == 0
    assert o.dparam[sn.SICONOS_DPARAM_RESIDU] < 1e-8
    e, u_chk = O.rfc3d_compute_error_port(P, r)
    np.testing.assert_array_equal(u, u_chk)
    assert e == pytest.approx(o.dparam[sn.SICONOS_DPARAM_RESIDU], rel=RTOL, abs=0)
    e2, u2 = np.zeros(1), np.zeros(5 * P.nc)
    rc, err = sn.rolling_friction_3d_compute_error(prob, r.copy(), u2, 1e-8, float(np.linalg.norm(P.q)))
    assert rc == 0 and err == pytest.approx(e, rel=RTOL, abs=0)
    np.testing.assert_array_equal(u2, u_chk)


def test_tiled_problem_bit_exact(sn):
    """200 independent copies of the 21-contact rockfall problem (4,200
    contacts): many blocks in the cooperative grid, same bits as the oracle."""
    import oracle as O
    P, _ = load_rfc3d("rfc3d_rockfall_21_54029")
    T = tiled(P, 200, 3)
    ctx = _ctx(sn, T)
    _, colour = ctx.colours()
    res = ctx.solve(0.0, 30)
    r, u = ctx.get_r_u()
    ref = O.rfc3d_nsgs_port(T, tol=0.0, maxiter=30, order=_order(colour))
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    ctx.close()


def test_bad_structure_is_rejected(sn):
    with pytest.raises(ValueError, match="diagonal"):
        sn.RollingContext(2, [0, 1, 2], [1, 0], np.tile(np.eye(5).reshape(-1), 2), np.zeros(10), [0.5, 0.5],
                          [0.1, 0.1])
    with pytest.raises(ValueError, match="friction"):
        sn.RollingContext(1, [0, 1], [0], np.eye(5).reshape(-1), -np.ones(5), [-0.5], [0.1])


@pytest.mark.parametrize("case", ["rfc3d_rockfall_14_25792", "rfc3d_rockfall_21_54029", "rfc3d_RFC3D_cube_1"])
def test_mixed_precision_reaches_tolerance(sn, case):
    """FP32 sweeps, then the reference's FP64 loop from their iterate: the
    same tolerance as the FP64 solver, the error the oracle computes for the
    final reaction, the sweeps split between the precisions."""
    import oracle as O
    P, g = load_rfc3d(case)
    ctx = _ctx(sn, P)
    ctx.set_precision(0)
    res = ctx.solve(1e-8, 10000)
    s32, s64 = ctx.last_sweeps()
    r, u = ctx.get_r_u()
    ctx.close()
    assert res["info"] == 0 and res["error"] < 1e-8
    assert s32 + s64 == res["iterations"] and s32 >= 1
    e, u_chk = O.rfc3d_compute_error_port(P, r)
    np.testing.assert_array_equal(u, u_chk)
    assert e == pytest.approx(res["error"], rel=RTOL, abs=0)


def test_mixed_precision_on_tiled_problem(sn):
    """Mixed precision on 200 copies of the rockfall problem: it meets the
    tolerance, and its FP64 part is the reference's loop from the FP32
    iterate, bit for bit the oracle's sweeps in colour order from it."""
    import oracle as O
    P, _ = load_rfc3d("rfc3d_rockfall_21_54029")
    T = tiled(P, 200, 3)
    ctx = _ctx(sn, T)
    _, colour = ctx.colours()
    ctx.set_precision(0, switch_tol=1e-5)
    res = ctx.solve(1e-8, 10000)
    s32, s64 = ctx.last_sweeps()
    r_mixed, _ = ctx.get_r_u()
    assert res["info"] == 0 and res["error"] < 1e-8 and s32 > 0 and s64 > 0
    # the FP32 iterate alone: the same FP32 sweeps within a budget of s32
    ctx.set_r(np.zeros(5 * T.nc))
    ctx.solve(1e-8, s32)
    assert ctx.last_sweeps() == (s32, 0)
    r32, _ = ctx.get_r_u()
    ctx.close()
    ref = O.rfc3d_nsgs_port(T, r0=r32, tol=1e-8, maxiter=10000 - s32, order=_order(colour))
    assert ref.iterations == s64
    np.testing.assert_array_equal(r_mixed, ref.r)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)


def test_precision_arguments_are_checked(sn):
    P, _ = load_rfc3d("rfc3d_RFC3D_cube_1")
    ctx = _ctx(sn, P)
    with pytest.raises(RuntimeError):
        ctx.set_precision(2)
    with pytest.raises(RuntimeError):
        ctx.set_precision(0, switch_tol=-1.0)
    ctx.close()
