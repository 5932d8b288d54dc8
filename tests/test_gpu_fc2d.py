"""GPU 2D NSGS (SICONOS_FRICTION_2D_NSGS_GPU) against the oracle.

The GPU sweep visits contacts in colour order; the oracle run with that
visiting order is the same sequential Gauss-Seidel, so reactions and
velocities agree bit for bit (FP64, no contraction, the reference's operation
order).  Errors are sums over contacts whose order differs (a block reduction
on the device, index order in the oracle): relative 1e-12.  Through the
driver, which keeps the reference's defaults, every fixture the reference
solves is solved to its tolerance."""
import numpy as np
import pytest

from test_fc2d_oracle import FC2D_CASES, load_fc2d

pytestmark = pytest.mark.gpu
RTOL = 1e-12


@pytest.fixture(scope="module")
def sn(built_lib):
    import siconos_gb300.numerics as sn
    try:
        c = sn.Fc2dContext(1, [0, 1], [0], [1.0, 0.0, 0.0, 1.0], [-1.0, 0.0], [0.5])
    except (RuntimeError, ValueError) as e:
        pytest.fail(f"no usable CUDA device for a -m gpu run: {e}")
    c.close()
    return sn


def _ctx(sn, P, colouring=0):
    return sn.Fc2dContext(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu, colouring)


def _order(colour):
    return np.argsort(colour, kind="stable").astype(np.int32)


@pytest.mark.parametrize("case", FC2D_CASES)
def test_fixed_sweeps_bit_exact(sn, case):
    import oracle as O
    P, _ = load_fc2d(case)
    ctx = _ctx(sn, P)
    ncol, colour = ctx.colours()
    assert ncol >= 1
    # colour classes are independent sets of the conflict graph
    rows = np.repeat(np.arange(P.nc), np.diff(P.rowptr))
    off = rows != P.colidx
    assert not np.any(colour[rows[off]] == colour[P.colidx[off]])
    n = 15
    res = ctx.solve(0.0, n)
    r, u = ctx.get_r_u()
    ref = O.fc2d_nsgs_port(P, tol=0.0, maxiter=n, order=_order(colour), trace_cap=n)
    assert res["iterations"] == ref.iterations == n
    assert res["info"] == ref.info == 1
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    np.testing.assert_allclose(ctx.trace(n), ref.trace, rtol=RTOL, atol=0)
    ctx.close()


@pytest.mark.parametrize("case", FC2D_CASES)
def test_converged_solve_matches_oracle(sn, case):
    import oracle as O
    P, g = load_fc2d(case)
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    res = ctx.solve(1e-5, 10000)
    r, u = ctx.get_r_u()
    ref = O.fc2d_nsgs_port(P, tol=1e-5, maxiter=10000, order=_order(colour))
    assert (res["info"], res["iterations"]) == (ref.info, ref.iterations)
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    # the colour order solves what the reference's natural order solves
    assert res["info"] == int(g["info"])
    ctx.close()


@pytest.mark.parametrize("case", FC2D_CASES)
def test_driver_solves_fixture(sn, case):
    """Through fc2d_driver with its defaults at the reference tests' settings
    (tol 1e-5, 10000 iterations), from zero."""
    import oracle as O
    P, g = load_fc2d(case)
    W = sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks, block_size=2)
    prob = sn.FrictionContactProblem(2, P.nc, W, P.q.copy(), P.mu.copy())
    o = sn.SolverOptions(sn.SICONOS_FRICTION_2D_NSGS_GPU)
    o.iparam[sn.SICONOS_IPARAM_MAX_ITER] = 10000
    o.dparam[sn.SICONOS_DPARAM_TOL] = 1e-5
    r, u = np.zeros(2 * P.nc), np.zeros(2 * P.nc)
    info = sn.fc2d_driver(prob, r, u, o)
    assert info == int(g["info"]) == 0
    assert o.dparam[sn.SICONOS_DPARAM_RESIDU] < 1e-5
    e, u_chk = O.fc2d_compute_error_port(P, r)
    assert e == pytest.approx(o.dparam[sn.SICONOS_DPARAM_RESIDU], rel=RTOL, abs=0)
    np.testing.assert_array_equal(u, u_chk)
    # a second call on the same options reuses the device W and starts from r
    it1 = int(o.iparam[sn.SICONOS_IPARAM_ITER_DONE])
    assert sn.fc2d_driver(prob, r, u, o) == 0
    assert int(o.iparam[sn.SICONOS_IPARAM_ITER_DONE]) <= it1


@pytest.mark.parametrize("shape", [(1, 32, 1), (1, 512, 2), (2, 64, 1), (8, 128, 2), (16, 32, 1), (16, 32, 2),
                                   (16, 512, 1), (16, 128, 2), (-1, 256, 1), (-1, 32, 1)])
def test_launch_shape_does_not_change_iterates(sn, shape):
    """Any cluster size (or a cooperative grid, -1), block size and place of
    the reactions gives the same reaction bits; the errors differ only by the
    order of their sums."""
    import oracle as O
    P, _ = load_fc2d("fc2d_fc2d_granularflowonwall_02020_00213")
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    try:
        got = ctx.set_launch(*shape)
    except RuntimeError as e:
        assert "does not fit" in str(e)
        pytest.skip(f"cluster shape {shape} cannot be resident on this device")
    if shape[0] < 0:
        assert got[0] < 0 and got[1:] == shape[1:]  # a grid of -got[0] blocks
    else:
        assert got == shape
    res = ctx.solve(0.0, 25)
    r, u = ctx.get_r_u()
    ref = O.fc2d_nsgs_port(P, tol=0.0, maxiter=25, order=_order(colour))
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    e = ctx.compute_error(float(np.sqrt(np.sum(P.q * P.q))))
    assert e == pytest.approx(ref.error, rel=RTOL, abs=0)
    # a second solve continues from the reactions the first one left
    ctx.solve(0.0, 3)
    r2, _ = ctx.get_r_u()
    ref2 = O.fc2d_nsgs_port(P, r0=ref.r, tol=0.0, maxiter=3, order=_order(colour))
    np.testing.assert_array_equal(r2, ref2.r)
    with pytest.raises(RuntimeError):
        ctx.set_launch(17, 0)
    with pytest.raises(RuntimeError):
        ctx.set_launch(1, 100)
    with pytest.raises(RuntimeError):
        ctx.set_launch(1, 32, 3)
    ctx.close()


def test_compute_error_matches_oracle(sn):
    import oracle as O
    P, g = load_fc2d("fc2d_FrictionContactProblem00237")
    W = sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks, block_size=2)
    prob = sn.FrictionContactProblem(2, P.nc, W, P.q, P.mu)
    r = g["r20"].copy()
    u = np.zeros_like(r)
    nq = float(np.sqrt(np.sum(P.q * P.q)))
    info, e = sn.fc2d_compute_error(prob, r, u, 1e-5, nq)
    e_ref, u_ref = O.fc2d_compute_error_port(P, r)
    np.testing.assert_array_equal(u, u_ref)
    assert e == pytest.approx(e_ref, rel=RTOL, abs=0)
    assert info == (1 if e > 1e-5 else 0)


def test_error_evaluation_modes(sn):
    """LIGHT stops at the first sweep whose light error is below tol and
    reports it; FULL and ADAPTIVE evaluate nothing in fc2d_nsgs (all sweeps,
    error INFINITY, info 1); through the driver the defaults come back."""
    import oracle as O
    P, _ = load_fc2d("fc2d_FC2D_SliderCrankLagrangian00001")
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    ref = O.fc2d_nsgs_port(P, tol=0.0, maxiter=400, order=_order(colour), trace_cap=400)
    tol = 1e-6
    first = int(np.argmax(ref.trace < tol)) + 1
    assert ref.trace[first - 1] < tol
    ctx.set_r(np.zeros(2 * P.nc))
    res = ctx.solve(tol, 400, sn.SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT)
    assert res["iterations"] == first
    assert res["error"] == pytest.approx(ref.trace[first - 1], rel=RTOL, abs=0)
    assert res["info"] == 0
    for mode in (sn.SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_FULL, 3):
        ctx.set_r(np.zeros(2 * P.nc))
        res = ctx.solve(tol, 37, mode)
        assert res["iterations"] == 37 and res["info"] == 1 and np.isinf(res["error"])
    ctx.close()


def test_singular_diagonal_and_bad_structure(sn):
    rowptr = np.array([0, 1, 2], np.int64)
    colidx = np.array([0, 1], np.int64)
    blocks = np.array([[1.0, 0.0, 0.0, 1.0], [1.0, 1.0, 1.0, 1.0]])
    ctx = sn.Fc2dContext(2, rowptr, colidx, blocks, [-1.0, 0.1, -1.0, 0.2], [0.3, 0.3])
    res = ctx.solve(1e-5, 100)
    assert res["info"] == 1 and res["iterations"] == 0 and np.isinf(res["error"])
    ctx.close()
    with pytest.raises(ValueError, match="diagonal"):
        sn.Fc2dContext(2, rowptr, np.array([1, 0], np.int64), blocks, [-1.0, 0.1, -1.0, 0.2], [0.3, 0.3])
    with pytest.raises(ValueError, match="out of range"):
        sn.Fc2dContext(2, rowptr, np.array([0, 5], np.int64), blocks, [-1.0, 0.1, -1.0, 0.2], [0.3, 0.3])


def test_dense_storage_problem(sn):
    """W given as a dense column-major matrix (NM_DENSE): the blocks holding a
    nonzero are kept, the solve equals the sparse-block one."""
    import oracle as O
    P, _ = load_fc2d("fc2d_FrictionContactProblem00071")
    W = sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks, block_size=2)
    dense = W.todense()
    res = {}
    for kind, M in (("sbm", W), ("dense", dense)):
        prob = sn.FrictionContactProblem(2, P.nc, M, P.q.copy(), P.mu.copy())
        o = sn.SolverOptions(sn.SICONOS_FRICTION_2D_NSGS_GPU)
        o.dparam[sn.SICONOS_DPARAM_TOL] = 1e-5
        o.iparam[sn.SICONOS_IPARAM_MAX_ITER] = 10000
        r, u = np.zeros(2 * P.nc), np.zeros(2 * P.nc)
        info = sn.fc2d_driver(prob, r, u, o)
        res[kind] = (info, int(o.iparam[sn.SICONOS_IPARAM_ITER_DONE]), r)
    assert res["sbm"][0] == res["dense"][0] == 0
    e, _ = O.fc2d_compute_error_port(P, res["dense"][2])
    assert e < 1e-5


def test_q_change_reuses_layout(sn):
    """New q and mu on the same W: the context's answer equals a fresh
    context's."""
    P, _ = load_fc2d("fc2d_FrictionContactProblem00727")
    ctx = _ctx(sn, P)
    q2 = P.q * 1.5
    mu2 = P.mu * 0.5
    ctx.set_q_mu(q2, mu2)
    a = ctx.solve(1e-5, 10000)
    ra, _ = ctx.get_r_u()
    import oracle as O
    P2 = O.Problem(P.nc, P.rowptr, P.colidx, P.blocks, q2, mu2, 2)
    fresh = _ctx(sn, P2)
    b = fresh.solve(1e-5, 10000)
    rb, _ = fresh.get_r_u()
    assert a["iterations"] == b["iterations"]
    np.testing.assert_array_equal(ra, rb)
    ctx.close()
    fresh.close()


@pytest.mark.parametrize("case", ["fc2d_FC2D_SliderCrankLagrangian00000", "fc2d_fc2d_granularflowonwall_02020_00213"])
def test_per_colour_design_solves_fixture(sn, case):
    """The reference's per-colour GPU design (the comparator of the bench)
    reaches the tolerance; its error is fc2d_compute_error of its reaction and
    its iterates track the oracle's colour-ordered sweep to rounding."""
    import oracle as O
    P, g = load_fc2d(case)
    pc = sn.Fc2dPerColour(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu)
    res = pc.solve(1e-5, 10000)
    r, u = pc.get_r_u()
    assert res["info"] == 0 and res["error"] < 1e-5
    e, u_ref = O.fc2d_compute_error_port(P, r)
    assert e == pytest.approx(res["error"], rel=1e-14, abs=0)
    np.testing.assert_array_equal(u, u_ref)
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    ctx.close()
    short = pc.solve(0.0, 5)
    r5, _ = pc.get_r_u()
    ref = O.fc2d_nsgs_port(P, tol=0.0, maxiter=5, order=_order(colour))
    assert short["iterations"] == 5
    np.testing.assert_allclose(r5, ref.r, rtol=0, atol=1e-9 * max(1.0, np.abs(ref.r).max()))
    pc.close()


@pytest.mark.parametrize("variant", ["graph", "blocklegacy"])
def test_reference_kernel_image(sn, variant):
    """The reference's own local-solve kernels, compiled from their sources
    into oracle/_ref by oracle/build_ref.py, in the comparator's sweep:
    fc2d_nsgs_graph_permut_cuda.cu:213-300 after scalar-CSR SpMVs in a graph,
    and fc2d_nsgs_graph_permut_cuda_blocklegacy.cu:215-300 after a BSR matvec
    per colour (:533-567).  After 5 sweeps the iterate equals the comparator
    kernel's to rounding (the reference build contracts products into FMAs,
    the comparator does not; the BSR matvec sums in another order), and from
    zero the solve reaches tol 1e-5 in the comparator's sweep count to within
    2 %, with fc2d_compute_error of its reaction below the tolerance."""
    from pathlib import Path
    import oracle as O
    name = "fc2d_nsgs_graph_permut_cuda" + ("_blocklegacy" if variant == "blocklegacy" else "")
    img = Path(O.__file__).resolve().parent / "_ref" / f"{name}.fatbin"
    if not img.exists():
        pytest.skip("the reference's fc2d CUDA image was not built (no reference checkout)")
    P, _ = load_fc2d("fc2d_fc2d_granularflowonwall_02020_00213")
    pc = sn.Fc2dPerColour(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu)
    rk = sn.Fc2dPerColour(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu)
    try:
        rk.use_kernel_file(img)
        if variant == "blocklegacy":
            rk.use_bsr(True)
        a = pc.solve(0.0, 5)
        b = rk.solve(0.0, 5)
        assert a["iterations"] == b["iterations"] == 5
        ra, _ = pc.get_r_u()
        rb, _ = rk.get_r_u()
        np.testing.assert_allclose(rb, ra, rtol=0, atol=1e-10 * max(1.0, np.abs(ra).max()))
        a = pc.solve(1e-5, 10000)
        b = rk.solve(1e-5, 10000)
        assert a["info"] == 0 and b["info"] == 0
        assert abs(b["iterations"] - a["iterations"]) <= max(2, 0.02 * a["iterations"])
        rb, _ = rk.get_r_u()
        e, _ = O.fc2d_compute_error_port(P, rb)
        assert e < 1e-5 and e == pytest.approx(b["error"], rel=1e-14, abs=0)
        with pytest.raises(RuntimeError):
            rk.use_kernel_file(img.with_name("no_such_image.fatbin"))
    finally:
        pc.close()
        rk.close()


def test_per_colour_bsr_matches_csr(sn):
    """The comparator's block-sparse sweep (BSR matvec per colour, diagonal
    blocks kept with zero values) and its scalar-CSR sweep give the same
    iterates to rounding, and switching back restores the graph sweep."""
    P, _ = load_fc2d("fc2d_FrictionContactProblem00727")
    pc = sn.Fc2dPerColour(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu)
    try:
        a = pc.solve(0.0, 10)
        ra, _ = pc.get_r_u()
        pc.use_bsr(True)
        b = pc.solve(0.0, 10)
        rb, _ = pc.get_r_u()
        assert a["iterations"] == b["iterations"] == 10
        np.testing.assert_allclose(rb, ra, rtol=0, atol=1e-10 * max(1.0, np.abs(ra).max()))
        pc.use_bsr(False)
        c = pc.solve(0.0, 10)
        rc, _ = pc.get_r_u()
        np.testing.assert_array_equal(rc, ra)
    finally:
        pc.close()


def test_fp32_phase_bit_exact(sn):
    """The FP32 phase of the mixed mode is the single-precision sweep of the
    oracle (oracle_fc2d_sweeps_f32) in colour order, bit for bit: 20 FP32
    sweeps (switch never reached), no FP64 budget left, the FP64 error of
    that iterate."""
    import oracle as O
    P, _ = load_fc2d("fc2d_fc2d_granularflowonwall_02020_00213")
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    ctx.set_precision(0, 1e-30, 1 << 20)
    res = ctx.solve(1e-5, 20)
    assert ctx.last_sweeps() == (20, 0) and res["iterations"] == 20
    r, u = ctx.get_r_u()
    r32 = O.fc2d_sweeps_f32_port(P, np.zeros(2 * P.nc), 20, order=_order(colour))
    np.testing.assert_array_equal(r, r32)
    e, u_ref = O.fc2d_compute_error_port(P, r32)
    np.testing.assert_array_equal(u, u_ref)
    assert res["error"] == pytest.approx(e, rel=RTOL, abs=0)
    ctx.close()


@pytest.mark.parametrize("case", FC2D_CASES)
def test_mixed_precision_solve(sn, case):
    """FP32 sweeps then the reference's FP64 loop: the result is the oracle's
    FP64 loop started from the oracle's FP32 iterate after the same number of
    FP32 sweeps, bit for bit, and it meets the tolerance the reference
    meets."""
    import oracle as O
    P, g = load_fc2d(case)
    ctx = _ctx(sn, P)
    _, colour = ctx.colours()
    order = _order(colour)
    ctx.set_precision(0)
    res = ctx.solve(1e-5, 10000)
    s32, s64 = ctx.last_sweeps()
    assert s32 + s64 == res["iterations"] and s32 >= 1
    r, u = ctx.get_r_u()
    r32 = O.fc2d_sweeps_f32_port(P, np.zeros(2 * P.nc), s32, order=order)
    ref = O.fc2d_nsgs_port(P, r0=r32, tol=1e-5, maxiter=10000 - s32, order=order)
    assert (res["info"], s64) == (ref.info, ref.iterations)
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    assert res["info"] == int(g["info"]) == 0 and res["error"] < 1e-5
    ctx.close()


def test_large_problem_runs_on_a_grid(sn):
    """8 copies of the 7,002-contact granular problem (56,016 contacts): the
    largest colour exceeds a full cluster, so the solve runs on a cooperative
    grid over every SM; same bits as the oracle in colour order."""
    import oracle as O
    from test_fc2d_oracle import tiled2d
    P, _ = load_fc2d("fc2d_fc2d_granularflowonwall_07002_00801")
    T = tiled2d(P, 8, 5)
    ctx = _ctx(sn, T)
    cs, nt, rx = ctx.launch_shape()
    assert cs < 0 and rx == 1
    _, colour = ctx.colours()
    res = ctx.solve(0.0, 12)
    r, u = ctx.get_r_u()
    ref = O.fc2d_nsgs_port(T, tol=0.0, maxiter=12, order=_order(colour))
    np.testing.assert_array_equal(r, ref.r)
    np.testing.assert_array_equal(u, ref.u)
    assert res["error"] == pytest.approx(ref.error, rel=RTOL, abs=0)
    ctx.set_precision(0, 1e-30, 1 << 20)
    ctx.set_r(np.zeros(2 * T.nc))
    ctx.solve(1e-5, 12)
    r32, _ = ctx.get_r_u()
    np.testing.assert_array_equal(r32, O.fc2d_sweeps_f32_port(T, np.zeros(2 * T.nc), 12, order=_order(colour)))
    ctx.close()
