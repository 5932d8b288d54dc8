"""The GPU global FC3D NSGS (include/gfc3dgpu.h) against the reference's
gfc3d_nsgs: r, u and v bit for bit with the reference's golden outputs and
with the oracle (which is pinned to the reference bit for bit), on the
reference's global test problems and on the sphere lattice in global form
up to the benchmark's 60x60x30 scene.  The error's norms are reduced in
another order on the GPU: the error agrees to 1e-12 relative."""
import numpy as np
import pytest

from conftest import GOLDEN
from test_gfc3d_oracle import GCASES, load_gcase

pytestmark = pytest.mark.gpu

ERR_RTOL = 1e-12  # FP64 norms summed in a fixed GPU order instead of sequentially


def _ctx(P):
    import siconos_gb300.numerics as sn
    return sn.Gfc3dContext.from_problem(P)


def _close(a, b):
    return abs(a - b) <= ERR_RTOL * max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("case", GCASES)
@pytest.mark.parametrize("setting", [("", 1e-8, 1000), ("_default", 1e-4, 10000), ("20", 0.0, 20)])
def test_context_equals_reference(gpu, case, setting):
    import oracle as O
    tag, tol, it = setting
    P, g = load_gcase(case)
    ref = O.gfc3d_nsgs_port(P, tol=tol, maxiter=it)
    c = _ctx(P)
    try:
        c.set_start()
        res = c.solve(tol, it)
        r, u, v = c.get()
        tr = c.trace(it)
    finally:
        c.close()
    assert res["info"] == int(g["info" + tag])
    assert res["iterations"] == ref.iterations
    assert _close(res["error"], float(g["error" + tag])), (res["error"], float(g["error" + tag]))
    assert np.array_equal(r, g["r" + tag])
    assert np.array_equal(u, g["u" + tag])
    assert np.array_equal(v, g["v" + tag])
    assert len(tr) == ref.iterations


@pytest.mark.parametrize("case", ["gfc3d_GFC3D_TwoRods1", "gfc3d_GFC3D_OneContact", "gfc3d_lattice_5x5x6_s1"])
@pytest.mark.parametrize("freq", [3, 7])
def test_error_evaluation_frequency(gpu, case, freq):
    import oracle as O
    P, _ = load_gcase(case)
    ref = O.gfc3d_nsgs_port(P, tol=1e-6, maxiter=500, freq=freq, trace_cap=500)
    c = _ctx(P)
    try:
        res = c.solve(1e-6, 500, freq)
        r, u, v = c.get()
        tr = c.trace(500)
    finally:
        c.close()
    assert res["info"] == ref.info and res["iterations"] == ref.iterations
    assert _close(res["error"], ref.error)
    assert np.array_equal(r, ref.r) and np.array_equal(u, ref.u) and np.array_equal(v, ref.v)
    np.testing.assert_allclose(tr, ref.trace, rtol=ERR_RTOL)


def test_start_zero_budget_and_continuation(gpu):
    """A given start, max_iter 0 (no iteration: the start's error, info -1),
    then a solve from that start, then a second solve continuing from the
    first one's iterate."""
    import oracle as O
    P, g = load_gcase("gfc3d_GFC3D_TwoRods1")
    r0, v0 = g["r20"] * 0.9, g["v20"] * 1.1
    c = _ctx(P)
    try:
        c.set_start(r0, v0)
        res = c.solve(1e-8, 0)
        r, u, v = c.get()
        ref = O.gfc3d_nsgs_port(P, r0=r0, v0=v0, tol=1e-8, maxiter=0)
        assert res["info"] == -1 and res["iterations"] == 0
        assert _close(res["error"], ref.error) and np.array_equal(u, ref.u) and np.array_equal(v, v0)
        assert np.array_equal(r, r0)
        res = c.solve(0.0, 3)
        ref = O.gfc3d_nsgs_port(P, r0=r0, v0=v0, tol=0.0, maxiter=3)
        r, u, v = c.get()
        assert res["iterations"] == 3 and np.array_equal(r, ref.r) and np.array_equal(v, ref.v)
        res = c.solve(1e-8, 1000)
        ref = O.gfc3d_nsgs_port(P, r0=ref.r, v0=ref.v, tol=1e-8, maxiter=1000)
        r, u, v = c.get()
        assert res["info"] == ref.info == 0 and res["iterations"] == ref.iterations
        assert np.array_equal(r, ref.r) and np.array_equal(u, ref.u) and np.array_equal(v, ref.v)
        assert _close(c.compute_error(), ref.error)
    finally:
        c.close()


def _problem(P, storage):
    """The reference-facing problem with M and H dense or sparse-block."""
    import siconos_gb300.numerics as sn
    M, H = P.dense()
    if storage == "dense":
        Mm, Hm = np.asfortranarray(M), np.asfortranarray(H)
    else:
        # 3-dof row blocks (the last one shorter where n is not a multiple of 3)
        rs = [3] * (P.n // 3) + ([P.n % 3] if P.n % 3 else [])
        Mm = sn.BlockMatrix.from_dense(M, rs, rs)
        Hm = sn.BlockMatrix.from_dense(H, rs, [3] * P.nc)
    return sn.GlobalFrictionContactProblem(3, P.nc, Mm, Hm, P.q.copy(), P.b.copy(), P.mu.copy())


@pytest.mark.parametrize("storage", ["dense", "sparse_block"])
@pytest.mark.parametrize("case", ["gfc3d_GFC3D_TwoRods1", "gfc3d_GFC3D_Example1", "gfc3d_lattice_5x5x6_s1"])
def test_driver_through_c_abi(gpu, storage, case):
    """gfc3d_driver with the new solver id, host buffers: the reference's
    outputs (tol 1e-8, 1000 iterations)."""
    import siconos_gb300.numerics as sn
    P, g = load_gcase(case)
    prob = _problem(P, storage)
    o = sn.SolverOptions(sn.SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU)
    assert o.iparam[0] == 1000 and o.dparam[0] == 1e-4 and o.iparam[14] == 0
    o.iparam[0] = 1000
    o.dparam[0] = 1e-8
    r, u, v = np.zeros(3 * P.nc), np.zeros(3 * P.nc), np.zeros(P.n)
    info = sn.gfc3d_driver(prob, r, u, v, o)
    assert info == int(g["info"]), sn.last_error()
    assert _close(o.dparam[1], float(g["error"]))
    assert np.array_equal(r, g["r"]) and np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
    # the solver entry the registry binds, called again on the same options
    r[:] = 0
    v[:] = 0
    assert sn.gfc3d_nsgs_gpu(prob, r, u, v, o) == info
    assert np.array_equal(r, g["r"])
    e_info, e = sn.gfc3d_compute_error(prob, r, u, v, 1e-8, float(np.linalg.norm(P.q)))
    assert _close(e, float(g["error"])) and e_info == (1 if e > 1e-8 else 0)
    o.release()


def test_driver_no_contact(gpu):
    """No contact: globalVelocity = M^-1 q (gfc3d_driver.c:107-114)."""
    import oracle as O
    import siconos_gb300.numerics as sn
    P, _ = load_gcase("gfc3d_GFC3D_TwoRods1")
    M, _H = P.dense()
    prob = sn.GlobalFrictionContactProblem(3, 0, np.asfortranarray(M), np.zeros((P.n, 0), order="F"), P.q.copy(),
                                           np.zeros(0), np.zeros(0))
    o = sn.SolverOptions(sn.SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU)
    v = np.zeros(P.n)
    assert sn.gfc3d_driver(prob, np.zeros(0), np.zeros(0), v, o) == 0, sn.last_error()
    ref = O.gfc3d_nsgs_port(O.GlobalProblem(P.n, 0, P.Mp, P.Mi, P.Mx, np.zeros(P.n + 1, np.int64),
                                            np.zeros(0, np.int64), np.zeros(0), P.q, np.zeros(0), np.zeros(0)))
    assert np.array_equal(v, ref.v)
    np.testing.assert_allclose(v, np.linalg.solve(M, P.q), rtol=1e-10, atol=1e-12)
    o.release()


def test_singular_m_and_bad_input_rejected(gpu):
    import siconos_gb300.numerics as sn
    P, _ = load_gcase("gfc3d_GFC3D_Example1")
    Mx = P.Mx.copy()
    Mx[:] = 0.0
    with pytest.raises(ValueError, match="singular"):
        sn.Gfc3dContext(P.n, P.nc, P.Mp, P.Mi, Mx, P.Hp, P.Hi, P.Hx, P.q, P.b, P.mu)
    Hi = P.Hi.copy()
    Hi[0] = 3 * P.nc  # a column past H's last
    with pytest.raises(ValueError, match="out of range"):
        sn.Gfc3dContext(P.n, P.nc, P.Mp, P.Mi, P.Mx, P.Hp, Hi, P.Hx, P.q, P.b, P.mu)


def test_lattice_60x60x30_bit_exact(gpu):
    """The benchmark's scene (648,000 dofs, 320,400 contacts, 11.5 M entries
    of H): 25 iterations equal the oracle's bit for bit, then the errors of
    both agree."""
    import oracle as O
    from siconos_gb300 import scene
    P = O.lattice_global(60, 60, 30, seed=1)
    s = scene.lattice_global(60, 60, 30, seed=1)
    assert np.array_equal(s.Hx, P.Hx) and np.array_equal(s.q, P.q)
    ref = O.gfc3d_nsgs_port(P, tol=0.0, maxiter=25, trace_cap=25)
    c = _ctx(P)
    try:
        info = c.info()
        assert info["diagonal"] and info["components"] == P.n
        res = c.solve(0.0, 25)
        r, u, v = c.get()
        tr = c.trace(25)
    finally:
        c.close()
    assert res["info"] == 1 and res["iterations"] == 25
    assert np.array_equal(r, ref.r) and np.array_equal(u, ref.u) and np.array_equal(v, ref.v)
    np.testing.assert_allclose(tr, ref.trace, rtol=ERR_RTOL)


def test_lattice_solve_to_default_tolerance(gpu):
    """20x20x10 lattice to the reference's default 1e-4: same iterations,
    same iterate as the oracle."""
    import oracle as O
    P = O.lattice_global(20, 20, 10, seed=3, mu=0.3)
    ref = O.gfc3d_nsgs_port(P, tol=1e-4, maxiter=10000)
    c = _ctx(P)
    try:
        res = c.solve(1e-4, 10000)
        r, u, v = c.get()
    finally:
        c.close()
    assert ref.info == 0 and res["info"] == 0 and res["iterations"] == ref.iterations
    assert np.array_equal(r, ref.r) and np.array_equal(v, ref.v)
    assert _close(res["error"], ref.error)


def test_wait_timeout_is_an_error_and_the_context_recovers(gpu):
    """A one-poll limit on the grid-barrier waits: the solve reports the
    timeout (the blocks leave, no hang); with the default limit the next
    solve gives the reference's iterate."""
    P, g = load_gcase("gfc3d_lattice_5x5x6_s1")
    c = _ctx(P)
    try:
        c.spin_limit(1)
        with pytest.raises(RuntimeError, match="poll limit"):
            for _ in range(20):  # one poll: a barrier that not every block reached yet gives up
                c.set_start()
                c.solve(0.0, 200)
        c.spin_limit(0)
        c.set_start()
        res = c.solve(0.0, 20)
        r, u, v = c.get()
    finally:
        c.close()
    assert res["iterations"] == 20
    assert np.array_equal(r, g["r20"]) and np.array_equal(v, g["v20"])


def test_fused_products_opt_in(gpu):
    """The opt-in fused multiply-adds: iterates equal to the reference's to
    rounding (200 iterations), the same tolerance reached in about as many
    iterations, the result's error re-evaluated by the oracle below it; the
    default arithmetic stays bit-exact on the same context."""
    import oracle as O
    P = O.lattice_global(20, 20, 10, seed=3, mu=0.3)
    ref200 = O.gfc3d_nsgs_port(P, tol=0.0, maxiter=200)
    ref = O.gfc3d_nsgs_port(P, tol=1e-4, maxiter=10000)
    c = _ctx(P)
    try:
        c.set_arithmetic(True)
        c.solve(0.0, 200)
        r, u, v = c.get()
        assert not np.array_equal(r, ref200.r)
        assert np.linalg.norm(r - ref200.r) <= 1e-10 * np.linalg.norm(ref200.r)
        assert np.linalg.norm(v - ref200.v) <= 1e-10 * np.linalg.norm(ref200.v)
        c.set_start()
        res = c.solve(1e-4, 10000)
        r, u, v = c.get()
        assert res["info"] == 0 and abs(res["iterations"] - ref.iterations) <= 0.02 * ref.iterations
        e, _ = O.gfc3d_compute_error_port(P, r, v)
        assert e < 1e-4 * (1 + 1e-9)
        c.set_arithmetic(False)
        c.set_start()
        c.solve(0.0, 200)
        r, u, v = c.get()
        assert np.array_equal(r, ref200.r) and np.array_equal(v, ref200.v)
    finally:
        c.close()
