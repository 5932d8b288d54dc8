"""The oracle pinned against the reference: the CPU restatement reproduces
the reference's own fc3d_driver results bit for bit on every golden fixture
(generated from the reference by tests/golden/make_golden.py), and the
Alart-Curnier function its 1000 known answers."""
import numpy as np
import pytest

import oracle as O
from conftest import FIXTURE_CASES, LATTICE_CASES, GOLDEN, load_case


@pytest.mark.parametrize("case", FIXTURE_CASES + LATTICE_CASES)
def test_port_matches_reference_20_iterations(case):
    P, g = load_case(case)
    res = O.nsgs_port(P, tol=1e-8, maxiter=20, trace_cap=20)
    assert res.info == int(g["info20"])
    assert res.iterations == int(g["iterations20"])
    assert np.array_equal(res.r, g["r20"])
    assert np.array_equal(res.u, g["u20"])
    assert res.error == float(g["error20"])
    assert np.array_equal(res.trace, g["trace20"])


@pytest.mark.parametrize("case", FIXTURE_CASES + LATTICE_CASES)
def test_port_matches_reference_full_solve(case):
    P, g = load_case(case)
    res = O.nsgs_port(P, tol=1e-8, maxiter=10000, trace_cap=20000)
    assert res.info == int(g["info"])
    assert res.iterations == int(g["iterations"])
    assert res.error == float(g["error"])
    assert np.array_equal(res.r, g["r"])
    assert np.array_equal(res.u, g["u"])
    assert np.array_equal(res.trace, g["trace"])


def test_ac_function_known_answers():
    z = np.load(GOLDEN / "ac_known_answers.npz")
    lib = O.port()
    for k in range(z["R"].shape[0]):
        F, A, B = np.zeros(3), np.zeros(9), np.zeros(9)
        lib.oracle_ac_std(np.ascontiguousarray(z["R"][k]), np.ascontiguousarray(z["V"][k]), float(z["mu"][k]),
                          np.ascontiguousarray(z["rho"][k]), F, A.ctypes.data, B.ctypes.data)
        assert np.array_equal(F, z["F"][k]), k
        assert np.array_equal(A, z["A"][k]), k
        assert np.array_equal(B, z["B"][k]), k


def test_gepp_solves_random_systems():
    rng = np.random.default_rng(0)
    lib = O.port()
    for _ in range(200):
        A = rng.normal(size=(3, 3))
        b = rng.normal(size=3)
        x = b.copy()
        assert lib.oracle_solve_3x3_gepp(np.ascontiguousarray(A.T.reshape(-1)), x) == 0
        assert np.allclose(A @ x, b, rtol=0, atol=1e-9 * (1 + np.abs(b).max()) * np.linalg.cond(A))
    sing = np.zeros(9)
    assert lib.oracle_solve_3x3_gepp(sing, np.ones(3)) == 1


def test_projection_on_cone_cases():
    lib = O.port()
    r = np.array([-1.0, 0.1, 0.0]); assert lib.oracle_projection_on_cone(r, 0.5) == 0 and not r.any()
    r = np.array([1.0, 0.1, 0.0]); assert lib.oracle_projection_on_cone(r, 0.5) == 1
    r = np.array([1.0, 2.0, 0.0]); assert lib.oracle_projection_on_cone(r, 0.5) == 2
    assert np.isclose(np.hypot(r[1], r[2]), 0.5 * r[0])


@pytest.mark.parametrize("case", FIXTURE_CASES + LATTICE_CASES)
@pytest.mark.parametrize("kind", [0, 1])
def test_host_colouring_valid_and_deterministic(case, kind):
    P, _ = load_case(case)
    lib = O.port()
    c1 = np.zeros(P.nc, np.int32)
    c2 = np.zeros(P.nc, np.int32)
    n1 = lib.oracle_colour_greedy(P.nc, P.rowptr, P.colidx, kind, c1)
    n2 = lib.oracle_colour_greedy(P.nc, P.rowptr, P.colidx, kind, c2)
    assert n1 == n2 and np.array_equal(c1, c2)
    assert lib.oracle_colour_check(P.nc, P.rowptr, P.colidx, c1) == 0
    deg = np.diff(P.rowptr).max()
    assert n1 <= 2 * deg + 1


def test_coloured_order_port_converges_on_small_lattice():
    P, g = load_case("lattice_3x3x2_s1")
    lib = O.port()
    col = np.zeros(P.nc, np.int32)
    lib.oracle_colour_greedy(P.nc, P.rowptr, P.colidx, 0, col)
    order = np.lexsort((np.arange(P.nc), col)).astype(np.int32)
    res = O.nsgs_port(P, tol=1e-8, maxiter=10000, order=order)
    assert res.info == 0 and res.error <= 1e-8
    e, _ = O.compute_error_port(P, g["r"])
    assert e <= 1e-8
