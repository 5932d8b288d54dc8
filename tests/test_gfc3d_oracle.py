"""The oracle of the global FC3D NSGS (oracle/gfc3d_oracle.c) against the
reference's own gfc3d_nsgs (gfc3d_nsgs.c:62-198, run through gfc3d_driver
by oracle/_ref): bit for bit on the committed golden outputs of the
reference's global test problems and of the sphere lattice in global form,
and against the live reference where it is built.  CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN

GCASES = sorted(p.stem for p in GOLDEN.glob("gfc3d_*.npz"))


def load_gcase(name):
    import oracle as O
    z = np.load(GOLDEN / f"{name}.npz")
    P = O.GlobalProblem(int(z["n"]), int(z["nc"]), z["Mp"], z["Mi"], z["Mx"], z["Hp"], z["Hi"], z["Hx"], z["q"],
                        z["b"], z["mu"])
    return P, {k: z[k] for k in z.files}


def test_cases_present():
    assert len(GCASES) == 8


@pytest.mark.parametrize("case", GCASES)
@pytest.mark.parametrize("setting", [("", 1e-8, 1000), ("_default", 1e-4, 10000), ("20", 0.0, 20)])
def test_oracle_equals_reference_golden(case, setting):
    import oracle as O
    tag, tol, it = setting
    P, g = load_gcase(case)
    res = O.gfc3d_nsgs_port(P, tol=tol, maxiter=it)
    assert res.info == int(g["info" + tag])
    assert res.error == float(g["error" + tag])
    assert np.array_equal(res.r, g["r" + tag])
    assert np.array_equal(res.u, g["u" + tag])
    assert np.array_equal(res.v, g["v" + tag])


@pytest.mark.parametrize("case", ["gfc3d_GFC3D_TwoRods1", "gfc3d_GFC3D_OneContact", "gfc3d_lattice_5x5x6_s1"])
@pytest.mark.parametrize("freq", [3, 7])
def test_error_evaluation_frequency_live(case, freq):
    """ERROR_EVALUATION_FREQUENCY: the loop keeps its last evaluated error."""
    import oracle as O
    if not O.ref_available():
        pytest.skip("oracle/_ref is not built here")
    P, _ = load_gcase(case)
    a = O.gfc3d_nsgs_port(P, tol=1e-6, maxiter=500, freq=freq)
    b = O.gfc3d_nsgs_ref(P, tol=1e-6, maxiter=500, freq=freq)
    assert a.info == b.info and a.error == b.error
    assert np.array_equal(a.r, b.r) and np.array_equal(a.u, b.u) and np.array_equal(a.v, b.v)
    if a.info == 0 and a.iterations < 500:
        assert a.iterations % freq == 0


def test_warm_start_and_zero_budget_live():
    """A start (r, v) and max_iter 0: no iteration, the error of the start
    with u = b + H^T v, info -1."""
    import oracle as O
    if not O.ref_available():
        pytest.skip("oracle/_ref is not built here")
    P, g = load_gcase("gfc3d_GFC3D_TwoRods1")
    r0, v0 = g["r20"] * 0.9, g["v20"] * 1.1
    a = O.gfc3d_nsgs_port(P, r0=r0, v0=v0, tol=1e-8, maxiter=0)
    b = O.gfc3d_nsgs_ref(P, r0=r0, v0=v0, tol=1e-8, maxiter=0)
    assert a.info == b.info == -1
    assert a.error == b.error and np.array_equal(a.u, b.u) and np.array_equal(a.v, v0)
    a = O.gfc3d_nsgs_port(P, r0=r0, v0=v0, tol=1e-8, maxiter=1000)
    b = O.gfc3d_nsgs_ref(P, r0=r0, v0=v0, tol=1e-8, maxiter=1000)
    assert a.info == b.info == 0 and a.error == b.error and np.array_equal(a.r, b.r)


def test_compute_error_equals_reference_live():
    import oracle as O
    if not O.ref_available():
        pytest.skip("oracle/_ref is not built here")
    for case in GCASES:
        P, g = load_gcase(case)
        e1, u1 = O.gfc3d_compute_error_port(P, g["r20"], g["v20"])
        e2, u2 = O.gfc3d_compute_error_ref(P, g["r20"], g["v20"])
        assert e1 == e2 and np.array_equal(u1, u2), case


def test_components_of_m():
    """M's connected components: one per dof for a diagonal M, one for the
    coupled rod models."""
    import oracle as O
    assert O.gfc3d_components(load_gcase("gfc3d_lattice_5x5x6_s1")[0])[0] == 900
    assert O.gfc3d_components(load_gcase("gfc3d_GFC3D_OneContact")[0])[0] == 1
    assert O.gfc3d_components(load_gcase("gfc3d_GFC3D_TwoRods1")[0])[0] == 2


def test_global_lattice_reduces_to_the_local_lattice(built_lib):
    """H^T M^-1 H of the global scene is the local scene's W divided by the
    mass scale, and H^T M^-1 q + b its q."""
    import oracle as O
    import siconos_gb300.numerics as sn
    from siconos_gb300 import scene
    g = O.lattice_global(4, 3, 3, seed=2, mass_scale=10.0)
    M, H = g.dense()
    W = H.T @ np.linalg.solve(M, H)
    s = scene.lattice(4, 3, 3, seed=2)
    Wl = sn.SparseBlockMatrix(s.nc, s.rowptr, s.colidx, s.blocks).todense()
    np.testing.assert_allclose(W * 10.0, Wl, atol=1e-12 * np.abs(Wl).max())
    np.testing.assert_allclose(H.T @ np.linalg.solve(M, g.q) + g.b, s.q, atol=1e-14)
    # the product library's generator gives the same arrays
    p = scene.lattice_global(4, 3, 3, seed=2)
    for k in ("Mp", "Mi", "Mx", "Hp", "Hi", "Hx", "q", "b"):
        assert np.array_equal(getattr(p, k), getattr(g, k)), k
