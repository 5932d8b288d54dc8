"""The reference's other NSGS options through the GPU solver: error
evaluations FULL (every iteration, or every `freq`), LIGHT and ADAPTIVE, the
local tolerance strategies ADAPTIVE and ADAPTIVE_N_CONTACT, relaxation and
the filter of local solutions (fc3d_nsgs.c:711-900,
fc3d_set_internalsolver_tolerance.c:31-63).  The first two run as a host
loop of single FP64 sweeps in colour order, relaxation and filter in the
FP64 sweep kernels; against the oracle's
loop with the same options in the same order (the oracle itself pinned to
the reference under these options by test_nsgs_options_oracle.py): the same
info and iteration count, the reaction bit for bit, the residual (infinite
where the reference leaves it so) to 1e-12, u to rounding where the
reference computes it and untouched where it does not."""
import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

COMBOS = {
    "full": dict(err_mode=0),
    "full_every3": dict(err_mode=0, freq=3),
    "light": dict(err_mode=1),
    "adaptive_eval": dict(err_mode=3),
    "lwff_adaptive_tol": dict(err_mode=2, strategy=0),
    "lwff_adaptive_n_contact": dict(err_mode=2, strategy=2),
    "light_adaptive_tol": dict(err_mode=1, strategy=0),
    "full_adaptive_n_contact_ratio3": dict(err_mode=0, strategy=2, ratio=3.0),
    "relax_0.8": dict(err_mode=2, relax=1, omega=0.8),
    "relax_1.2_full": dict(err_mode=0, relax=1, omega=1.2),
    "filter": dict(err_mode=2, filter=1),
    "relax_filter_adaptive_tol": dict(err_mode=2, relax=1, omega=0.9, filter=1, strategy=0),
}
CASES = ["fixture_KaplasTower_i1061_4", "fixture_Confeti_ex13_Fc3D_SBM", "lattice_5x5x6_s1",
         "fixture_BoxesStack1_i100000_32"]


@pytest.mark.parametrize("combo", sorted(COMBOS))
@pytest.mark.parametrize("case", CASES)
def test_options_match_coloured_oracle(built_lib, case, combo):
    import oracle as O
    import siconos_gb300.numerics as sn
    P, _ = load_case(case)
    o = dict(O.DEFAULT_NSGS_OPTIONS, **COMBOS[combo])
    maxiter = 30 if o["err_mode"] == 3 else 800
    W = sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks)
    prob = sn.FrictionContactProblem(3, P.nc, W, P.q.copy(), P.mu.copy())
    so = sn.SolverOptions()
    so.iparam[sn.SICONOS_IPARAM_MAX_ITER] = maxiter
    so.dparam[sn.SICONOS_DPARAM_TOL] = 1e-8
    so.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] = o["err_mode"]
    so.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY] = o["freq"]
    so.iparam[sn.SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY] = o["strategy"]
    so.dparam[sn.SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO] = o["ratio"]
    so.iparam[10] = o["relax"]  # SICONOS_FRICTION_3D_NSGS_RELAXATION
    so.dparam[10] = o["omega"]  # SICONOS_FRICTION_3D_NSGS_RELAXATION_VALUE
    so.iparam[16] = o["filter"]  # SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION
    r = np.zeros(3 * P.nc)
    u = np.full(3 * P.nc, 7.25)
    info = sn.fc3d_nsgs_gpu(prob, r, u, so)
    _, col = sn.colour(P.rowptr, P.colidx, sn.FC3DGPU_COLOURING_DEFAULT)
    order = np.lexsort((np.arange(P.nc), col)).astype(np.int32)
    ref = O.nsgs_port(P, tol=1e-8, maxiter=maxiter, order=order, options=o, u0=np.full(3 * P.nc, 7.25))
    assert info == ref.info, (info, ref.info, sn.last_error())
    assert so.iparam[sn.SICONOS_IPARAM_ITER_DONE] == ref.iterations
    np.testing.assert_array_equal(r, ref.r)
    err = so.dparam[sn.SICONOS_DPARAM_RESIDU]
    if np.isinf(ref.error) or ref.error == 1e24:
        assert err == ref.error
    else:
        assert abs(err - ref.error) <= 1e-12 * max(ref.error, 1e-300)
    if ref.u_written:
        np.testing.assert_allclose(u, ref.u, rtol=0, atol=1e-12 * (1 + np.abs(ref.u).max()))
    else:
        assert np.all(u == 7.25)
    so.release()
