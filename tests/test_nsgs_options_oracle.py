"""The oracle's NSGS loop under the reference's other options, pinned to
the reference itself (oracle/_ref): the error evaluations FULL (every
iteration, or every `freq` iterations), LIGHT and ADAPTIVE (which the
reference's loop has no branch for, so it runs to the budget), the local
tolerance strategies ADAPTIVE and ADAPTIVE_N_CONTACT, the relaxation of each
new reaction, the filter of local solutions and contact freezing
(fc3d_nsgs.c:711-900, fc3d_set_internalsolver_tolerance.c:31-63).  Equal bit
for bit: info, iterations, final error (infinite where the reference leaves
it so), the per-iteration error its callback reports, r, and u (left as
given where the reference never computes it)."""
import numpy as np
import pytest

from conftest import FIXTURE_CASES, LATTICE_CASES, load_case

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
    "filter_light": dict(err_mode=1, filter=1),
    "relax_filter_adaptive_tol": dict(err_mode=2, relax=1, omega=0.9, filter=1, strategy=0),
    "freeze5": dict(freeze=5),
    "freeze3_light": dict(freeze=3, err_mode=1),
    "freeze2_full": dict(freeze=2, err_mode=0),
    "freeze7_relax": dict(freeze=7, relax=1, omega=0.9),
}
CASES = [c for c in FIXTURE_CASES if "Rover" not in c] + ["fixture_Rover4144"] + LATTICE_CASES


def _ref_available():
    import oracle as O
    return O.ref() is not None


@pytest.mark.parametrize("combo", sorted(COMBOS))
@pytest.mark.parametrize("case", CASES)
def test_options_oracle_equals_reference(case, combo):
    import oracle as O
    if not _ref_available():
        pytest.skip("oracle/_ref is not built")
    P, _ = load_case(case)
    o = dict(O.DEFAULT_NSGS_OPTIONS, **COMBOS[combo])
    mi = 40 if o["err_mode"] == 3 else 2000
    u0 = np.full(3 * P.nc, 7.25)
    a = O.nsgs_ref(P, tol=1e-8, maxiter=mi, trace_cap=mi, options=o, u0=u0)
    b = O.nsgs_port(P, tol=1e-8, maxiter=mi, trace_cap=mi, options=o, u0=u0)
    assert (a.info, a.iterations) == (b.info, b.iterations)
    assert a.error == b.error or (np.isnan(a.error) and np.isnan(b.error))
    np.testing.assert_array_equal(a.r, b.r)
    np.testing.assert_array_equal(a.u, b.u)
    np.testing.assert_array_equal(a.trace, b.trace)
    if o["err_mode"] in (1, 3):
        assert not b.u_written and np.all(b.u == 7.25) and np.isinf(b.error)


def test_default_options_unchanged():
    """The options path with the defaults is the default loop."""
    import oracle as O
    P, _ = load_case("fixture_KaplasTower_i1061_4")
    a = O.nsgs_port(P, tol=1e-8, maxiter=3000, trace_cap=3000)
    b = O.nsgs_port(P, tol=1e-8, maxiter=3000, trace_cap=3000, options={})
    assert (a.info, a.iterations, a.error) == (b.info, b.iterations, b.error)
    np.testing.assert_array_equal(a.r, b.r)
    np.testing.assert_array_equal(a.trace, b.trace)
