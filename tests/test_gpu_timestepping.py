"""Time stepping (consecutive solves, q on a random walk, contacts kept):
every checked step's device fc3d_compute_error agrees with the oracle's FP64
evaluation of the same reaction, every step reaches the tolerance, and the
previous-step start saves sweeps over the zero start."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _checker():
    import oracle as O

    def check(sc, r, q):
        P = O.Problem(sc.nc, sc.rowptr, sc.colidx, sc.blocks, q, sc.mu)
        e, _ = O.compute_error_port(P, r)
        return e
    return check


def _mlp():
    from siconos_gb300.learned import DEFAULT_WEIGHTS, WarmStartMLP
    if not DEFAULT_WEIGHTS.exists():
        pytest.fail(f"trained weights missing: {DEFAULT_WEIGHTS}")
    m = WarmStartMLP(0)
    m.load()
    return m


@pytest.mark.parametrize("warm,assembly", [("previous", "host"), ("learned", "host"), ("previous", "device")])
def test_sequence_small(built_lib, warm, assembly):
    from siconos_gb300.timestep import run_sequence, summarise
    m = _mlp() if warm == "learned" else None
    run = run_sequence(dims=(10, 10, 6), steps=30, seed=9, tol=1e-4, max_iter=2000, warm=warm, mlp=m,
                       check_every=5, checker=_checker(), assembly=assembly)
    s = summarise(run)
    assert s["converged"] == 30
    assert s["check_rel_diff_max"] <= 1e-10
    if m is not None:
        m.close()


def test_previous_step_start_saves_sweeps(built_lib):
    from siconos_gb300.timestep import run_sequence, summarise
    z = summarise(run_sequence(dims=(10, 10, 6), steps=8, seed=9, tol=1e-4, max_iter=2000, warm="zero"))
    p = summarise(run_sequence(dims=(10, 10, 6), steps=8, seed=9, tol=1e-4, max_iter=2000, warm="previous"))
    assert p["sweeps_mean"] < z["sweeps_mean"]


def test_sequence_80x80x40(built_lib):
    """The full time-stepping case: 761,600 contacts, 200 steps, W and q
    assembled on the device, learned warm start with the previous step as
    fallback, tol 1e-3, the oracle's FP64 error on every 10th step."""
    from siconos_gb300.timestep import run_sequence, summarise
    m = _mlp()
    run = run_sequence(dims=(80, 80, 40), steps=200, seed=5, tol=1e-3, max_iter=1500, warm="learned", mlp=m,
                       check_every=10, checker=_checker(), assembly="device")
    m.close()
    s = summarise(run)
    print(s)
    assert run["scene"]["contacts"] == 761600
    assert s["checked_steps"] == 20
    assert s["check_rel_diff_max"] <= 1e-10
    assert s["converged"] == 200, s
