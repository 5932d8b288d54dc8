"""What the trained warm start gains over the method without it, on a
held-out lattice (seed not used in training), at equal final tolerance.

Measured on GB300 (60x60x30, seed 424242, tol 1e-3): from zero the proposal
lowers the initial error from 0.339 to 0.149 but the solve needs 564 sweeps
against 565; after a time step the previous reaction (initial error 0.088)
beats the proposal (0.104), so the fallback keeps it and the sweeps are the
same (173).  NSGS's sweeps go into the stack-wide error components that
per-contact features cannot predict.  The test asserts that outcome: a
rejected proposal changes nothing, a taken one has the lower initial error
and stays within a few percent of the plain start's sweeps."""
import json

import pytest

pytestmark = pytest.mark.gpu


def test_learned_start_vs_plain(built_lib):
    from siconos_gb300.learned import DEFAULT_WEIGHTS, WarmStartMLP, evaluate
    assert DEFAULT_WEIGHTS.exists()
    m = WarmStartMLP(0)
    meta = m.load()
    assert "config" in meta and "history" in meta
    r = evaluate(m, dims=(24, 24, 12), seed=777001, tol=1e-3, max_iter=3000)
    m.close()
    sweeps = {k: {s: (v["sweeps32"] + v["sweeps64"]) for s, v in r[k].items()} for k in ("step0", "step1")}
    print(json.dumps(sweeps))
    for step, fallback in (("step0", "zero"), ("step1", "previous")):
        plain, learned = r[step][fallback], r[step]["learned"]
        assert plain["info"] == 0 and learned["info"] == 0
        assert learned["error"] <= 1e-3 and plain["error"] <= 1e-3
        n_plain, n_learned = sweeps[step][fallback], sweeps[step]["learned"]
        if learned["taken"]:
            assert learned["error_proposal"] < learned["error_fallback"]
            assert n_learned <= 1.05 * n_plain + 2
        else:
            # same start, same deterministic sweeps
            assert n_learned == n_plain
    # the previous step's reaction saves sweeps over a zero start
    assert sweeps["step1"]["previous"] < sweeps["step1"]["zero"]
