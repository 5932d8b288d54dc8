"""What the trained warm start gains over the method without it, on a
held-out lattice (seed not used in training), at equal final tolerance.

The fallback rule bounds the loss: when the proposal's initial error is not
below the fallback's, the solve starts from the fallback and its sweeps are
exactly those of the plain start.  The measured gain is printed; on the
lattice family the per-contact proposal does not beat a zero start by the
initial-error rule, nor the previous step's reaction."""
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
    print(json.dumps({k: {s: (v["sweeps32"] + v["sweeps64"]) for s, v in r[k].items()}
                      for k in ("step0", "step1")}))
    for step, fallback in (("step0", "zero"), ("step1", "previous")):
        plain, learned = r[step][fallback], r[step]["learned"]
        assert plain["info"] == 0 and learned["info"] == 0
        assert learned["error"] <= 1e-3 and plain["error"] <= 1e-3
        if learned["taken"]:
            assert learned["error_proposal"] < learned["error_fallback"]
        else:
            # same start, same deterministic sweeps
            assert learned["sweeps32"] + learned["sweeps64"] == plain["sweeps32"] + plain["sweeps64"]
    # the previous step's reaction saves sweeps over a zero start
    s1 = r["step1"]
    assert s1["previous"]["sweeps32"] + s1["previous"]["sweeps64"] < s1["zero"]["sweeps32"] + s1["zero"]["sweeps64"]
