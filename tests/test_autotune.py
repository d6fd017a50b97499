"""Autotuner: coordinate descent and cache on CPU; on the GPU, the knobs
change no result bit and the tuner picks valid values."""

import json

import numpy as np
import pytest

from vajax_gb300.autotune import KNOBS, _load, _store, coordinate_descent, pattern_key


def test_pattern_key_is_stable_and_distinct():
    a = pattern_key([0, 1, 2], [0, 1], [3], "GB300")
    assert a == pattern_key(np.array([0, 1, 2]), np.array([0, 1]), [3], "GB300")
    assert a != pattern_key([0, 1, 2], [1, 0], [3], "GB300")
    assert a != pattern_key([0, 1, 2], [0, 1], [4], "GB300")
    assert a != pattern_key([0, 1, 2], [0, 1], [3], "other")


def test_coordinate_descent_picks_the_fastest_value_per_phase():
    state = {"factor_ctas_per_sm": 4, "solve_ctas_per_sm": 4, "eval_block": 64}
    calls = []

    def set_knob(name, v):
        calls.append((name, v))
        state[name] = v

    def measure():
        f = {2: 3.0, 3: 2.0, 4: 2.5}[state["factor_ctas_per_sm"]]
        s = {1: 1.0, 2: 1.0, 4: 0.5}[state["solve_ctas_per_sm"]]
        e = {32: 0.9, 64: 0.8, 128: 0.7, 256: 0.95}[state["eval_block"]]
        return {"factor_ms": f, "solve_ms": s, "eval_ms": e, "assemble_ms": 0.1}

    chosen, timings = coordinate_descent(set_knob, measure, dict(state))
    assert chosen == {"factor_ctas_per_sm": 3, "solve_ctas_per_sm": 4, "eval_block": 128}
    assert state == chosen
    assert set(timings) == {k[0] for k in KNOBS}
    assert timings["factor_ctas_per_sm"] == {2: 3.0, 3: 2.0, 4: 2.5}


def test_ties_keep_the_current_value():
    state = {"eval_block": 64}
    chosen, _ = coordinate_descent(lambda n, v: state.__setitem__(n, v), lambda: {"eval_ms": 1.0}, dict(state),
                                   knobs=(("eval_block", (32, 64, 128), "eval_ms"),))
    assert chosen["eval_block"] == 64


def test_cache_round_trip(tmp_path):
    p = tmp_path / "sub" / "tuning.json"
    assert _load(p) == {}
    _store(p, {"k": {"eval_block": 128}})
    assert _load(p) == {"k": {"eval_block": 128}}
    p.write_text("not json")
    assert _load(p) == {}
    json.loads(json.dumps(_load(p)))


@pytest.mark.gpu
def test_knobs_change_no_result_bit_and_tuner_runs(cuda, tmp_path):
    import torch

    from vajax_gb300.autotune import autotune
    from vajax_gb300.engine import CircuitEngine
    from vajax_gb300.generators import random_gate_network
    from vajax_gb300.runtime import DeviceCircuit
    c, _ = random_gate_network(n_gates=2000, seed=1)
    eng = CircuitEngine(c).parse()
    rc = eng.rc
    dc = DeviceCircuit(rc)
    X = np.zeros(rc.n_nodes + len(rc.vsources))
    X[: rc.n_nodes] = eng.initial_guess()
    vs = torch.as_tensor(rc.source_values(0.0), device=cuda)

    def newton3():
        r = dc.nr_solve(torch.as_tensor(X, device=cuda), vs, max_iter=3, c0=1e11)
        return r["X"].cpu().numpy()

    ref = newton3()
    for knob, values, _ in KNOBS:
        for v in values:
            dc.set_tuning(knob, v)
            assert dc.tuning()[knob] == v
            assert np.array_equal(newton3(), ref), (knob, v)
        dc.set_tuning(knob, {"factor_ctas_per_sm": 4, "solve_ctas_per_sm": 4, "eval_block": 64}[knob])
    with pytest.raises(Exception):
        dc.set_tuning("eval_block", 48)
    with pytest.raises(Exception):
        dc.set_tuning("factor_ctas_per_sm", 5)
    cache = tmp_path / "t.json"
    out = autotune(dc, torch.as_tensor(X, device=cuda), rc.source_values(0.0), reps=2, cache=cache)
    assert not out["cached"] and set(out["tuning"]) == {k[0] for k in KNOBS}
    assert dc.tuning() == out["tuning"]
    again = autotune(dc, torch.as_tensor(X, device=cuda), rc.source_values(0.0), reps=2, cache=cache)
    assert again["cached"] and again["tuning"] == out["tuning"]
    assert np.array_equal(newton3(), ref)


def test_tuning_knobs_validate_on_the_host():
    """vgb_set_tuning / vgb_get_tuning on an analysed host-only circuit: valid values
    stick, invalid ones return an error status and change nothing."""
    from vajax_gb300.generators import random_gate_network
    from vajax_gb300.runtime import DeviceCircuit
    c, _ = random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)
    dc = DeviceCircuit(c.resolve(), device=False)
    assert dc.tuning() == {"factor_ctas_per_sm": 4, "solve_ctas_per_sm": 4, "eval_block": 64}
    dc.set_tuning("eval_block", 128)
    dc.set_tuning("solve_ctas_per_sm", 1)
    assert dc.tuning()["eval_block"] == 128 and dc.tuning()["solve_ctas_per_sm"] == 1
    for knob, bad in (("eval_block", 48), ("eval_block", 512), ("solve_ctas_per_sm", 0), ("solve_ctas_per_sm", 5),
                      ("factor_ctas_per_sm", 0), ("factor_ctas_per_sm", 5)):
        before = dc.tuning()
        with pytest.raises(Exception):
            dc.set_tuning(knob, bad)
        assert dc.tuning() == before
    # changing the factorisation CTAs re-schedules the task list on the host; the
    # schedule stays a topological order of the same tasks
    n_tasks = dc.solver_info()["tasks"]
    dc.set_tuning("factor_ctas_per_sm", 2)
    assert dc.solver_info()["tasks"] == n_tasks
    dc.set_transient_graph(False)
    dc.set_transient_graph(True)
    with pytest.raises(Exception):
        dc._check(dc.lib.vgb_set_tuning(dc.h, 3, 2))
    with pytest.raises(Exception):
        dc._check(dc.lib.vgb_set_tuning(dc.h, 99, 1))
    dc.close()
