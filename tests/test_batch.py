"""Batched transient of many replicas of one small circuit (vgb_batch_*).

Every replica must take the steps it takes alone: the same accepted and
rejected steps and Newton iterations, node voltages within 1e-6 V (the
transient contract's fixed-step tolerance) of the FP64 oracle and of the
single-circuit transient path.  Fixtures from tests/golden/make_configs.py.
"""

from pathlib import Path

import numpy as np
import pytest

import tests.golden.make_configs as M
import tests.golden.make_golden as G
from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
from vajax_gb300.generators import random_gate_network, ring_oscillator

HERE = Path(__file__).resolve().parent / "golden"
V_TOL = 1e-6


def load(name):
    with np.load(HERE / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def _ring_corners(n, seed):
    corners = create_monte_carlo_corners(n, seed=seed)
    return [batch_circuit(ring_oscillator(), [c]).resolve() for c in corners]


# ---- CPU: pattern checks and the library's own argument checks -------------------

def test_same_pattern_and_fits():
    from vajax_gb300.batch import fits, same_pattern
    a, b = _ring_corners(2, 3)
    assert same_pattern(a, b) and fits(a)
    five = batch_circuit(ring_oscillator(stages=5), create_monte_carlo_corners(1, seed=3)).resolve()
    assert not same_pattern(a, five)
    big = random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0].resolve()
    assert not fits(big)


def test_batch_create_checks_without_a_gpu():
    """Creation touches no GPU: a circuit too large for the engine and a
    replica count below one are refused with a message; a ring is taken."""
    import ctypes as C
    from vajax_gb300.runtime import DeviceCircuit
    big = random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0].resolve()
    dc = DeviceCircuit(big, device=False)
    h = C.c_void_p()
    assert dc.lib.vgb_batch_create(dc.h, 4, C.byref(h)) == 1
    assert b"n_aug" in dc.lib.vgb_last_error(dc.h)
    dc.close()
    ring = DeviceCircuit(ring_oscillator().resolve(), device=False)
    assert ring.lib.vgb_batch_create(ring.h, 0, C.byref(h)) == 1
    assert ring.lib.vgb_batch_create(ring.h, 3, C.byref(h)) == 0
    assert ring.lib.vgb_batch_set_group(h, 7, 0, None, None, None) == 1
    assert b"group out of range" in ring.lib.vgb_batch_last_error(h)
    ring.lib.vgb_batch_destroy(h)
    ring.close()


# ---- GPU -------------------------------------------------------------------------

@pytest.mark.gpu
def test_batched_ring_all_20000_steps_match_oracle(cuda):
    """Config 1 through the batched engine (one replica, uic start computed on
    the device): every 10th row of the 20,000 fixed steps within 1e-6 V of the
    oracle, and the same 60,000 Newton iterations."""
    from vajax_gb300.batch import BatchedTransient
    fx = load("ring7_fixed_20000")
    rc = ring_oscillator().resolve()
    bt = BatchedTransient([rc])
    cfg = G.tran_cfg(rc, True, M.RING_STEPS * 1e-12, 1e-12, M.RING_STEPS + 1)
    out = bt.transient(cfg, fx["X0"][None, :])
    bt.close()
    assert out["coop_units"] >= 1  # the EKV devices went through the cooperative evaluation
    assert int(out["n_steps"][0]) == M.RING_STEPS + 1
    assert int(out["total_nr_iters"][0]) == int(fx["total_nr_iters"])
    np.testing.assert_allclose(out["times"][0][fx["rows"]], fx["times"], rtol=0, atol=1e-20)
    err = float(np.max(np.abs(out["V"][0][fx["rows"]] - fx["V"])))
    assert err < V_TOL, err


@pytest.mark.gpu
def test_cooperative_evaluation_matches_single_warp(cuda):
    """96 ring corners (adaptive gear2, 0.4 ns) with the cooperative model
    evaluation and with one warp per item: the same steps, rejections and
    Newton iterations in every replica, step times within 1e-9 relative and
    node voltages within 1e-9 V (a multiply-add split between warps is not
    fused, so the last bits may differ)."""
    from vajax_gb300.batch import BatchedTransient, uic_start
    rcs = _ring_corners(96, 5)
    rc = rcs[0]
    cfg = G.tran_cfg(rc, False, 0.4e-9, 1e-12, 3000, max_dt=1e-10)
    X0 = np.stack([uic_start(r, {"c0.n1": 1.2, "c0.vdd": 1.2}) for r in rcs])
    outs = []
    for coop in (True, False):
        bt = BatchedTransient(rcs, coop=coop)
        outs.append(bt.transient(cfg, X0))
        bt.close()
    a, b = outs
    assert a["coop_units"] > 0 and b["coop_units"] == 0
    for key in ("n_steps", "rejected", "total_nr_iters", "nr_failures"):
        assert np.array_equal(a[key], b[key]), key
    n = int(a["n_steps"].max())
    # step control sees the last bits through the LTE estimate: times agree to the contract's 1e-9
    np.testing.assert_allclose(a["times"][:, :n], b["times"][:, :n], rtol=1e-9)
    assert float(np.max(np.abs(a["V"][:, :n] - b["V"][:, :n]))) < 1e-9


@pytest.mark.gpu
def test_batched_ring_corners_match_oracle(cuda):
    """The benchmark's 1,024 Monte-Carlo ring corners in one batched run,
    2,000 fixed 1 ps steps from n1 = VDD: each sampled corner within 1e-6 V of
    the oracle's run of that corner alone."""
    from vajax_gb300.batch import BatchedTransient, uic_start
    fx = load("corners_ring_sampled")
    rcs = _ring_corners(M.CORNER_COUNT, M.CORNER_SEED)
    bt = BatchedTransient(rcs)
    rc = rcs[0]
    cfg = G.tran_cfg(rc, True, M.CORNER_STEPS * 1e-12, 1e-12, M.CORNER_STEPS + 1)
    X0 = np.stack([uic_start(r, {"c0.n1": 1.2, "c0.vdd": 1.2}) for r in rcs])
    out = bt.transient(cfg, X0)
    bt.close()
    assert out["coop_units"] == 0  # 448 item warps, more than the SMs: one warp each
    assert np.all(out["n_steps"] == M.CORNER_STEPS + 1)
    worst = 0.0
    for k in fx["sample"]:
        k = int(k)
        for j, name in enumerate(fx[f"names_{k}"]):
            col = rc.node_names["c0." + str(name)]
            worst = max(worst, float(np.max(np.abs(out["V"][k][fx["rows"], col] - fx[f"V_{k}"][:, j]))))
    assert worst < V_TOL, worst


@pytest.mark.gpu
def test_adaptive_corner_batch_each_replica_as_alone(cuda):
    """An adaptive batch of 24 ring corners (-40/27/125 C, VTH and mobility
    spread): each replica takes exactly the steps of its own run through the
    single-circuit transient (same step count, rejections and Newton
    iterations, times to 1e-9 relative) and its node voltages agree within
    1e-6 V."""
    from oracle.mna import OracleSystem
    from vajax_gb300.batch import BatchedTransient, uic_start
    from vajax_gb300.devices import load_model
    from vajax_gb300.runtime import DeviceCircuit
    rcs = _ring_corners(24, 5)
    rc = rcs[0]
    cfg = G.tran_cfg(rc, False, 1.5e-9, 1e-12, 4001, max_dt=1e-9)
    X0 = np.stack([uic_start(r, {"c0.n1": 1.2, "c0.vdd": 1.2}) for r in rcs])
    Q0, I0 = [], []
    for k, r in enumerate(rcs):  # one start state for both runs
        S = OracleSystem(r, {g.model: load_model(g.model) for g in r.groups})
        _, _, q, i, _, _ = S.build_system(X0[k], r.source_values(0.0))
        Q0.append(q)
        I0.append(i)
    Q0, I0 = np.stack(Q0), np.stack(I0)
    bt = BatchedTransient(rcs)
    out = bt.transient(cfg, X0, Q0, I0)
    bt.close()
    steps = set()
    for k, r in enumerate(rcs):
        dc = DeviceCircuit(r, precision=2)
        alone = dc.transient(cfg, X0[k], Q0[k], I0[k])
        dc.close()
        n = alone["n_steps"]
        steps.add(n)
        assert int(out["n_steps"][k]) == n, k
        assert int(out["rejected"][k]) == alone["rejected"], k
        assert int(out["total_nr_iters"][k]) == alone["total_nr_iters"], k
        np.testing.assert_allclose(out["times"][k][:n], alone["times"][:n], rtol=1e-9)
        assert float(np.max(np.abs(out["V"][k][:n] - alone["V"][:n]))) < V_TOL, k
    assert len(steps) > 1  # the corners really do take different step sequences


@pytest.mark.gpu
def test_batched_adaptive_ring_matches_oracle_period(cuda):
    """The nominal ring, adaptive over 5 ns, through the batched engine: the
    oracle's step sequence and its oscillation period within 0.1 %."""
    from vajax_gb300.batch import BatchedTransient
    fx = load("ring7_adaptive_5ns")
    rc = ring_oscillator().resolve()
    cfg = G.tran_cfg(rc, False, 5e-9, 1e-12, 20001, max_dt=1e-9)
    bt = BatchedTransient([rc])
    out = bt.transient(cfg, fx["X0"][None, :], fx["Q0"][None, :], fx["I0"][None, :])
    bt.close()
    n = int(out["n_steps"][0])
    up = M.rising_crossings(out["times"][0][:n], out["V"][0][:n, rc.node_names["n1"]])
    period = float(np.mean(np.diff(up[2:])))
    assert abs(period / float(fx["period"]) - 1.0) < 1e-3
    assert n == len(fx["times"]) and int(out["rejected"][0]) == int(fx["rejected"])
    np.testing.assert_allclose(out["times"][0][:n], fx["times"], rtol=1e-9)
    assert float(np.max(np.abs(out["V"][0][:n] - fx["V"]))) < V_TOL
