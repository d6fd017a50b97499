"""The CUDA path against the FP64 oracle at the benchmark configurations.

Fixtures come from tests/golden/make_configs.py (oracle outputs).  Tolerances
are the transient Newton contract's: per-instance currents, charges and
Jacobian entries within 1e-10 relative; fixed-step node voltages within
1e-6 V; adaptive runs take the same steps (count, rejections, times to 1e-9
relative); the adaptive ring's oscillation period within 0.1 %.

The CPU tests at the end re-run the oracle on the first steps of each
fixture, so that a drift of the oracle shows up without a GPU.
"""

from pathlib import Path

import numpy as np
import pytest

import tests.golden.make_configs as M
import tests.golden.make_golden as G
from vajax_gb300.generators import ring_oscillator

HERE = Path(__file__).resolve().parent / "golden"
V_TOL = 1e-6


def load(name):
    with np.load(HERE / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def _ring_device(precision=2):
    """The ring on the single-circuit path with the dense LU (n_aug <= 128)."""
    from vajax_gb300.runtime import DeviceCircuit
    rc = ring_oscillator().resolve()
    return rc, DeviceCircuit(rc, precision=precision)


# ---- config 1: the 7-stage ring ------------------------------------------------

@pytest.mark.gpu
def test_ring_all_20000_fixed_steps_match_oracle(cuda):
    fx = load("ring7_fixed_20000")
    rc, dc = _ring_device()
    cfg = G.tran_cfg(rc, True, M.RING_STEPS * 1e-12, 1e-12, M.RING_STEPS + 1)
    g = dc.transient(cfg, fx["X0"], fx["Q0"], fx["I0"])
    assert g["n_steps"] == M.RING_STEPS + 1
    assert g["total_nr_iters"] == int(fx["total_nr_iters"])
    np.testing.assert_allclose(g["times"][fx["rows"]], fx["times"], rtol=0, atol=1e-20)
    err = float(np.max(np.abs(g["V"][fx["rows"]] - fx["V"])))
    assert err < V_TOL, err
    assert float(np.max(np.abs(g["V"][-1] - fx["V_last"]))) < V_TOL


@pytest.mark.gpu
def test_ring_adaptive_period_matches_oracle(cuda):
    """Adaptive gear2 over ~14 periods: the same accepted and rejected steps
    as the oracle, and the period (rising crossings of VDD/2 at n1) within
    0.1 % of the oracle's."""
    fx = load("ring7_adaptive_5ns")
    rc, dc = _ring_device()
    cfg = G.tran_cfg(rc, False, 5e-9, 1e-12, 20001, max_dt=1e-9)
    g = dc.transient(cfg, fx["X0"], fx["Q0"], fx["I0"])
    n = g["n_steps"]
    up = M.rising_crossings(g["times"][:n], g["V"][:n, rc.node_names["n1"]])
    period = float(np.mean(np.diff(up[2:])))
    assert abs(period / float(fx["period"]) - 1.0) < 1e-3, (period, float(fx["period"]))
    assert n == len(fx["times"]) and g["rejected"] == int(fx["rejected"])
    np.testing.assert_allclose(g["times"][:n], fx["times"], rtol=1e-9)
    assert float(np.max(np.abs(g["V"][:n] - fx["V"]))) < V_TOL


# ---- corner temperatures and parameters: device evaluation ---------------------

@pytest.mark.gpu
def test_ekv_eval_at_corner_temperatures_matches_oracle(cuda):
    """EKV NMOS/PMOS at -40, 27 and 125 C with shifted VTO and scaled KP per
    instance: every output within 1e-10 relative (per-column floor 1e-3 of
    the column's largest value, as for the default-temperature fixture)."""
    import torch
    from vajax_gb300.runtime import DeviceCircuit
    fx = load("ekv_corner_eval")
    rc = M.corner_eval_circuit().resolve()
    g0 = rc.groups[0]
    assert g0.temperatures is not None and len(set(np.round(g0.temperatures, 2))) == 3
    dc = DeviceCircuit(rc)
    X = torch.as_tensor(fx["X"], device=cuda)
    for gi in range(len(rc.groups)):
        out = dc.eval_group(gi, X)
        for key, name in (("rr", "res_resist"), ("rq", "res_react"), ("jr", "jac_resist"), ("jq", "jac_react")):
            ref = fx[f"{key}_{gi}"]
            got = out[name].cpu().numpy()
            floor = np.maximum(np.max(np.abs(ref), axis=0, keepdims=True), 1e-300)
            err = float(np.max(np.abs(got - ref) / (np.abs(ref) + 1e-3 * floor)))
            assert err < 1e-10, (gi, key, err)


# ---- config 4 on the block-diagonal path: batched Monte-Carlo ring corners ------

@pytest.mark.gpu
def test_block_diagonal_ring_corners_match_oracle(cuda):
    """The 1,024 Monte-Carlo ring corners as one block-diagonal circuit
    (every copy in one shared Newton loop), 2,000 fixed 1 ps steps; each
    sampled corner within 1e-6 V of the oracle's run of that corner alone."""
    from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    fx = load("corners_ring_sampled")
    corners = create_monte_carlo_corners(M.CORNER_COUNT, seed=M.CORNER_SEED)
    opts = SimulationOptions(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic",
                             ic={f"c{k}.{n}": 1.2 for k in range(M.CORNER_COUNT) for n in ("n1", "vdd")})
    eng = CircuitEngine(batch_circuit(ring_oscillator(), corners), opts)
    eng.parse()
    eng.prepare(t_stop=M.CORNER_STEPS * 1e-12, dt=1e-12, max_steps=M.CORNER_STEPS + 1)
    res = eng.run_transient()
    eng.device.close()
    worst = 0.0
    for k in fx["sample"]:
        k = int(k)
        assert len(res.times) == M.CORNER_STEPS + 1
        for j, name in enumerate(fx[f"names_{k}"]):
            v = res.voltages[f"c{k}.{name}"][fx["rows"]]
            worst = max(worst, float(np.max(np.abs(v - fx[f"V_{k}"][:, j]))))
    assert worst < V_TOL, worst


# ---- config 2: the 80k-transistor network ---------------------------------------

def _switch_run(precision="fp64"):
    fx = load("gates23530_switch")
    X, Q, I, maxc = M.dc_state()
    eng = M.switch_engine()
    eng.precision = precision
    eng.refine_sweeps = 1
    eng.prepare(t_stop=eng.t_stop, dt=eng.dt, max_steps=M.NET_STEPS + 1)
    g = eng.device.transient(M.switch_cfg(eng), X, Q, I, maxc)
    eng.device.close()
    return fx, g


def _switch_check(fx, g):
    """The oracle's step sequence, and the largest node-voltage difference to
    the oracle: every node at the last step, the fixture's node sample at
    every step."""
    n = g["n_steps"]
    assert n == len(fx["times"])
    assert g["rejected"] == int(fx["rejected"])
    np.testing.assert_allclose(g["times"][:n], fx["times"], rtol=1e-9)
    V = g["V"][:n]
    err_last = float(np.max(np.abs(V[-1] - fx["V_last"])))
    err_rows = float(np.max(np.abs(V[:, fx["sample"]] - fx["V_sample"])))
    return max(err_last, err_rows)


@pytest.mark.gpu
def test_network_80k_matches_oracle(cuda):
    """The benchmarked 23,530-gate network, its inputs switching from 10 ps
    on, adaptive gear2 with the benchmark's settings from the oracle's DC
    point through the first input edges: the oracle's step times, rejections,
    Newton iterations and Newton failures, every node within 1e-6 V."""
    fx, g = _switch_run()
    assert g["total_nr_iters"] == int(fx["total_nr_iters"])
    assert g["nr_failures"] == int(fx["nr_failures"])
    err = _switch_check(fx, g)
    assert err < V_TOL, err


@pytest.mark.gpu
def test_network_80k_mixed_precision_against_oracle(cuda):
    """FP32 LU with one FP64-residual refinement sweep (the default) on the
    same adaptive run: the oracle's steps, node voltages within 1e-6 V of the
    FP64 oracle."""
    fx, g = _switch_run(precision="mixed")
    err = _switch_check(fx, g)
    assert err < V_TOL, err


# ---- CPU: the oracle still reproduces the first steps of each fixture -----------

def test_oracle_ring_fixed_prefix():
    from oracle.transient import run_transient
    fx = load("ring7_fixed_20000")
    rc, S = G.system(ring_oscillator())
    X0, Q0, I0 = M.ring_start(rc, S)
    assert np.array_equal(X0, fx["X0"])
    steps = 300
    cfg = G.tran_cfg(rc, True, steps * 1e-12, 1e-12, steps + 1)
    o = run_transient(S, cfg, X0, Q0, I0)
    rows = fx["rows"][fx["rows"] <= steps]
    assert np.max(np.abs(o["V"][rows] - fx["V"][: len(rows)])) < 1e-12


def test_oracle_ring_adaptive_prefix():
    from oracle.transient import run_transient
    fx = load("ring7_adaptive_5ns")
    rc, S = G.system(ring_oscillator())
    X0, Q0, I0 = M.ring_start(rc, S)
    cfg = G.tran_cfg(rc, False, 5e-9, 1e-12, 101, max_dt=1e-9)
    o = run_transient(S, cfg, X0, Q0, I0)
    np.testing.assert_allclose(o["times"][:101], fx["times"][:101], rtol=1e-12)
    assert np.max(np.abs(o["V"][:101] - fx["V"][:101])) < 1e-12
    assert abs(float(fx["period"]) - 3.5762e-10) < 1e-13


def test_oracle_corner_eval_fixture():
    fx = load("ekv_corner_eval")
    got = M.ekv_corner_eval()
    for k in fx:
        scale = max(float(np.max(np.abs(fx[k]))), 1e-300)
        assert float(np.max(np.abs(got[k] - fx[k]))) / scale < 1e-12, k


def test_oracle_ring_corner_prefix():
    from oracle.transient import run_transient
    fx = load("corners_ring_sampled")
    k = int(fx["sample"][1])
    rc, S = G.system(M.corner_ring(k))
    X0, Q0, I0 = M.ring_start(rc, S, prefix="c0.")
    steps = 100
    cfg = G.tran_cfg(rc, True, steps * 1e-12, 1e-12, steps + 1)
    o = run_transient(S, cfg, X0, Q0, I0)
    rows = fx["rows"][fx["rows"] <= steps]
    got = np.stack([o["V"][rows, rc.node_names["c0." + str(n)]] for n in fx[f"names_{k}"]], axis=1)
    assert np.max(np.abs(got - fx[f"V_{k}"][: len(rows)])) < 1e-12


def test_network_fixture_matches_the_benchmark_network():
    """The switch network has the benchmark network's nodes in the same
    order (so the stored DC point applies), and the fixture's rows cover the
    external nodes."""
    fx = load("gates23530_switch")
    X, _, _, _ = M.dc_state()
    rc = M.switch_network().resolve()
    assert rc.n_nodes + len(rc.vsources) == len(X)
    assert len(fx["V_last"]) == rc.n_external
    assert fx["V_sample"].shape == (len(fx["times"]), M.NET_SAMPLE)
    assert np.all(fx["sample"] < rc.n_external)
    assert len(fx["times"]) == M.NET_STEPS + 1
