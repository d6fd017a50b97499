"""Oracle fixtures at the benchmark configurations (test infrastructure).

Each fixture is the FP64 oracle's answer on one of the benchmarked circuits;
the GPU tests in tests/test_config_parity.py and tests/test_batch.py compare
the CUDA path against them with the contract tolerances.  The reference's own
JAX path cannot run here, so these are oracle outputs; the oracle is pinned
to the reference's known-answer tests in tests/test_oracle_pins.py.

  ring7_fixed_20000     7-stage ring, fixed-step gear2 at 1 ps for all 20,000
                        steps from n1 = VDD (every 10th output row kept)
  ring7_adaptive_5ns    the same ring, adaptive gear2 over 5 ns (~14 periods):
                        step sequence, waveforms and the oscillation period
  ekv_corner_eval       EKV NMOS/PMOS outputs at -40, 27 and 125 C with
                        per-instance VTO shifts and KP scales
  corners_ring_sampled  8 of the 1,024 Monte-Carlo ring corners (seed 7), each
                        run alone: 2,000 fixed 1 ps steps (every 10th row kept)
  gates23530_switch     the 80k-transistor network (23,530 gates, seed 1) with
                        its input edges moved to 2 ps periods so that the
                        first steps switch gates: 6 fixed trapezoidal steps at
                        1 ps and 6 adaptive gear2 steps, from the oracle's DC
                        point (oracle/data); every node at the last step, a
                        seeded sample of 4,096 nodes at every step

  python tests/golden/make_configs.py [name ...]     # one process per fixture

Each fixture takes up to about 10 minutes of CPU; run them in parallel.
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle.transient import run_transient  # noqa: E402
from tests.golden.make_golden import system, tran_cfg  # noqa: E402
from vajax_gb300.generators import ring_oscillator  # noqa: E402

RING_STEPS = 20000
KEEP = 10  # output rows kept from the long runs
CORNER_SEED = 7
CORNER_COUNT = 1024
CORNER_SAMPLE = (0, 101, 257, 384, 511, 640, 777, 1023)
CORNER_STEPS = 2000
NET_GATES = 23530
NET_PERIOD = 10e-12  # input period and edge of the fixture network (the benchmark's: 0.5 ns, 50 ps)
NET_EDGE = 8e-12
NET_STEPS = 60  # accepted adaptive steps: through the first input edges (10 to 18 ps)
NET_SAMPLE = 4096  # nodes kept at every step; the last step keeps every node


def ring_start(rc, S, prefix=""):
    """n1 = VDD and vdd = VDD, all other nodes 0 (uic), charges and branch
    current from one system build there, as the engine's uic start does."""
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[rc.node_names[prefix + "n1"]] = 1.2
    X0[rc.node_names[prefix + "vdd"]] = 1.2
    _, _, Q0, I0, _, _ = S.build_system(X0, rc.source_values(0.0))
    return X0, Q0, I0


def rising_crossings(times, v, level=0.6):
    out = []
    for k in range(1, len(v)):
        if v[k - 1] < level <= v[k]:
            out.append(times[k - 1] + (level - v[k - 1]) * (times[k] - times[k - 1]) / (v[k] - v[k - 1]))
    return np.asarray(out)


def ring7_fixed_20000():
    rc, S = system(ring_oscillator())
    X0, Q0, I0 = ring_start(rc, S)
    cfg = tran_cfg(rc, True, RING_STEPS * 1e-12, 1e-12, RING_STEPS + 1)
    o = run_transient(S, cfg, X0, Q0, I0)
    assert o["n_steps"] == RING_STEPS + 1
    return {"X0": X0, "Q0": Q0, "I0": I0, "rows": np.arange(0, RING_STEPS + 1, KEEP),
            "times": o["times"][::KEEP], "V": o["V"][::KEEP], "V_last": o["V"][-1],
            "total_nr_iters": np.int64(o["total_nr_iters"])}


def ring7_adaptive_5ns():
    rc, S = system(ring_oscillator())
    X0, Q0, I0 = ring_start(rc, S)
    cfg = tran_cfg(rc, False, 5e-9, 1e-12, 20001, max_dt=1e-9)
    o = run_transient(S, cfg, X0, Q0, I0)
    n = int(o["n_steps"])
    times, V = o["times"][:n], o["V"][:n]
    up = rising_crossings(times, V[:, rc.node_names["n1"]])
    return {"X0": X0, "Q0": Q0, "I0": I0, "times": times, "V": V, "rejected": np.int64(o["rejected"]),
            "total_nr_iters": np.int64(o["total_nr_iters"]), "crossings": up,
            "period": np.float64(np.mean(np.diff(up[2:])))}


def corner_eval_circuit():
    """96 NMOS + 96 PMOS EKV instances, each with its own temperature from
    {-40, 27, 125} C, VTO shifted by N(0, 30 mV) and KP scaled by N(1, 0.05)."""
    from vajax_gb300.circuit import Circuit
    from vajax_gb300.generators import NMOS, PMOS
    rng = np.random.default_rng(23)
    c = Circuit("ekv_corner_points")
    temps = (233.15, 300.15, 398.15)
    for k in range(96):
        for pre, card, sign in (("mn", NMOS, 1.0), ("mp", PMOS, -1.0)):
            p = dict(card)
            p["VTO"] = card["VTO"] + sign * rng.normal(0.0, 0.03)
            p["KP"] = card["KP"] * rng.normal(1.0, 0.05)
            c.add(f"{pre}{k}", "ekv", [f"{pre}d{k}", f"{pre}g{k}", f"{pre}s{k}", f"{pre}b{k}"],
                  temperature=temps[k % 3], **p)
    return c


def ekv_corner_eval():
    rc, S = system(corner_eval_circuit())
    rng = np.random.default_rng(29)
    X = np.zeros(rc.n_nodes)
    X[1:] = rng.uniform(-0.3, 1.5, rc.n_nodes - 1)
    out = {"X": X}
    for gi in range(len(S.groups)):
        rr, rq, jr, jq = S.eval_group(gi, X)
        out.update({f"rr_{gi}": rr, f"rq_{gi}": rq, f"jr_{gi}": jr, f"jq_{gi}": jq})
    return out


def corner_ring(k):
    """Monte-Carlo ring corner k of the benchmark's 1,024 (seed 7), alone, node names c0.*."""
    from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
    corners = create_monte_carlo_corners(CORNER_COUNT, seed=CORNER_SEED)
    return batch_circuit(ring_oscillator(), [corners[k]])


def corners_ring_sampled():
    out = {"sample": np.asarray(CORNER_SAMPLE, np.int64), "rows": np.arange(0, CORNER_STEPS + 1, KEEP)}
    for k in CORNER_SAMPLE:
        rc, S = system(corner_ring(k))
        X0, Q0, I0 = ring_start(rc, S, prefix="c0.")
        cfg = tran_cfg(rc, True, CORNER_STEPS * 1e-12, 1e-12, CORNER_STEPS + 1)
        o = run_transient(S, cfg, X0, Q0, I0)
        assert o["n_steps"] == CORNER_STEPS + 1
        names = sorted((n for n, i in rc.node_names.items() if 0 < i < rc.n_external), key=rc.node_names.get)
        out[f"V_{k}"] = np.stack([o["V"][::KEEP, rc.node_names[n]] for n in names], axis=1)
        out[f"names_{k}"] = np.asarray([n[len("c0."):] for n in names])
        print(f"corner {k} done", flush=True)
    return out


def switch_network():
    """The benchmark's network with its input period cut to 10 ps (8 ps
    edges): the same gates, nets and DC point, but inputs switch from t =
    10 ps on."""
    from vajax_gb300.generators import random_gate_network
    return random_gate_network(n_gates=NET_GATES, depth=60, n_inputs=32, seed=1, c_wire=5e-15, period=NET_PERIOD,
                               edge=NET_EDGE)[0]


def switch_engine():
    """Engine over switch_network() with the benchmark's adaptive settings
    (engine defaults, gear2, t_stop 20 ns, dt0 1 ps), host side only."""
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    eng = CircuitEngine(switch_network(), SimulationOptions(tran_method="gear2"))
    eng.parse()
    eng.t_stop, eng.dt = 20e-9, 1e-12
    eng.config = eng._config(20e-9, 1e-12, None)
    eng.max_steps = NET_STEPS + 1
    return eng


def switch_cfg(eng):
    """The benchmark's adaptive gear2 settings for NET_STEPS accepted steps.
    Fixed steps are not used here: across a switching edge the model (which
    has no limiting) drives Newton out of range at fixed steps in the oracle
    with every method and step tried; the adaptive controller rejects and
    shrinks the step instead."""
    cfg = eng.transient_cfg()
    cfg.update(max_steps=NET_STEPS + 1)
    return cfg


def dc_state():
    from oracle.make_dc_state import dc_state_path
    z = np.load(dc_state_path(NET_GATES, 1))
    return z["X"], z["Q"], z["I"], z["maxc"]


def gates23530_switch():
    from oracle.mna import OracleSystem
    from vajax_gb300.devices import load_model
    eng = switch_engine()
    rc = eng.rc
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups}, gmin=eng.options.gmin)
    X, Q, I, maxc = dc_state()
    t0 = time.time()
    o = run_transient(S, switch_cfg(eng), X, Q, I, maxc)
    n = int(o["n_steps"])
    print("adaptive %.0f s" % (time.time() - t0), n, "steps", o["rejected"], "rejected", o["nr_failures"],
          "Newton failures", flush=True)
    assert n == NET_STEPS + 1
    V = o["V"][:n]
    sample = np.sort(np.random.default_rng(5).choice(V.shape[1], NET_SAMPLE, replace=False))
    return {"times": o["times"][:n], "V_last": V[-1], "sample": sample.astype(np.int32), "V_sample": V[:, sample],
            "rejected": np.int64(o["rejected"]), "total_nr_iters": np.int64(o["total_nr_iters"]),
            "nr_failures": np.int64(o["nr_failures"])}


FIXTURES = {
    "ring7_fixed_20000": ring7_fixed_20000,
    "ring7_adaptive_5ns": ring7_adaptive_5ns,
    "ekv_corner_eval": ekv_corner_eval,
    "corners_ring_sampled": corners_ring_sampled,
    "gates23530_switch": gates23530_switch,
}


def main(names):
    for name in names or FIXTURES:
        t0 = time.time()
        np.savez_compressed(HERE / f"{name}.npz", **FIXTURES[name]())
        print(f"wrote {name} ({time.time() - t0:.0f} s)", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
