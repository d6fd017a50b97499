"""Generate the golden fixtures in this folder from the FP64 oracle.

The reference's own code cannot run in this environment (it needs jax,
jaxlib and an OpenVAF build), so the fixtures are oracle outputs; the oracle
itself is pinned to the reference's known-answer tests in
tests/test_oracle_pins.py.  The fixtures freeze the oracle's answers on small
seeded cases so that the GPU tests can compare against committed vectors and
the CPU suite notices any drift of the oracle.

    python tests/golden/make_golden.py        # rewrites *.npz here
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.dc import dc_operating_point  # noqa: E402
from oracle.mna import OracleSystem  # noqa: E402
from oracle.transient import run_transient  # noqa: E402
from vajax_gb300.devices import load_model  # noqa: E402
from vajax_gb300.engine import CircuitEngine  # noqa: E402
from vajax_gb300.generators import random_gate_network, ring_oscillator  # noqa: E402


def gates120():
    return random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0]


def gates60():
    return random_gate_network(n_gates=60, depth=6, n_inputs=8, seed=7)[0]


CASES = {"ring7": ring_oscillator, "gates120": gates120, "gates60": gates60}


def system(circuit):
    rc = circuit.resolve()
    return rc, OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})


def tran_cfg(rc, fixed, t_stop, dt, max_steps, max_dt=1e30):
    return dict(t_stop=t_stop, dt=dt, max_dt=max_dt, min_dt=1e-15, reltol=1e-3, abstol=1e-12, vntol=1e-6,
                lte_ratio=3.5, redo_factor=2.5, grow_factor=2.0, tran_ft=0.25, nr_damping=1.0, gshunt_init=0.0,
                gshunt_target=0.0, gshunt_steps=5, warmup_steps=2, max_consecutive_rejects=5,
                fixed_step=1.0 if fixed else 0.0, method=2, n_external=rc.n_external, max_steps=max_steps,
                tran_itl=20)


def pattern_fixture(name):
    rc, S = system(CASES[name]())
    out = {"indptr": S.indptr.astype(np.int32), "indices": S.indices.astype(np.int32),
           "diag": np.asarray(S.diag_pos, np.int32)}
    for gi, g in enumerate(S.groups):
        out[f"csr_pos_{gi}"] = np.asarray(g["csr_pos"], np.int32)
    return out


def eval_fixture():
    """EKV NMOS/PMOS outputs at 64 seeded terminal-voltage points each."""
    from vajax_gb300.circuit import Circuit
    from vajax_gb300.generators import NMOS, PMOS
    rng = np.random.default_rng(11)
    c = Circuit("ekv_points")
    n = 64
    for k in range(n):
        c.add(f"mn{k}", "ekv", [f"d{k}", f"g{k}", f"s{k}", f"b{k}"], **NMOS)
        c.add(f"mp{k}", "ekv", [f"pd{k}", f"pg{k}", f"ps{k}", f"pb{k}"], **PMOS)
    rc, S = system(c)
    X = np.zeros(rc.n_nodes)
    X[1:] = rng.uniform(-0.3, 1.5, rc.n_nodes - 1)
    out = {"X": X}
    for gi in range(len(S.groups)):
        rr, rq, jr, jq = S.eval_group(gi, X)
        out.update({f"rr_{gi}": rr, f"rq_{gi}": rq, f"jr_{gi}": jr, f"jq_{gi}": jq})
    return out


def ring_fixture(steps=200):
    rc, S = system(ring_oscillator())
    X0 = np.zeros(rc.n_nodes + 1)
    X0[rc.node_names["n1"]] = 1.2
    X0[rc.node_names["vdd"]] = 1.2
    _, _, Q0, I0, _, _ = S.build_system(X0, rc.source_values(0.0))
    cfg = tran_cfg(rc, True, steps * 1e-12, 1e-12, steps + 1)
    o = run_transient(S, cfg, X0, Q0, I0)
    return {"X0": X0, "Q0": Q0, "I0": I0, "times": o["times"], "V": o["V"], "I": o["I"]}


def network_fixture():
    """DC operating point (from the logic nodeset) and 40 adaptive BDF2 steps of gates60."""
    c = gates60()
    rc, S = system(c)
    eng = CircuitEngine(c).parse()
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    r = dc_operating_point(S, rc.source_values(0.0), X0.copy())
    assert r["converged"]
    cfg = tran_cfg(rc, False, 2e-9, 0.25e-12, 41, max_dt=2e-9 / 50)
    o = run_transient(S, cfg, r["X"], r["Q"], r["I_vsource"], r["max_res_contrib"])
    return {"X_guess": X0, "X_dc": r["X"], "Q_dc": r["Q"], "I_dc": r["I_vsource"], "maxc_dc": r["max_res_contrib"],
            "times": o["times"], "V": o["V"], "I": o["I"], "rejected": np.int64(o["rejected"])}


FIXTURES = {
    "pattern_ring7": lambda: pattern_fixture("ring7"),
    "pattern_gates120": lambda: pattern_fixture("gates120"),
    "ekv_eval": eval_fixture,
    "ring7_fixed_bdf2": ring_fixture,
    "gates60_dc_adaptive": network_fixture,
}


def main():
    for name, fn in FIXTURES.items():
        np.savez_compressed(HERE / f"{name}.npz", **fn())
        print("wrote", name)


if __name__ == "__main__":
    main()
