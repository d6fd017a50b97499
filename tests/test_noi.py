"""NOI (noise-correlation) node constraint: the Newton update of a NOI node is
exactly 0 (reference: solver_factories.py:37-137 masks, :775-782 enforce_noi;
full_mna.py:360-369 and :734-739 for which nodes are NOI and their 0 V start).

CPU: the NOI naming rule, the resolved circuit's NOI list, and a known answer
of the oracle.  GPU: the device Newton loop against the oracle through the C
ABI, with a circuit node marked NOI.
"""

import numpy as np
import pytest

from oracle.mna import OracleSystem, nr_solve
from vajax_gb300 import circuit as circuit_mod
from vajax_gb300.circuit import Circuit, is_noi_node
from vajax_gb300.devices import ModelInfo, load_model


def test_noi_naming_rule():
    assert is_noi_node("NOI") and is_noi_node("noi") and is_noi_node("node4")
    assert not is_noi_node("node3") and not is_noi_node("di") and not is_noi_node("NOISE")


def test_resolved_circuit_lists_noi_nodes(monkeypatch):
    real = circuit_mod.model_info

    def fake(key):
        if key != "psp_like":
            return real(key)
        return ModelInfo(key="psp_like", model_id=0, nodes=("d", "g", "s", "b", "NOI", "gp"),
                         terminals=("d", "g", "s", "b"), internal=("NOI", "gp"), user_params=("w",),
                         defaults={"w": 1e-6}, jac=((0, 0),), has_temperature=False)

    monkeypatch.setattr(circuit_mod, "model_info", fake)
    c = Circuit("noi")
    c.vsource("v1", "vdd", "0", "dc", dc=1.0)
    c.add("m1", "psp_like", ["vdd", "g", "0", "0"])
    c.add("m2", "psp_like", ["g", "g", "0", "0"])
    rc = c.resolve()
    grp = rc.groups[0]
    noi_row = grp.node_map[4]
    assert sorted(rc.noi_nodes) == sorted(int(x) for x in noi_row)
    assert set(rc.noi_nodes) <= set(rc.internal_nodes)
    assert not set(int(x) for x in grp.node_map[5]) & set(rc.noi_nodes)


def _tee():
    # vdd -R1- n1 -R2- n2 -R3- 0, and n1 -R4- 0; n2 is held as a NOI node
    c = Circuit("tee")
    c.vsource("v1", "vdd", "0", "dc", dc=1.2)
    c.add("r1", "resistor", ["vdd", "n1"], r=1000.0)
    c.add("r2", "resistor", ["n1", "n2"], r=2000.0)
    c.add("r3", "resistor", ["n2", "0"], r=500.0)
    c.add("r4", "resistor", ["n1", "0"], r=4000.0)
    return c


def _oracle(rc):
    return OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})


def test_oracle_noi_known_answer():
    rc = _tee().resolve()
    n1, n2 = rc.node_names["n1"], rc.node_names["n2"]
    rc.noi_nodes = [n2]
    S = _oracle(rc)
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[rc.node_names["vdd"]] = 1.2
    X0[n2] = 0.25
    r = nr_solve(S, X0, rc.source_values(0.0))
    assert r["converged"]
    assert r["X"][n2] == 0.25  # the NOI node never moves
    g1, g2, g4 = 1 / 1000.0, 1 / 2000.0, 1 / 4000.0
    expect = (1.2 * g1 + 0.25 * g2) / (g1 + g2 + g4)
    assert abs(r["X"][n1] - expect) < 1e-9
    # without the constraint n2 follows the resistors
    rc.noi_nodes = []
    r2 = nr_solve(_oracle(rc), X0, rc.source_values(0.0))
    assert abs(r2["X"][n2] - 0.25) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["tee", "gates120"])
def test_device_newton_with_noi_matches_oracle(cuda, case):
    import torch

    from vajax_gb300.engine import CircuitEngine
    from vajax_gb300.generators import random_gate_network
    from vajax_gb300.runtime import DeviceCircuit
    if case == "tee":
        c = _tee()
        rc = c.resolve()
        noi = [rc.node_names["n2"]]
        X0 = np.zeros(rc.n_nodes + len(rc.vsources))
        X0[rc.node_names["vdd"]] = 1.2
        X0[noi[0]] = 0.25
        iters = 20
    else:
        c, _ = random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)
        eng = CircuitEngine(c).parse()
        rc = eng.rc
        # two gate nodes held fixed at their nodeset value; Newton runs to convergence
        # (intermediate iterates of the two LU orderings differ by rounding that the
        # node-limited steps amplify, the converged points agree)
        noi = sorted(rc.node_names[n] for n in list(c.nodeset)[:2])
        X0 = np.zeros(rc.n_nodes + len(rc.vsources))
        X0[: rc.n_nodes] = eng.initial_guess()
        iters = 100
    rc.noi_nodes = noi
    dc = DeviceCircuit(rc)
    S = _oracle(rc)
    vs = rc.source_values(0.0)
    ro = nr_solve(S, X0, vs, max_iterations=iters, node_limit=0.3)
    Xd = torch.as_tensor(X0, device=cuda)
    rd = dc.nr_solve(Xd, torch.as_tensor(vs, device=cuda), max_iter=iters, node_limit=0.3)
    Xg = rd["X"].cpu().numpy()
    assert ro["converged"] and rd["converged"]
    assert rd["iterations"] == ro["iterations"]
    for k in noi:
        assert Xg[k] == X0[k]
    err = np.max(np.abs(Xg - ro["X"]))
    assert err < 1e-9, err
