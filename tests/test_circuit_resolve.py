"""Instance parameters in the resolved circuit (CPU).

Each instance's parameters overwrite the model defaults; a name matches
case-insensitively when not found as given, and a name given twice in one
instance keeps its last value.  Values equal across the group are stored once
(``shared``), the rest per instance (``varying``).  Checked against a direct
per-instance restatement for netlists that reuse a few cards and for netlists
whose instances all differ.
"""

import numpy as np
import pytest

from vajax_gb300.circuit import Circuit
from vajax_gb300.devices import model_info


def _expected(info, params):
    vals = [info.defaults[p] for p in info.user_params]
    for name, v in params.items():
        names = list(info.user_params)
        k = names.index(name) if name in names else [p.lower() for p in names].index(name.lower())
        vals[k] = float(v)
    return vals


def _values(group):
    n_dev = group.node_map.shape[1]
    out = np.repeat(group.shared[:, None], n_dev, axis=1)
    for j, k in enumerate(group.varying_idx):
        out[k] = group.varying[j]
    return out


def _circuit(cards):
    c = Circuit("params")
    c.vsource("v1", "a", "0", "dc", dc=1.0)
    for i, p in enumerate(cards):
        c.add(f"r{i}", "resistor", ["a", f"n{i}"], **p)
        c.add(f"g{i}", "resistor", [f"n{i}", "0"])
    return c


CARDS = {
    # a few cards reused many times (one column slice per distinct card)
    "reused": [({"r": 10.0}, {"r": 20.0, "has_noise": 0}, {}, {"R": 7.0})[i % 4] for i in range(64)],
    # every instance different (gathered per column)
    "distinct": [{"r": 1.0 + i, "has_noise": i % 2} for i in range(64)],
    # case variants of one name in one instance: the last one wins
    "repeated_names": [{"r": 3.0, "R": 4.0 + (i % 2)} for i in range(32)],
}


@pytest.mark.parametrize("name", list(CARDS))
def test_instance_values_match_direct_restatement(name):
    cards = CARDS[name]
    c = _circuit(cards)
    rc = c.resolve()
    info = model_info("resistor")
    (grp,) = rc.groups
    got = _values(grp)
    by_name = dict(zip(grp.names, range(len(grp.names))))
    for inst in c.instances:
        assert np.array_equal(got[:, by_name[inst.name]], _expected(info, inst.params)), inst.name
    # a column is stored per instance only where the values differ
    for k in range(got.shape[0]):
        assert (k in set(grp.varying_idx.tolist())) == bool(np.any(got[k] != got[k, 0]))


def test_unknown_parameter_is_rejected():
    c = _circuit([{"r": 1.0}] * 20 + [{"rr": 2.0}])
    with pytest.raises(KeyError, match="rr"):
        c.resolve()


def test_internal_nodes_numbered_instance_by_instance(monkeypatch):
    from vajax_gb300 import circuit as circuit_mod
    from vajax_gb300.devices import ModelInfo
    real = circuit_mod.model_info

    def fake(key):  # a four-terminal model with two internal nodes, the first a NOI node
        if key != "int2":
            return real(key)
        return ModelInfo(key="int2", model_id=0, nodes=("d", "g", "s", "b", "NOI", "gi"), terminals=("d", "g", "s", "b"),
                         internal=("NOI", "gi"), user_params=("w",), defaults={"w": 1e-6}, jac=((0, 0),),
                         has_temperature=False)

    monkeypatch.setattr(circuit_mod, "model_info", fake)
    c = Circuit("internal")
    c.vsource("v1", "vdd", "0", "dc", dc=1.0)
    for i in range(5):
        c.add(f"m{i}", "int2", ["vdd", f"g{i}", "0", "0"], w=1e-6 * (1 + i % 2))
    c.add("r0", "resistor", ["vdd", "g0"], r=1e3)
    rc = c.resolve()
    grp = next(g for g in rc.groups if g.model == "int2")
    n_ext = rc.n_external
    # after the external nodes, two per instance, instances in order
    assert np.array_equal(grp.node_map[4:].T.ravel(), np.arange(n_ext, n_ext + 10))
    assert rc.internal_nodes == list(range(n_ext, n_ext + 10))
    assert rc.noi_nodes == list(range(n_ext, n_ext + 10, 2))
    assert rc.n_nodes == n_ext + 10
