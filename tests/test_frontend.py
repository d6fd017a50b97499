"""Verilog-A front end and MIR interpreter (CPU)."""

import numpy as np
import pytest

from oracle.mir_interp import eval_model
from vajax_gb300.devices import load_model, model_keys
from vajax_gb300.va.frontend import compile_va

RC_SRC = """
`include "disciplines.vams"
module rc(a, b);
  inout a, b; electrical a, b;
  parameter real r = 2.0 from (0:inf);
  parameter real c = 1e-12;
  analog begin
    I(a, b) <+ V(a, b) / r;
    I(a, b) <+ ddt(c * V(a, b) * V(a, b));
  end
endmodule
"""


def test_rc_residuals_and_jacobian():
    m = compile_va(RC_SRC)
    v = np.array([0.5, -1.0, 2.0])
    out = eval_model(m, {"r": 2.0, "c": 1e-12}, {"V(a,b)": v}, 300.0, 3)
    np.testing.assert_allclose(out["res_resist"][:, 0], v / 2.0)
    np.testing.assert_allclose(out["res_resist"][:, 1], -v / 2.0)
    np.testing.assert_allclose(out["res_react"][:, 0], 1e-12 * v * v)
    keys = [(j["row_node_name"], j["col_node_name"]) for j in m["dae"]["jacobian"]]
    aa = keys.index(("a", "a"))
    ab = keys.index(("a", "b"))
    np.testing.assert_allclose(out["jac_resist"][:, aa], 0.5)
    np.testing.assert_allclose(out["jac_resist"][:, ab], -0.5)
    np.testing.assert_allclose(out["jac_react"][:, aa], 2e-12 * v)


def test_bundled_models_present():
    assert set(model_keys()) >= {"resistor", "capacitor", "ekv", "ekv_longchannel"}


@pytest.mark.parametrize("key", ["ekv", "ekv_longchannel"])
def test_mosfet_jacobian_matches_finite_differences(key):
    m = load_model(key)
    nodes = [n["name"] for n in m["dae"]["nodes"]]
    labels = [n for n, k in zip(m["param_names"], m["param_kinds"]) if k == "voltage"]
    rng = np.random.default_rng(3)
    n = 48
    V = rng.uniform(-0.1, 1.3, size=(n, len(nodes)))
    V[:, nodes.index("b")] = 0.0
    params = {"W": 1e-6, "L": 0.1e-6}
    if key == "ekv":
        params.update(COX=1.7e-2, XJ=4e-8, GAMMA=0.4, PHI=0.8, LAMBDA=0.3, UCRIT=5e6, VTO=0.4, KP=5e-4)

    def volts(Vn):
        d = {}
        for lab in labels:
            a, b = (lab[2:-1].split(",") + [None])[:2]
            d[lab] = Vn[:, nodes.index(a)] - (Vn[:, nodes.index(b)] if b else 0.0)
        return d

    base = eval_model(m, params, volts(V), 300.15, n)
    h = 1e-6
    for ji, j in enumerate(m["dae"]["jacobian"]):
        r, c = nodes.index(j["row_node_name"]), nodes.index(j["col_node_name"])
        Vp, Vm = V.copy(), V.copy()
        Vp[:, c] += h
        Vm[:, c] -= h
        op, om = eval_model(m, params, volts(Vp), 300.15, n), eval_model(m, params, volts(Vm), 300.15, n)
        for kind, rk in (("jac_resist", "res_resist"), ("jac_react", "res_react")):
            fd = (op[rk][:, r] - om[rk][:, r]) / (2 * h)
            an = base[kind][:, ji]
            scale = np.abs(fd).max() + 1e-30
            # median over instances: a few may sit on a branch switch of the model
            assert np.median(np.abs(fd - an)) / scale < 1e-5, (key, j["row_node_name"], j["col_node_name"], kind)


def test_codegen_emits_every_model():
    from vajax_gb300.codegen.cuda import emit_model
    for key in model_keys():
        src = emit_model(load_model(key))
        assert "static void eval" in src and "goto" in src or key in ("capacitor",)
