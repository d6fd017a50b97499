"""Committed golden fixtures (tests/golden, made by make_golden.py).

CPU tests check that the oracle and the host-side analysis still reproduce
the fixtures; GPU tests check the CUDA path against them through the C ABI
with the contract tolerances (pattern and maps bit-exact, device outputs
within 1e-10 relative, node voltages within 1e-6 V).
"""

from pathlib import Path

import numpy as np
import pytest

import tests.golden.make_golden as G

HERE = Path(__file__).resolve().parent / "golden"


def load(name):
    with np.load(HERE / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def rel_err(a, b):
    scale = max(float(np.max(np.abs(b))) if b.size else 0.0, 1e-300)
    return float(np.max(np.abs(a - b))) / scale if b.size else 0.0


# ---- CPU: oracle and host analysis reproduce the fixtures ---------------------

@pytest.mark.parametrize("case", ["ring7", "gates120"])
def test_oracle_pattern_matches_fixture(case):
    fx = load(f"pattern_{case}")
    got = G.pattern_fixture(case)
    for k in fx:
        assert np.array_equal(got[k], fx[k]), k


@pytest.mark.parametrize("case", ["ring7", "gates120"])
def test_host_analysis_pattern_matches_fixture(case):
    from vajax_gb300.runtime import DeviceCircuit
    fx = load(f"pattern_{case}")
    rc = G.CASES[case]().resolve()
    dc = DeviceCircuit(rc, device=False)
    indptr, indices = dc.pattern()
    assert np.array_equal(indptr, fx["indptr"]) and np.array_equal(indices, fx["indices"])
    for gi in range(len(rc.groups)):
        assert np.array_equal(dc.stamp_positions(gi), fx[f"csr_pos_{gi}"])
    diag, _ = dc.special_positions()
    assert np.array_equal(diag, fx["diag"])


def test_oracle_eval_matches_fixture():
    fx = load("ekv_eval")
    got = G.eval_fixture()
    for k in fx:
        assert rel_err(got[k], fx[k]) < 1e-12, k


def test_oracle_ring_matches_fixture():
    fx = load("ring7_fixed_bdf2")
    got = G.ring_fixture()
    assert np.array_equal(got["times"], fx["times"])
    assert np.max(np.abs(got["V"] - fx["V"])) < 1e-9


def test_oracle_network_matches_fixture():
    fx = load("gates60_dc_adaptive")
    got = G.network_fixture()
    assert np.max(np.abs(got["X_dc"] - fx["X_dc"])) < 1e-9
    assert len(got["times"]) == len(fx["times"]) and int(got["rejected"]) == int(fx["rejected"])
    np.testing.assert_allclose(got["times"], fx["times"], rtol=1e-9)
    assert np.max(np.abs(got["V"] - fx["V"])) < 1e-9


# ---- GPU: the CUDA path against the fixtures ----------------------------------

def _device(circuit):
    from vajax_gb300.runtime import DeviceCircuit
    rc = circuit.resolve()
    return rc, DeviceCircuit(rc)


@pytest.mark.gpu
def test_gpu_eval_matches_fixture(cuda):
    import torch
    from vajax_gb300.circuit import Circuit
    from vajax_gb300.generators import NMOS, PMOS
    fx = load("ekv_eval")
    c = Circuit("ekv_points")
    for k in range(64):
        c.add(f"mn{k}", "ekv", [f"d{k}", f"g{k}", f"s{k}", f"b{k}"], **NMOS)
        c.add(f"mp{k}", "ekv", [f"pd{k}", f"pg{k}", f"ps{k}", f"pb{k}"], **PMOS)
    rc, dc = _device(c)
    X = torch.as_tensor(fx["X"], device=cuda)
    for gi in range(len(rc.groups)):
        out = dc.eval_group(gi, X)
        for key, name in (("rr", "res_resist"), ("rq", "res_react"), ("jr", "jac_resist"), ("jq", "jac_react")):
            ref = fx[f"{key}_{gi}"]
            got = out[name].cpu().numpy()
            floor = np.maximum(np.max(np.abs(ref), axis=0, keepdims=True), 1e-300)
            err = np.max(np.abs(got - ref) / (np.abs(ref) + 1e-3 * floor))
            assert err < 1e-10, (gi, key, err)


@pytest.mark.gpu
def test_gpu_ring_matches_fixture(cuda):
    fx = load("ring7_fixed_bdf2")
    rc, dc = _device(G.ring_oscillator())
    steps = len(fx["times"]) - 1
    cfg = G.tran_cfg(rc, True, steps * 1e-12, 1e-12, steps + 1)
    g = dc.transient(cfg, fx["X0"], fx["Q0"], fx["I0"])
    assert g["n_steps"] == steps + 1
    np.testing.assert_allclose(g["times"], fx["times"], rtol=0, atol=1e-20)
    assert np.max(np.abs(g["V"] - fx["V"])) < 1e-6


@pytest.mark.gpu
def test_gpu_network_matches_fixture(cuda):
    import torch
    fx = load("gates60_dc_adaptive")
    c = G.gates60()
    rc, dc = _device(c)
    r = dc.nr_solve(torch.as_tensor(fx["X_guess"], device=cuda), torch.as_tensor(rc.source_values(0.0), device=cuda),
                    max_iter=20)
    if not r["converged"]:
        r = dc.nr_solve(torch.as_tensor(fx["X_guess"], device=cuda),
                        torch.as_tensor(rc.source_values(0.0), device=cuda), max_iter=100, node_limit=0.3)
        r = dc.nr_solve(r["X"], torch.as_tensor(rc.source_values(0.0), device=cuda), max_iter=20)
    assert r["converged"]
    assert np.max(np.abs(r["X"].cpu().numpy() - fx["X_dc"])) < 1e-9
    cfg = G.tran_cfg(rc, False, 2e-9, 0.25e-12, 41, max_dt=2e-9 / 50)
    g = dc.transient(cfg, fx["X_dc"], fx["Q_dc"], fx["I_dc"], fx["maxc_dc"])
    assert g["n_steps"] == len(fx["times"]) and g["rejected"] == int(fx["rejected"])
    np.testing.assert_allclose(g["times"], fx["times"], rtol=1e-9)
    assert np.max(np.abs(g["V"] - fx["V"])) < 1e-6
