"""GPU path vs the FP64 oracle, through the C ABI.

Tolerances (from the transient Newton contract): CSR pattern and stamp maps
bit-exact; per-instance currents, charges and Jacobian entries within 1e-10
relative; fixed-step node voltages within 1e-6 V.
"""

import numpy as np
import pytest

from oracle.mna import OracleSystem, nr_solve
from oracle.transient import run_transient
from vajax_gb300.circuit import Circuit
from vajax_gb300.devices import load_model
from vajax_gb300.generators import random_gate_network, ring_oscillator

pytestmark = pytest.mark.gpu

REL = 1e-10


def _pair(circuit, precision=0):
    from vajax_gb300.runtime import DeviceCircuit
    rc = circuit.resolve()
    dc = DeviceCircuit(rc, precision=precision)
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    return rc, dc, S


def _divider():
    c = Circuit("divider")
    c.vsource("v1", "vsrc", "0", "dc", dc=1.0)
    c.add("r1", "resistor", ["vsrc", "node1"], r=1000.0)
    c.add("r2", "resistor", ["node1", "0"], r=1000.0)
    return c


def _small_network(seed=5, gates=120):
    c, _ = random_gate_network(n_gates=gates, depth=6, n_inputs=8, seed=seed)
    return c


def _close(a, b, rel=REL, floor=0.0):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(np.max(np.abs(b)) if b.size else 0.0, floor, 1e-300)
    err = np.max(np.abs(a - b)) / scale if b.size else 0.0
    assert err <= rel, f"max rel error {err:.3e} > {rel:.1e}"


CIRCUITS = [("divider", _divider), ("ring7", ring_oscillator), ("gates120", _small_network)]


@pytest.mark.parametrize("name,make", CIRCUITS)
def test_pattern_and_maps_bit_exact(cuda, name, make):
    rc, dc, S = _pair(make())
    indptr, indices = dc.pattern()
    assert np.array_equal(indptr, S.indptr) and np.array_equal(indices, S.indices)
    for gi in range(len(rc.groups)):
        assert np.array_equal(dc.stamp_positions(gi), S.groups[gi]["csr_pos"]), gi
    diag, vs = dc.special_positions()
    assert np.array_equal(diag, S.diag_pos)
    assert np.array_equal(vs, S.vs_pos)


@pytest.mark.parametrize("name,make", CIRCUITS)
def test_device_eval_matches_interpreter(cuda, name, make):
    import torch
    rc, dc, S = _pair(make())
    rng = np.random.default_rng(11)
    X = np.concatenate([[0.0], rng.uniform(-0.1, 1.3, rc.n_nodes - 1), rng.normal(0, 1e-4, len(rc.vsources))])
    Xd = torch.as_tensor(X, device=cuda)
    for gi in range(len(rc.groups)):
        gpu = {k: v.cpu().numpy() for k, v in dc.eval_group(gi, Xd).items()}
        rr, rq, jr, jq = S.eval_group(gi, X)
        for key, ref in (("res_resist", rr), ("res_react", rq), ("jac_resist", jr), ("jac_react", jq)):
            # allclose-style, as the reference's OSDI comparison (rtol 1e-10 plus an absolute
            # floor): |gpu - ref| <= 1e-10 |ref| + 1e-13 max|column|.  The floor covers values
            # that are the small residue of a cancellation, where fused multiply-adds on the
            # GPU and separately rounded products in numpy differ in the last bits.
            col = np.max(np.abs(ref), axis=0, keepdims=True)
            bound = REL * np.abs(ref) + 1e-13 * col
            excess = np.abs(gpu[key] - ref) - bound
            assert np.all(excess <= 0), (name, gi, key, float(np.max(excess)))


@pytest.mark.parametrize("name,make", CIRCUITS)
def test_build_system_matches_oracle(cuda, name, make):
    import torch
    rc, dc, S = _pair(make())
    rng = np.random.default_rng(2)
    X = np.concatenate([[0.0], rng.uniform(0.0, 1.2, rc.n_nodes - 1), rng.normal(0, 1e-4, len(rc.vsources))])
    Qp = rng.normal(0, 1e-15, rc.n_nodes - 1)
    vs = rc.source_values(1e-10)
    c0, c1, c2 = 1.5e12, -2e12, 0.5e12
    t = lambda a: torch.as_tensor(np.asarray(a, np.float64), device=cuda)  # noqa: E731
    csr, f, Q, maxc, fres = dc.build_system(t(X), t(vs) if len(vs) else None, None, t(Qp), None, None,
                                            c0=c0, c1=c1, c2=c2)
    rcsr, rf, rQ, _, rmaxc, rfres = S.build_system(X, vs, None, Qp, c0, 0.0, c1, 0.0, None, c2, None)
    _close(csr.cpu().numpy(), rcsr)
    _close(f.cpu().numpy(), rf)
    _close(Q.cpu().numpy(), rQ)
    _close(maxc.cpu().numpy(), rmaxc)
    # deterministic (atomic-free) stamping: a second build is bit-identical
    csr2 = dc.build_system(t(X), t(vs) if len(vs) else None, None, t(Qp), None, None, c0=c0, c1=c1, c2=c2)[0]
    assert torch.equal(csr, csr2)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,make", CIRCUITS)
def test_linear_solve(cuda, name, make, precision):
    import torch
    rc, dc, S = _pair(make(), precision)
    rng = np.random.default_rng(4)
    X = np.concatenate([[0.0], rng.uniform(0.0, 1.2, rc.n_nodes - 1), np.zeros(len(rc.vsources))])
    vs = rc.source_values(0.0)
    csr = S.build_system(X, vs, None, None, 1.5e12)[0]
    b = rng.normal(size=S.n_aug)
    x = dc.linear_solve(torch.as_tensor(csr, device=cuda), torch.as_tensor(b, device=cuda)).cpu().numpy()
    J = S.dense(csr)
    ref = np.linalg.solve(J, b)
    _close(x, ref, rel=1e-9)


@pytest.mark.parametrize("precision", [0, 1])
def test_linear_solve_large_fronts(cuda, precision):
    """A 2000-gate network: fronts above the shared-memory size run as tile tasks."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    import torch
    c, _ = random_gate_network(n_gates=2000, seed=3)
    rc = c.resolve()
    from vajax_gb300.runtime import DeviceCircuit
    dc = DeviceCircuit(rc, precision=precision)
    assert dc.solver_info()["max_front"] > 64
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    rng = np.random.default_rng(9)
    X = np.concatenate([[0.0], rng.uniform(0.0, 1.2, rc.n_nodes - 1), np.zeros(len(rc.vsources))])
    # transient Jacobians at 1 ps and 30 ps BDF2 steps: static pivoting relies on the c0*C
    # diagonal; at random operating points the pivot growth stays below 10 down to c0 = 5e10
    for c0 in (1.5e12, 5e10):
        csr = S.build_system(X, rc.source_values(0.0), None, None, c0)[0]
        b = rng.normal(size=S.n_aug)
        x = dc.linear_solve(torch.as_tensor(csr, device=cuda), torch.as_tensor(b, device=cuda)).cpu().numpy()
        A = sp.csr_matrix((csr, S.indices, S.indptr), shape=(S.n_aug, S.n_aug))
        ref = spl.spsolve(A.tocsc(), b)
        res = np.max(np.abs(A @ x - b)) / np.max(np.abs(b))
        assert res < 1e-9, (c0, res)
        _close(x, ref, rel=1e-8)


def test_newton_divider(cuda):
    import torch
    rc, dc, S = _pair(_divider())
    X = np.zeros(rc.n_nodes + 1)
    X[1:rc.n_nodes] = 0.5
    Xd = torch.as_tensor(X, device=cuda)
    r = dc.nr_solve(Xd, torch.as_tensor(rc.source_values(0.0), device=cuda), max_iter=100)
    Xg = r["X"].cpu().numpy()
    assert r["converged"]
    v1 = 1e-3 / (2e-3 + 1e-12)
    assert abs(Xg[rc.node_names["node1"]] - v1) < 1e-12
    assert abs(Xg[rc.node_names["vsrc"]] - 1.0) < 1e-12
    assert abs(Xg[rc.n_nodes] - (-(1.0 - v1) / 1000.0 - 1e-12)) < 1e-15


@pytest.mark.parametrize("name,make", CIRCUITS[1:])
def test_dc_operating_point_matches_oracle(cuda, name, make):
    """Mid-rail / nodeset start, plain Newton, node-limited Newton, then the
    gshunt / source-stepping homotopy."""
    from oracle.dc import dc_operating_point
    from vajax_gb300.engine import CircuitEngine
    c = make()
    eng = CircuitEngine(c).parse()
    rc = eng.rc
    eng.device = _pair(c)[1]
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    Xg, Qg, Ig, maxcg, ok = eng.initial_state()
    ro = dc_operating_point(S, rc.source_values(0.0), X0)
    assert ok and ro["converged"]
    assert np.max(np.abs(Xg[: rc.n_nodes] - ro["X"][: rc.n_nodes])) < 1e-9
    _close(Qg, ro["Q"], rel=1e-9)


def test_node_limited_newton_matches_oracle(cuda):
    """Newton with the per-node step clip from the logic nodeset of a 500-gate
    network: same iteration count and operating point as the oracle."""
    import torch
    from vajax_gb300.engine import CircuitEngine
    c, _ = random_gate_network(n_gates=500, depth=12, n_inputs=32, seed=1)
    rc, dc, S = _pair(c)
    eng = CircuitEngine(c).parse()
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    vs = rc.source_values(0.0)
    ro = nr_solve(S, X0.copy(), vs, max_iterations=100, node_limit=0.3)
    r = dc.nr_solve(torch.as_tensor(X0.copy(), device=cuda), torch.as_tensor(vs, device=cuda), max_iter=100,
                    node_limit=0.3)
    assert ro["converged"] and r["converged"]
    assert r["iterations"] == ro["iterations"]
    assert np.max(np.abs(r["X"].cpu().numpy() - ro["X"])) < 1e-9


def _cfg(rc, fixed, t_stop, dt, max_steps, method=2):
    return dict(t_stop=t_stop, dt=dt, max_dt=1e30, min_dt=1e-15, reltol=1e-3, abstol=1e-12, vntol=1e-6,
                lte_ratio=3.5, redo_factor=2.5, grow_factor=2.0, tran_ft=0.25, nr_damping=1.0, gshunt_init=0.0,
                gshunt_target=0.0, gshunt_steps=5, warmup_steps=2, max_consecutive_rejects=5,
                fixed_step=1.0 if fixed else 0.0, method=method, n_external=rc.n_external, max_steps=max_steps,
                tran_itl=20)


def test_fixed_step_ring_matches_oracle(cuda):
    """Fixed-step BDF2 ring, node voltages within 1e-6 V of the FP64 oracle."""
    import torch
    rc, dc, S = _pair(ring_oscillator())
    X0 = np.zeros(rc.n_nodes + 1)
    X0[rc.node_names["n1"]] = 1.2
    X0[rc.node_names["vdd"]] = 1.2
    _, _, Q0, I0, _, _ = S.build_system(X0, rc.source_values(0.0))
    steps = 400
    cfg = _cfg(rc, True, steps * 1e-12, 1e-12, steps + 1)
    g = dc.transient(cfg, X0, Q0, I0)
    o = run_transient(S, cfg, X0, Q0, I0)
    assert g["n_steps"] == o["n_steps"] == steps + 1
    np.testing.assert_allclose(g["times"], o["times"], rtol=0, atol=1e-20)
    err = np.max(np.abs(g["V"] - o["V"]))
    assert err < 1e-6, err
    # and the ring actually oscillates
    v1 = g["V"][:, rc.node_names["n1"]]
    assert v1.max() > 1.0 and v1.min() < 0.2


def test_adaptive_network_matches_oracle(cuda):
    """Adaptive BDF2 with predictor/LTE on a small gate network."""
    rc, dc, S = _pair(_small_network(seed=7, gates=60))
    from vajax_gb300.engine import CircuitEngine
    import torch
    eng = CircuitEngine(_small_network(seed=7, gates=60)).parse()
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.init_mid_rail()
    vs = rc.source_values(0.0)
    from oracle.dc import dc_operating_point
    ro = dc_operating_point(S, vs, X0.copy())
    assert ro["converged"]
    cfg = _cfg(rc, False, 2e-9, 0.25e-12, 61)
    cfg["max_dt"] = 2e-9 / 50
    o = run_transient(S, cfg, ro["X"], ro["Q"], ro["I_vsource"], ro["max_res_contrib"])
    g = dc.transient(cfg, ro["X"], ro["Q"], ro["I_vsource"], ro["max_res_contrib"])
    assert g["n_steps"] == o["n_steps"]
    assert g["rejected"] == o["rejected"]
    np.testing.assert_allclose(g["times"], o["times"], rtol=1e-9)
    assert np.max(np.abs(g["V"] - o["V"])) < 1e-6


def test_transient_session_slices_match_one_call(cuda):
    """vgb_tran_* in slices of 7 accepted steps reproduces vgb_transient bit for bit."""
    rc, dc, S = _pair(_small_network(seed=7, gates=60))
    from vajax_gb300.engine import CircuitEngine
    eng = CircuitEngine(_small_network(seed=7, gates=60)).parse()
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    from oracle.dc import dc_operating_point
    ro = dc_operating_point(S, rc.source_values(0.0), X0.copy())
    cfg = _cfg(rc, False, 2e-9, 0.25e-12, 41)
    cfg["max_dt"] = 2e-9 / 50
    args = (ro["X"], ro["Q"], ro["I_vsource"], ro["max_res_contrib"])
    one = dc.transient(cfg, *args)
    sess = dc.session(cfg, *args)
    total = 0
    while not sess.done:
        total += sess.advance(7)
    sl = sess.read()
    sess.close()
    assert sl["n_steps"] == one["n_steps"] == 41
    assert total == 40
    assert np.array_equal(sl["times"], one["times"]) and np.array_equal(sl["V"], one["V"])
    assert np.array_equal(sl["I"], one["I"])
    assert sl["rejected"] == one["rejected"] and sl["total_nr_iters"] == one["total_nr_iters"]
