"""The sparse LU with a weighted matching and scaling, on the GPU through the
C ABI (vgb_solver_match): the high-gain ring's DC operating point on the
sparse path (no dense fallback), Jacobians solved to a small residual, and a
transient whose results do not depend on the matching beyond rounding.

Residuals are normwise backward errors |J x - b|_inf / (|J|_inf |x|_inf +
|b|_inf) and relative residuals |J x - b|_inf / |b|_inf.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.mna import OracleSystem
from vajax_gb300.devices import load_model
from vajax_gb300.generators import random_gate_network, ring_oscillator

pytestmark = pytest.mark.gpu


def _device(c, precision=0):
    from vajax_gb300.runtime import DeviceCircuit
    rc = c.resolve()
    return rc, DeviceCircuit(rc, precision=precision)


def _residuals(dc, csr, x, b):
    indptr, indices = dc.pattern()
    n = len(indptr) - 1
    A = sp.csr_matrix((csr, indices, indptr), shape=(n, n))
    r = A @ x - b
    berr = np.max(np.abs(r)) / (np.max(np.abs(A).sum(axis=1)) * np.max(np.abs(x)) + np.max(np.abs(b)))
    return berr, np.max(np.abs(r)) / np.max(np.abs(b)), A


@pytest.mark.parametrize("stages", [21, 31])
def test_ring_dc_on_the_sparse_path(cuda, stages):
    """The DC operating point of a 21- and a 31-stage ring on the sparse LU
    (the dense LU with partial pivoting is what these take by default): the
    matching is computed at the mid-rail start and the Newton loop converges
    to the oracle's operating point."""
    from oracle.dc import dc_operating_point
    from vajax_gb300.engine import CircuitEngine
    c = ring_oscillator(stages=stages)
    eng = CircuitEngine(c).parse()
    eng.options.sparse_pivoting = "matching"
    rc, dev = _device(c, precision=0)
    eng.device = dev
    Xg, Qg, Ig, maxcg, ok = eng.initial_state()
    assert ok and dev.matched and dev.precision == 0
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    ro = dc_operating_point(S, rc.source_values(0.0), X0)
    assert ro["converged"]
    assert np.max(np.abs(Xg[: rc.n_nodes] - ro["X"][: rc.n_nodes])) < 1e-9


@pytest.mark.parametrize("stages", [31])
def test_ring_jacobian_solve(cuda, stages):
    """The ring's Jacobian at the mid-rail start, solved on the sparse path
    with the matching: backward error at rounding level, and the same
    solution as a partial-pivoting LU."""
    import scipy.sparse.linalg as spl
    import torch
    from vajax_gb300.engine import CircuitEngine
    c = ring_oscillator(stages=stages)
    rc, dev = _device(c)
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = CircuitEngine(c).parse().initial_guess()
    csr = dev.build_system(torch.as_tensor(X0, device=cuda), torch.as_tensor(rc.source_values(0.0), device=cuda))[0]
    dev.set_matching(csr)
    b = np.random.default_rng(7).standard_normal(dev.n_aug)
    x = dev.linear_solve(csr, torch.as_tensor(b, device=cuda)).cpu().numpy()
    berr, rel, A = _residuals(dev, csr.cpu().numpy(), x, b)
    assert berr < 1e-14 and rel < 1e-9, (berr, rel)
    xr = spl.spsolve(A.tocsc(), b)
    assert np.max(np.abs(x - xr)) <= 1e-9 * np.max(np.abs(xr))


@pytest.mark.parametrize("point", ["dc", "random"])
def test_network_jacobian_at_small_c0(cuda, point):
    """A 2,000-gate network's Jacobian with c0 = 1e8 (the capacitive diagonal
    far from dominant), solved on the sparse path with the matching.

    At the DC operating point (condition number about 3e9) the relative
    residual stays below 1e-9.  At a random operating point the matrix is
    singular to working precision (smallest singular value about 2e-22, where
    a partial-pivoting LU leaves a relative residual above 1e2 too), so the
    measure there is the normwise backward error, which stays at rounding
    level."""
    import torch
    from vajax_gb300.engine import CircuitEngine
    c, _ = random_gate_network(n_gates=2000, depth=20, n_inputs=32, seed=3)
    rc, dev = _device(c)
    vs = torch.as_tensor(rc.source_values(0.0), device=cuda)
    X = np.zeros(rc.n_nodes + len(rc.vsources))
    if point == "dc":
        X[: rc.n_nodes] = CircuitEngine(c).parse().initial_guess()
        r = dev.nr_solve(torch.as_tensor(X, device=cuda), vs, max_iter=100, node_limit=0.3)
        assert r["converged"]
        X = r["X"].cpu().numpy()
    else:
        X[1: rc.n_nodes] = np.random.default_rng(1).uniform(0.0, 1.2, rc.n_nodes - 1)
    csr = dev.build_system(torch.as_tensor(X, device=cuda), vs, c0=1e8)[0]
    dev.set_matching(csr)
    b = np.random.default_rng(2).standard_normal(dev.n_aug)
    x = dev.linear_solve(csr, torch.as_tensor(b, device=cuda)).cpu().numpy()
    berr, rel, _ = _residuals(dev, csr.cpu().numpy(), x, b)
    assert berr < 1e-15, (berr, rel)
    if point == "dc":
        assert rel < 1e-9, (berr, rel)


def test_transient_with_and_without_matching(cuda):
    """A fixed-step transient of a 120-gate network: the matching changes the
    elimination, not the answer (node voltages within 1e-9 V, same Newton
    iterations)."""
    import torch
    from vajax_gb300.engine import CircuitEngine
    c, _ = random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)
    out = []
    for matched in (False, True):
        rc, dev = _device(c)
        X0 = np.zeros(rc.n_nodes + len(rc.vsources))
        X0[: rc.n_nodes] = CircuitEngine(c).parse().initial_guess()
        vs = torch.as_tensor(rc.source_values(0.0), device=cuda)
        r = dev.nr_solve(torch.as_tensor(X0, device=cuda), vs, max_iter=100, node_limit=0.3)
        assert r["converged"]
        X = r["X"].cpu().numpy()
        if matched:
            csr = dev.build_system(torch.as_tensor(X, device=cuda), vs)[0]
            dev.set_matching(csr)
        Q0 = r["Q"].cpu().numpy()
        I0 = r["I_vsource"].cpu().numpy()
        cfg = dict(t_stop=200e-12, dt=1e-12, max_dt=1e30, min_dt=1e-15, reltol=1e-3, abstol=1e-12, vntol=1e-6,
                   lte_ratio=3.5, redo_factor=2.5, grow_factor=2.0, tran_ft=0.25, nr_damping=1.0,
                   gshunt_init=0.0, gshunt_target=0.0, gshunt_steps=5, warmup_steps=2,
                   max_consecutive_rejects=5, fixed_step=1.0, method=2, n_external=rc.n_external,
                   max_steps=202, tran_itl=20)
        out.append(dev.transient(cfg, X, Q0, I0))
    a, b = out
    assert a["n_steps"] == b["n_steps"]
    assert a["total_nr_iters"] == b["total_nr_iters"]
    assert np.max(np.abs(a["V"] - b["V"])) < 1e-9
