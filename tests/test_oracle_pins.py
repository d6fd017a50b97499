"""Pin the oracle against the reference's own known-answer tests.

The expected numbers come from the reference test suite:
tests/test_integration_methods.py:27-185 (integration coefficients and
formulas), tests/test_adaptive_timestep.py:19-283 (predictor / LTE helpers)
and tests/test_fori_loop_nr.py:15-193 (Newton on a resistive divider,
V(node1) = 0.5 V and V(vsrc) = 1.0 V to 1e-10).
"""

import numpy as np
import pytest

from oracle import predictor as P
from oracle.mna import OracleSystem, nr_solve
from vajax_gb300.circuit import Circuit
from vajax_gb300.devices import load_model


class TestIntegrationCoefficients:
    def test_backward_euler(self):
        c = P.compute_coefficients(P.BE, 1e-12)
        assert c.c0 == pytest.approx(1e12) and c.c1 == pytest.approx(-1e12)
        assert c.c2 == 0.0 and c.d1 == 0.0 and c.history_depth == 1 and not c.needs_dqdt_history
        assert c.error_coeff == pytest.approx(0.5)

    def test_trap(self):
        c = P.compute_coefficients(P.TRAP, 1e-12)
        assert c.c0 == pytest.approx(2e12) and c.c1 == pytest.approx(-2e12)
        assert c.c2 == 0.0 and c.d1 == -1.0 and c.needs_dqdt_history
        assert c.error_coeff == pytest.approx(1.0 / 12.0)

    def test_gear2(self):
        c = P.compute_coefficients(P.GEAR2, 1e-12)
        assert c.c0 == pytest.approx(1.5e12) and c.c1 == pytest.approx(-2e12) and c.c2 == pytest.approx(0.5e12)
        assert c.d1 == 0.0 and c.history_depth == 2
        assert c.error_coeff == pytest.approx(2.0 / 9.0)

    def test_formulas(self):
        dt = 1e-12
        Qn, Qp, Qp2, dQ = np.array([1e-15, 2e-15]), np.array([0.5e-15, 1e-15]), np.array([0.25e-15, 0.5e-15]), \
            np.array([1e-3, 2e-3])
        np.testing.assert_allclose(P.apply_integration(Qn, Qp, P.compute_coefficients(P.BE, dt)), (Qn - Qp) / dt)
        np.testing.assert_allclose(P.apply_integration(Qn, Qp, P.compute_coefficients(P.TRAP, dt), dQdt_prev=dQ),
                                   2.0 / dt * (Qn - Qp) - dQ)
        np.testing.assert_allclose(P.apply_integration(Qn, Qp, P.compute_coefficients(P.GEAR2, dt), Q_prev2=Qp2),
                                   (3 * Qn - 4 * Qp + Qp2) / (2 * dt))

    def test_variable_bdf2_reduces_to_constant(self):
        c0, c1, c2 = P.variable_bdf2(1e-12, 1e-12)
        assert c0 == pytest.approx(1.5e12) and c1 == pytest.approx(-2e12) and c2 == pytest.approx(0.5e12)


class TestPredictor:
    def test_order_zero(self):
        c = P.compute_predictor_coeffs([], 1e-9, 1)
        assert c.order == 0 and c.a[0] == pytest.approx(1.0)

    def test_linear_uniform(self):
        c = P.compute_predictor_coeffs([1e-9], 1e-9, 1)
        assert c.order == 1
        np.testing.assert_allclose(c.a, [2.0, -1.0], rtol=1e-10)

    def test_quadratic_uniform(self):
        c = P.compute_predictor_coeffs([1e-9, 1e-9], 1e-9, 2)
        np.testing.assert_allclose(c.a, [3.0, -3.0, 1.0], rtol=1e-10)

    def test_variable_sums_to_one(self):
        c = P.compute_predictor_coeffs([2e-9, 1e-9], 1e-9, 2)
        assert sum(c.a) == pytest.approx(1.0, rel=1e-10)

    def test_order_limited(self):
        assert P.compute_predictor_coeffs([1e-9], 1e-9, 5).order == 1

    def test_predict_trends(self):
        c1 = P.compute_predictor_coeffs([1e-9], 1e-9, 1)
        np.testing.assert_allclose(P.predict(c1, [np.array([1.0, 2.0, 3.0])] * 2), [1.0, 2.0, 3.0])
        assert P.predict(c1, [np.array([2.0]), np.array([1.0])])[0] == pytest.approx(3.0)
        c2 = P.compute_predictor_coeffs([1e-9, 1e-9], 1e-9, 2)
        assert P.predict(c2, [np.array([4.0]), np.array([1.0]), np.array([0.0])])[0] == pytest.approx(9.0)

    def test_loop_predictor_matches_helpers(self):
        # adaptive.py's predictor (used in the loop) gives the same uniform-step coefficients
        Vh = np.zeros((4, 1))
        Vh[:3, 0] = [4.0, 1.0, 0.0]
        vp, err = P.predict_voltage(Vh, np.full(4, 1e-9), 3, 1e-9)
        assert vp[0] == pytest.approx(9.0)
        assert err == pytest.approx(-(-1.0) * (-2.0) * (-3.0) / 6)


class TestLTE:
    def test_scaling(self):
        lte = P.estimate_lte(np.array([1.0, 2.0]), np.array([1.1, 2.2]), -0.25, 0.5)
        np.testing.assert_allclose(lte, (0.5 / 0.75) * np.array([0.1, 0.2]), rtol=1e-10)
        np.testing.assert_allclose(P.estimate_lte(np.ones(3), np.ones(3), -0.25, 0.5), 0.0, atol=1e-15)

    def test_new_timestep(self):
        dt, r = P.compute_new_timestep(np.array([1e-6]), np.array([1.0]), 1e-3, 1e-6, 1.0, 1e-9, 1)
        assert dt > 1e-9 and r < 1.0
        dt, r = P.compute_new_timestep(np.array([1e-2]), np.array([1.0]), 1e-3, 1e-6, 1.0, 1e-9, 1)
        assert dt < 1e-9 and r > 1.0
        dt, _ = P.compute_new_timestep(np.array([1e-15]), np.array([1.0]), 1e-3, 1e-6, 1.0, 1e-9, 1, 1e-15, 1e-6)
        assert 1e-15 <= dt <= 1e-6

    def test_reject_threshold(self):
        dt, r = P.compute_new_timestep(np.array([1e-1]), np.array([1.0]), 1e-3, 1e-12, 3.5, 1e-9, 1)
        if r > 2.5:
            assert 1e-9 / dt > 2.5


def _divider():
    c = Circuit("divider")
    c.vsource("v1", "vsrc", "0", "dc", dc=1.0)
    c.add("r1", "resistor", ["vsrc", "node1"], r=1000.0)
    c.add("r2", "resistor", ["node1", "0"], r=1000.0)
    return c


def test_newton_resistive_divider():
    """tests/test_fori_loop_nr.py: V(node1)=0.5 V, V(vsrc)=1.0 V, I(V1)=-0.5 mA within 1e-10."""
    rc = _divider().resolve()
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    X = np.zeros(rc.n_nodes + 1)
    X[1:rc.n_nodes] = 0.5
    r = nr_solve(S, X, rc.source_values(0.0), max_iterations=100)
    assert r["converged"]
    X = r["X"]
    # reference assertion: jnp.allclose(X[1], 0.5, atol=1e-10) (default rtol 1e-5)
    assert np.isclose(X[rc.node_names["node1"]], 0.5, atol=1e-10)
    assert np.isclose(X[rc.node_names["vsrc"]], 1.0, atol=1e-10)
    # exact solution with gmin = 1e-12 on the node diagonal
    v1 = 1e-3 / (2e-3 + 1e-12)
    assert abs(X[rc.node_names["node1"]] - v1) < 1e-12
    assert abs(X[rc.node_names["vsrc"]] - 1.0) < 1e-12
    assert abs(X[rc.n_nodes] - (-(1.0 - v1) / 1000.0 - 1e-12)) < 1e-15
