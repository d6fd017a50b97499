"""Integration coefficients, predictor and LTE helpers — test oracle only.

Test infrastructure (see ``oracle/mir_interp.py`` for the usage rule).  Plain
numpy restatements of:

* ``vajax/analysis/integration.py:88-183`` (``compute_coefficients``,
  ``apply_integration``);
* ``vajax/analysis/transient/predictor.py:38-309`` (the NumPy predictor/LTE
  helpers the reference's ``tests/test_adaptive_timestep.py`` pins);
* ``vajax/analysis/transient/adaptive.py:94-339`` (``predict_voltage_jax`` and
  ``compute_lte_timestep_jax``, the versions the transient loop runs).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np

BE, TRAP, GEAR2 = 0, 1, 2


@dataclass
class IntegrationCoeffs:
    c0: float
    c1: float
    c2: float
    d1: float
    history_depth: int
    needs_dqdt_history: bool
    error_coeff: float


def compute_coefficients(method: int, dt: float) -> IntegrationCoeffs:
    """integration.py:88-138."""
    inv = 1.0 / dt
    if method == BE:
        return IntegrationCoeffs(inv, -inv, 0.0, 0.0, 1, False, 0.5)
    if method == TRAP:
        return IntegrationCoeffs(2.0 * inv, -2.0 * inv, 0.0, -1.0, 1, True, 1.0 / 12.0)
    if method == GEAR2:
        return IntegrationCoeffs(1.5 * inv, -2.0 * inv, 0.5 * inv, 0.0, 2, False, 2.0 / 9.0)
    raise ValueError(method)


def apply_integration(Q_new, Q_prev, c: IntegrationCoeffs, Q_prev2=None, dQdt_prev=None):
    """integration.py:141-166."""
    d = c.c0 * np.asarray(Q_new) + c.c1 * np.asarray(Q_prev)
    if c.history_depth >= 2 and Q_prev2 is not None:
        d = d + c.c2 * np.asarray(Q_prev2)
    if c.needs_dqdt_history and dQdt_prev is not None:
        d = d + c.d1 * np.asarray(dQdt_prev)
    return d


def variable_bdf2(dt: float, dt_prev: float) -> Tuple[float, float, float]:
    """Variable-step BDF2 coefficients (full_mna.py:1864-1891)."""
    w = dt / dt_prev if dt_prev > 0 else 1.0
    wp1 = 1.0 + w
    return (1.0 + 2.0 * w) / (wp1 * dt), -wp1 / dt, (w * w) / (wp1 * dt)


@dataclass
class PredictorCoeffs:
    a: np.ndarray
    error_coeff: float
    order: int


def compute_predictor_coeffs(past_dt: Sequence[float], new_dt: float, order: int) -> PredictorCoeffs:
    """predictor.py:38-91: Lagrange extrapolation to t_{n+1} from past points."""
    if order < 1:
        raise ValueError(f"Order must be >= 1, got {order}")
    if len(past_dt) < order:
        order = len(past_dt)
    if order == 0:
        return PredictorCoeffs(np.array([1.0]), 1.0, 0)
    tau = np.zeros(order + 1)
    cum = 0.0
    for i in range(order + 1):
        tau[i] = -(1.0 + cum / new_dt)
        if i < len(past_dt):
            cum += past_dt[i]
    n = order + 1
    A = np.array([[tau[i] ** j for i in range(n)] for j in range(n)])
    b = np.zeros(n)
    b[0] = 1.0
    try:
        a = np.linalg.solve(A, b)
    except np.linalg.LinAlgError:
        a = np.zeros(n)
        a[0] = 1.0
    err = -1.0 + sum(a[i] * tau[i] ** (order + 1) for i in range(n))
    return PredictorCoeffs(a, float(err), order)


def predict(coeffs: PredictorCoeffs, V_history: List[np.ndarray]) -> np.ndarray:
    """predictor.py:190-215."""
    if not V_history:
        raise ValueError("Need at least one past solution for prediction")
    n = len(coeffs.a)
    hist = list(V_history) + [V_history[-1]] * max(0, n - len(V_history))
    out = coeffs.a[0] * np.asarray(hist[0])
    for i in range(1, n):
        out = out + coeffs.a[i] * np.asarray(hist[i])
    return out


def estimate_lte(V_pred, V_corr, pred_err: float, integ_err: float) -> np.ndarray:
    """predictor.py:218-249."""
    denom = integ_err - pred_err
    if abs(denom) < 1e-15:
        return np.asarray(V_corr) - np.asarray(V_pred)
    return (integ_err / denom) * (np.asarray(V_corr) - np.asarray(V_pred))


def compute_new_timestep(lte, V_ref, reltol, abstol, lte_ratio, current_dt, order, min_dt=1e-18,
                         max_dt=float("inf")) -> Tuple[float, float]:
    """predictor.py:252-309."""
    tol = np.maximum(np.abs(V_ref) * reltol, abstol)
    ratios = np.abs(lte) / (tol * lte_ratio)
    max_ratio = float(np.max(ratios))
    if max_ratio > 0:
        dt_new = current_dt * max_ratio ** (-1.0 / (order + 1))
    else:
        dt_new = current_dt * 2.0
    return max(min_dt, min(max_dt, dt_new)), max_ratio


def predict_voltage(V_history: np.ndarray, dt_history: np.ndarray, history_count: int, new_dt: float,
                    max_order: int = 2) -> Tuple[np.ndarray, float]:
    """adaptive.py:94-218 (the predictor the transient loop runs)."""
    order = max(min(history_count - 1, max_order), 0)
    cum = np.cumsum(dt_history)
    tau = -(new_dt + np.concatenate([[0.0], cum[:-1]])) / new_dt
    ratio1 = new_dt / max(dt_history[0], 1e-30)
    a1 = np.array([1.0 + ratio1, -ratio1, 0.0])
    err1 = -ratio1 * (1 + ratio1) / 2
    tau0, tau1, tau2 = -1.0, tau[1], tau[2]

    def floor(d):
        return 1e-30 if abs(d) < 1e-30 else d

    d0 = floor((tau0 - tau1) * (tau0 - tau2))
    d1 = floor((tau1 - tau0) * (tau1 - tau2))
    d2 = floor((tau2 - tau0) * (tau2 - tau1))
    a2 = np.array([(0 - tau1) * (0 - tau2) / d0, (0 - tau0) * (0 - tau2) / d1, (0 - tau0) * (0 - tau1) / d2])
    err2 = -tau0 * tau1 * tau2 / 6
    if order == 0:
        a, err = np.array([1.0, 0.0, 0.0]), 1.0
    elif order == 1:
        a, err = a1, err1
    else:
        a, err = a2, err2
    a = np.where(np.arange(3) <= order, a, 0.0)
    return np.einsum("i,ij->j", a, V_history[:3]), float(err)


def lte_timestep(V_new, V_pred, pred_err, dt, history_count, reltol, abstol, lte_ratio, grow_factor, integ_err,
                 V_max_historic, max_order=2) -> Tuple[float, float]:
    """adaptive.py:221-339."""
    lte = (V_new - V_pred) * (integ_err / (integ_err - pred_err))
    Vcur = np.maximum(np.abs(V_new), np.abs(V_pred))
    Vs = np.maximum(V_max_historic, Vcur)
    tol = reltol * Vs + abstol
    norm = float(np.max(np.abs(lte) / tol))
    order = min(history_count - 1, max_order)
    factor = (lte_ratio / max(norm, 1e-10)) ** (1.0 / (order + 1))
    factor = min(max(factor, 0.1), grow_factor)
    return dt * factor, norm
