"""Transient loops — FP64 test oracle.

Test infrastructure only (see ``oracle/mir_interp.py``).  Restates
``FullMNAStrategy._run_fixed_step`` (``vajax/analysis/transient/full_mna.py:
1198-1441``) and the adaptive while-loop body (``full_mna.py:1792-2196``) in
plain numpy on top of :func:`oracle.mna.nr_solve`.
"""

from __future__ import annotations

from typing import Dict

import numpy as np

from oracle.mna import OracleSystem, nr_solve
from oracle.predictor import lte_timestep, predict_voltage


def run_transient(sys_: OracleSystem, cfg: Dict[str, float], X0, Q0=None, I0=None, maxc0=None,
                  max_steps_run: int | None = None):
    rc = sys_.rc
    n_nodes, n_unk, n_v = sys_.n_nodes, sys_.n_unk, sys_.n_vsrc
    n_ext = int(cfg["n_external"])
    max_steps = int(cfg["max_steps"])
    t_stop, dt = cfg["t_stop"], cfg["dt"]
    reltol, abstol, vntol = cfg["reltol"], cfg["abstol"], cfg["vntol"]
    itl = int(cfg["tran_itl"])
    method = int(cfg["method"])
    conv_mask = None
    if rc.internal_nodes:
        conv_mask = np.ones(sys_.n_aug, bool)
        conv_mask[np.asarray(rc.internal_nodes) - 1] = False
    X = np.array(X0, np.float64)
    z = np.zeros(n_unk)
    Q_prev = z.copy() if Q0 is None else np.array(Q0, np.float64)
    dQdt_prev = z.copy()
    Q_prev2 = z.copy()
    nvo = max(n_v, 1)
    times = np.zeros(max_steps)
    V_out = np.zeros((max_steps, n_ext))
    I_out = np.zeros((max_steps, nvo))
    V_out[0] = X[:n_ext]
    total_nr = 0
    nr_fail = 0

    def isrc(t):
        return rc.source_values(t, True) if rc.isources else np.zeros(0)

    if cfg["fixed_step"]:
        n_steps = min(int(t_stop / dt), max_steps - 1)
        n_steps = max(n_steps, 1)
        if max_steps_run is not None:
            n_steps = min(n_steps, max_steps_run)
        inv = 1.0 / dt
        c0, c1, d1, c2 = inv, -inv, 0.0, 0.0
        if method == 1:
            c0, c1, d1 = 2 * inv, -2 * inv, -1.0
        elif method == 2:
            c0, c1, c2 = 1.5 * inv, -2.0 * inv, 0.5 * inv
        floor_ = np.full(n_unk, abstol)
        for i in range(n_steps):
            t_next = (float(i) + 1.0) * dt
            r = nr_solve(sys_, X, rc.source_values(t_next), isrc(t_next), Q_prev, c0, 0.0, c1, d1, dQdt_prev, c2,
                         Q_prev2, res_tol_floor=floor_, max_iterations=itl, reltol=reltol, abstol=abstol,
                         vntol=vntol, nr_damping=cfg["nr_damping"], conv_mask=conv_mask)
            total_nr += r["iterations"]
            nr_fail += 0 if r["converged"] else 1
            times[i + 1] = t_next
            V_out[i + 1] = r["X"][:n_ext]
            if n_v:
                I_out[i + 1, :n_v] = r["I_vsource"]
            X = r["X"]
            Q_prev2 = Q_prev
            Q_prev = r["Q"]
            dQdt_prev = r["dQdt"]
        n = n_steps + 1
        return dict(times=times[:n], V=V_out[:n], I=I_out[:n, :n_v], n_steps=n, rejected=0,
                    total_nr_iters=total_nr, nr_failures=nr_fail)

    # adaptive loop
    if I0 is not None and n_v:
        I_out[0, :n_v] = I0
    max_history = 4
    V_hist = np.zeros((max_history, n_nodes))
    V_hist[0] = X[:n_nodes]
    dt_hist = np.full(max_history, dt)
    hc, warm, consec = 1, 0, 0
    t = 0.0
    step_idx = 1
    rejected = 0
    Vmax = np.abs(X[:n_nodes])
    hmaxc = z.copy() if maxc0 is None else np.array(maxc0, np.float64)
    min_dt, max_dt = cfg["min_dt"], cfg["max_dt"]
    loops = 0
    while t < t_stop and step_idx < max_steps:
        if max_steps_run is not None and loops >= max_steps_run:
            break
        loops += 1
        dt_cur = dt
        inv = 1.0 / dt_cur
        if method == 0:
            c0, c1, d1, c2, err_i = inv, -inv, 0.0, 0.0, -0.5
        elif method == 1:
            c0, c1, d1, c2, err_i = 2 * inv, -2 * inv, -1.0, 0.0, 1.0 / 24.0
        else:
            dtp = dt_hist[0]
            w = dt_cur / dtp if dtp > 0 else 1.0
            wp1 = 1.0 + w
            c0, c1, d1, c2 = (1 + 2 * w) / (wp1 * dt_cur), -wp1 / dt_cur, 0.0, (w * w) / (wp1 * dt_cur)
            err_i = -2.0 / 9.0
        t_next = t + dt_cur
        can_predict = warm >= int(cfg["warmup_steps"]) and hc >= 2
        V_pred, pred_err = predict_voltage(V_hist, dt_hist, hc, dt_cur, 2)
        X_init = X.copy()
        if can_predict:
            X_init[:n_nodes] = V_pred
        gs = int(cfg["gshunt_steps"])
        ramp = min(max(step_idx / gs, 0.0), 1.0) if gs > 0 else 1.0
        gshunt = cfg["gshunt_init"] + ramp * (cfg["gshunt_target"] - cfg["gshunt_init"])
        floor_ = np.maximum(hmaxc * reltol, abstol)
        r = nr_solve(sys_, X_init, rc.source_values(t_next), isrc(t_next), Q_prev, c0, gshunt, c1, d1, dQdt_prev, c2,
                     Q_prev2, res_tol_floor=floor_, max_iterations=itl, reltol=reltol, abstol=abstol, vntol=vntol,
                     nr_damping=cfg["nr_damping"], conv_mask=conv_mask)
        total_nr += r["iterations"]
        conv = r["converged"]
        nr_failed = not conv
        nr_fail += 1 if nr_failed else 0
        at_min = dt_cur <= min_dt
        nr_failed_at_min = nr_failed and at_min
        V_new = r["X"][:n_nodes]
        dt_lte, _ = lte_timestep(V_new, V_pred, pred_err, dt_cur, hc, reltol, abstol, cfg["lte_ratio"],
                                 cfg["grow_factor"], err_i, Vmax)
        lte_reject = (dt_cur / dt_lte > cfg["redo_factor"]) and can_predict and conv
        nr_reject = nr_failed and not at_min
        force = consec >= int(cfg["max_consecutive_rejects"])
        reject = (lte_reject or nr_reject) and not force
        accept = not reject
        consec = 0 if accept else (consec + 1 if lte_reject else consec)
        dt_from_lte = dt_lte if can_predict else dt_cur
        dt_halved = max(dt_cur * cfg["tran_ft"], min_dt)
        last_good = dt_hist[0] if hc > 0 else min_dt * 16
        dt_rec = max(last_good / 8.0, min_dt * 2.0)
        new_dt = (dt_rec if at_min else dt_halved) if nr_failed else dt_from_lte
        new_dt = min(max(new_dt, min_dt), max_dt)
        new_dt = min(new_dt, t_stop - t_next)
        use_new = accept and not nr_failed_at_min
        if use_new:
            X = r["X"].copy()
            Q_prev2 = Q_prev
            Q_prev = r["Q"]
            dQdt_prev = r["dQdt"]
            V_hist = np.roll(V_hist, 1, axis=0)
            V_hist[0] = V_new
            dt_hist = np.roll(dt_hist, 1)
            dt_hist[0] = dt_cur
            hc = min(hc + 1, max_history)
            warm += 1
            Vmax = np.maximum(Vmax, np.abs(V_new))
            hmaxc = np.maximum(hmaxc, r["max_res_contrib"])
        if accept:
            times[step_idx] = t_next
            V_out[step_idx] = X[:n_ext]
            if n_v:
                I_out[step_idx, :n_v] = 0.0 if nr_failed_at_min else r["I_vsource"]
            step_idx += 1
            t = t_next
        if reject:
            rejected += 1
        dt = new_dt
    n = step_idx
    return dict(times=times[:n], V=V_out[:n], I=I_out[:n, :n_v], n_steps=n, rejected=rejected,
                total_nr_iters=total_nr, nr_failures=nr_fail)
