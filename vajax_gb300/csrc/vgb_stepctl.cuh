// Transient step controller, shared by the host-driven step loop and the
// one-thread kernels of the step graph (both instantiate the templates on
// their own state struct, which carries the same field names).
#pragma once

#include <cmath>

namespace vgb {

// ---------------------------------------------------------------------------
// predictor coefficients (adaptive.py:94-178)
// ---------------------------------------------------------------------------

struct Pred {
    double a[3];
    double err;
};

__host__ __device__ inline Pred predictor_coeffs(const double dt_hist[4], int history_count, double new_dt,
                                                 int max_order) {
    int order = history_count - 1 < max_order ? history_count - 1 : max_order;
    order = order > 0 ? order : 0;
    const double cum0 = 0.0, cum1 = dt_hist[0];
    (void)cum0;
    const double tau1 = -(new_dt + cum1) / new_dt;
    const double tau2 = -(new_dt + dt_hist[0] + dt_hist[1]) / new_dt;
    Pred p{};
    if (order == 0) {
        p.a[0] = 1.0; p.a[1] = 0.0; p.a[2] = 0.0;
        p.err = 1.0;
    } else if (order == 1) {
        const double r1 = new_dt / fmax(dt_hist[0], 1e-30);
        p.a[0] = 1.0 + r1; p.a[1] = -r1; p.a[2] = 0.0;
        p.err = -r1 * (1 + r1) / 2;
    } else {
        const double tau0 = -1.0;
        double d0 = (tau0 - tau1) * (tau0 - tau2);
        double d1 = (tau1 - tau0) * (tau1 - tau2);
        double d2 = (tau2 - tau0) * (tau2 - tau1);
        if (fabs(d0) < 1e-30) d0 = 1e-30;
        if (fabs(d1) < 1e-30) d1 = 1e-30;
        if (fabs(d2) < 1e-30) d2 = 1e-30;
        p.a[0] = (0 - tau1) * (0 - tau2) / d0;
        p.a[1] = (0 - tau0) * (0 - tau2) / d1;
        p.a[2] = (0 - tau0) * (0 - tau1) / d2;
        p.err = -tau0 * tau1 * tau2 / 6;
    }
    return p;
}


// ---------------------------------------------------------------------------
// Step controller (full_mna.py:1236-1253 fixed coefficients, :1851-1891 BDF2
// coefficients, :1984-2147 LTE control and commit; adaptive.py:94-339).  One
// implementation for both step loops: the host-driven loop calls it on the
// session and the transient graph calls it from one-thread kernels on the
// device state.  S is either; both carry the same field names.
// ---------------------------------------------------------------------------

struct StepPlan {
    double k[5];  // c0, c1, d1, c2, gshunt
    double t_next, kl, pa[3];
    int can_predict, slot[3];
};

struct StepCommit {
    int use_new, accept, zero_current, row, slot;
};

template <class S>
__host__ __device__ inline StepPlan ctl_plan(const S& s) {
    StepPlan p{};
    const double dt_cur = s.dt;
    const double inv = 1.0 / dt_cur;
    p.k[0] = inv;
    p.k[1] = -inv;
    if (s.fixed) {
        if (s.method == 1) { p.k[0] = 2 * inv; p.k[1] = -2 * inv; p.k[2] = -1.0; }
        else if (s.method == 2) { p.k[0] = 1.5 * inv; p.k[1] = -2.0 * inv; p.k[3] = 0.5 * inv; }
        p.t_next = ((double)s.fixed_i + 1.0) * dt_cur;
        return p;
    }
    double err_integ;
    if (s.method == 0) {
        err_integ = -0.5;
    } else if (s.method == 1) {
        p.k[0] = 2 * inv; p.k[1] = -2 * inv; p.k[2] = -1.0;
        err_integ = 1.0 / 24.0;
    } else {
        const double dt_prev = s.dt_hist[0];
        const double w = dt_prev > 0 ? dt_cur / dt_prev : 1.0;
        const double wp1 = 1.0 + w;
        p.k[0] = (1.0 + 2.0 * w) / (wp1 * dt_cur);
        p.k[1] = -wp1 / dt_cur;
        p.k[3] = (w * w) / (wp1 * dt_cur);
        err_integ = -2.0 / 9.0;
    }
    p.t_next = s.t + dt_cur;
    p.can_predict = (s.warmup_count >= s.warmup_steps && s.history_count >= 2) ? 1 : 0;
    const Pred pr = predictor_coeffs(s.dt_hist, s.history_count, dt_cur, 2);
    int order = s.history_count - 1 < 2 ? s.history_count - 1 : 2;
    order = order > 0 ? order : 0;
    p.pa[0] = pr.a[0];
    p.pa[1] = order >= 1 ? pr.a[1] : 0.0;
    p.pa[2] = order >= 2 ? pr.a[2] : 0.0;
    for (int q = 0; q < 3; ++q) p.slot[q] = (s.head + q) % 4;
    const double ramp = s.gshunt_steps > 0 ? fmin(fmax((double)s.step_idx / s.gshunt_steps, 0.0), 1.0) : 1.0;
    p.k[4] = s.gshunt_init + ramp * (s.gshunt_target - s.gshunt_init);
    p.kl = err_integ / (err_integ - pr.err);
    return p;
}

// Accept / reject, next dt, history update and the commit of the step; writes
// the accepted time into tout.  Returns the commit parameters.
template <class S>
__host__ __device__ inline StepCommit ctl_finish(S& s, const StepPlan& p, double lte_norm, int nr_iters,
                                                 bool converged, double* tout) {
    StepCommit m{};
    s.total_nr += nr_iters;
    const bool nr_failed = !converged;
    if (nr_failed) s.nr_fail_count++;
    if (s.fixed) {
        const int i = s.fixed_i;
        m.use_new = 1; m.accept = 1; m.zero_current = 0; m.row = i + 1; m.slot = (i + 1) % 4;
        tout[i + 1] = p.t_next;
        s.fixed_i = i + 1;
        s.step_idx = s.fixed_i + 1;
        if (s.fixed_i >= s.fixed_n) s.done = true;
        return m;
    }
    const double dt_cur = s.dt;
    const int lte_order = s.history_count - 1 < 2 ? s.history_count - 1 : 2;
    double factor = pow(s.lte_ratio / fmax(lte_norm, 1e-10), 1.0 / (lte_order + 1));
    factor = fmin(fmax(factor, 0.1), s.grow_factor);
    const double dt_lte = dt_cur * factor;
    const bool at_min_dt = dt_cur <= s.min_dt;
    const bool nr_failed_at_min = nr_failed && at_min_dt;
    const bool lte_reject = (dt_cur / dt_lte > s.redo_factor) && p.can_predict && converged;
    const bool nr_reject = nr_failed && !at_min_dt;
    const bool force_accept = s.consecutive >= s.max_consec;
    const bool reject = (lte_reject || nr_reject) && !force_accept;
    const bool accept = !reject;
    s.consecutive = accept ? 0 : (lte_reject ? s.consecutive + 1 : s.consecutive);
    const double dt_from_lte = p.can_predict ? dt_lte : dt_cur;
    const double dt_nr_halved = fmax(dt_cur * s.tran_ft, s.min_dt);
    const double last_good = s.history_count > 0 ? s.dt_hist[0] : s.min_dt * 16.0;
    const double dt_recovery = fmax(last_good / 8.0, s.min_dt * 2.0);
    double new_dt = nr_failed ? (at_min_dt ? dt_recovery : dt_nr_halved) : dt_from_lte;
    new_dt = fmin(fmax(new_dt, s.min_dt), s.max_dt);
    new_dt = fmin(new_dt, s.t_stop - p.t_next);
    const bool use_new = accept && !nr_failed_at_min;
    const int new_head = use_new ? (s.head + 3) % 4 : s.head;
    m.use_new = use_new ? 1 : 0;
    m.accept = accept ? 1 : 0;
    m.zero_current = nr_failed_at_min ? 1 : 0;
    m.row = s.step_idx;
    m.slot = new_head;
    if (use_new) {
        s.head = new_head;
        for (int q = 3; q > 0; --q) s.dt_hist[q] = s.dt_hist[q - 1];
        s.dt_hist[0] = dt_cur;
        s.history_count = s.history_count + 1 < 4 ? s.history_count + 1 : 4;
        s.warmup_count++;
    }
    if (accept) {
        tout[s.step_idx] = p.t_next;
        s.t = p.t_next;
        s.step_idx++;
        s.min_dt_used = fmin(s.min_dt_used, dt_cur);
        s.max_dt_used = fmax(s.max_dt_used, dt_cur);
    }
    if (reject) s.rejected++;
    s.dt = new_dt;
    if (!(s.t < s.t_stop && s.step_idx < s.max_steps)) s.done = true;
    return m;
}

} // namespace vgb
