// The transient step controller (vgb_stepctl.cuh) replayed on the host from a
// script of Newton outcomes and LTE norms (test infrastructure).  The state is
// initialised as a transient session's setup does.
#include <algorithm>

#include "vgb_stepctl.cuh"

using namespace vgb;

namespace {
struct Ctl {
    double t_stop, max_dt, min_dt, lte_ratio, redo_factor, grow_factor, tran_ft, gshunt_init, gshunt_target;
    int gshunt_steps, warmup_steps, max_consec, method, max_steps, fixed, fixed_n;
    double t, dt, dt_hist[4];
    int head, history_count, warmup_count, consecutive, step_idx, fixed_i;
    long long total_nr;
    int rejected, nr_fail_count;
    bool done;
    double min_dt_used, max_dt_used;
};
}  // namespace

// cfg: the 22-value transient configuration (vgb_transient layout).  Attempt a
// takes nr_iters[a], converged[a] and lte_norm[a].  Writes per attempt
// plan[11a..11a+10] = c0, c1, d1, c2, gshunt, t_next, kl, can_predict and the
// predictor weights of the three latest solutions (newest first), and
// commit[2a..2a+1] = accept, use_new; times[max_steps] the accepted times;
// summary = attempts, step_idx, rejected, total_nr, nr_failures, t, dt, done.
// Returns 0, or 1 when the script ran out before the run was done.
extern "C" int ctl_replay(const double* cfg, int n_script, const int* nr_iters, const int* converged,
                          const double* lte_norm, double* plan, int* commit, double* times, double* summary) {
    Ctl s{};
    s.t_stop = cfg[0];
    s.dt = cfg[1];
    s.max_dt = cfg[2];
    s.min_dt = cfg[3];
    s.lte_ratio = cfg[7];
    s.redo_factor = cfg[8];
    s.grow_factor = cfg[9];
    s.tran_ft = cfg[10];
    s.gshunt_init = cfg[12];
    s.gshunt_target = cfg[13];
    s.gshunt_steps = (int)cfg[14];
    s.warmup_steps = (int)cfg[15];
    s.max_consec = (int)cfg[16];
    s.fixed = cfg[17] != 0.0;
    s.method = (int)cfg[18];
    s.max_steps = (int)cfg[20];
    s.t = 0.0;
    for (double& d : s.dt_hist) d = s.dt;
    s.head = 0;
    s.history_count = 1;
    s.step_idx = 1;
    s.min_dt_used = s.max_dt_used = s.dt;
    if (s.fixed) s.fixed_n = std::max(1, std::min((int)(s.t_stop / s.dt), s.max_steps - 1));
    s.done = !s.fixed && !(s.t < s.t_stop && s.step_idx < s.max_steps);
    int a = 0;
    for (; !s.done && a < n_script; ++a) {
        const StepPlan p = ctl_plan(s);
        double* o = plan + 11 * a;
        for (int q = 0; q < 5; ++q) o[q] = p.k[q];
        o[5] = p.t_next;
        o[6] = p.kl;
        o[7] = p.can_predict;
        for (int q = 0; q < 3; ++q) o[8 + q] = p.pa[q];
        const StepCommit m = ctl_finish(s, p, lte_norm[a], nr_iters[a], converged[a] != 0, times);
        commit[2 * a] = m.accept;
        commit[2 * a + 1] = m.use_new;
    }
    summary[0] = a;
    summary[1] = s.fixed ? s.fixed_i + 1 : s.step_idx;
    summary[2] = s.rejected;
    summary[3] = (double)s.total_nr;
    summary[4] = s.nr_fail_count;
    summary[5] = s.t;
    summary[6] = s.dt;
    summary[7] = s.done ? 1 : 0;
    return s.done ? 0 : 1;
}
