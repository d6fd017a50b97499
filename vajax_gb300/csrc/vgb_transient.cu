// Device-resident transient analysis: fixed-step and adaptive BDF2/trap/BE
// with the polynomial predictor and LTE step control of the reference
// (vajax/analysis/transient/full_mna.py:1198-1441 fixed step, :1792-2196
// adaptive body; vajax/analysis/transient/adaptive.py:94-339 predictor/LTE).
//
// All vectors stay on the GPU.  The host keeps only the scalar controller
// state (t, dt, history ring indices, counters) and reads one small status
// record per Newton iteration.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "vgb_core.h"

namespace vgb {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

__global__ void dqdt_kernel(const double* Q, const double* Qp, const double* dQp, const double* Qp2, double c0,
                            double c1, double d1, double c2, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = c0 * Q[i] + c1 * Qp[i] + d1 * dQp[i] + c2 * Qp2[i];
}

void launch_dqdt(const double* Q, const double* Qp, const double* dQp, const double* Qp2, double c0, double c1,
                 double d1, double c2, double* out, int n, cudaStream_t s) {
    if (n) dqdt_kernel<<<ceil_div(n, 256), 256, 0, s>>>(Q, Qp, dQp, Qp2, c0, c1, d1, c2, out, n);
}

// X_init (predictor, full_mna.py:1897-1911) and the historic NR tolerance
// floor (full_mna.py:1925-1928).
__global__ void predict_kernel(int n_nodes, int n_x, int n_unk, const double* X, double* Xc, double* Vpred,
                               const double* h0, const double* h1, const double* h2, double a0, double a1,
                               double a2, int can_predict, const double* hist_maxc, double reltol, double abstol,
                               double* floor_) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_nodes) {
        const double vp = a0 * h0[i] + a1 * h1[i] + a2 * h2[i];
        Vpred[i] = vp;
        Xc[i] = can_predict ? vp : X[i];
    } else if (i < n_x) {
        Xc[i] = X[i];
    }
    if (i < n_unk) floor_[i] = hist_maxc ? fmax(hist_maxc[i] * reltol, abstol) : abstol;
}

// LTE norm (adaptive.py:221-264): max_i |(V_new - V_pred) * k| / (reltol * V_scale + abstol)
__global__ void lte_kernel(int n_nodes, const double* Vnew, const double* Vpred, const double* Vmax, double k,
                           double reltol, double abstol, NRStatus* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n_nodes) {
        const double lte = (Vnew[i] - Vpred[i]) * k;
        const double vcur = fmax(fabs(Vnew[i]), fabs(Vpred[i]));
        const double vs = fmax(Vmax[i], vcur);
        const double tol = reltol * vs + abstol;
        v = fabs(lte) / tol;
        if (v != v) v = INFINITY;
    }
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && i < n_nodes + 32)
        atomicMax(&st->lte_norm, (unsigned long long)__double_as_longlong(v));
}

// Accept / reject commit (full_mna.py:2078-2147).
__global__ void commit_kernel(int n_nodes, int n_x, int n_unk, int n_ext, int n_vsrc, int use_new, int accept,
                              int zero_current, const double* Xc, double* X, const double* Q, double* Qp,
                              const double* dQ, double* dQp, double* Qp2, double* hist_slot, double* Vmax,
                              const double* maxc, double* hist_maxc, const double* Ivs, double* Vout_row,
                              double* Iout_row) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (use_new) {
        if (i < n_x) X[i] = Xc[i];
        if (i < n_unk) {
            Qp2[i] = Qp[i];
            Qp[i] = Q[i];
            dQp[i] = dQ[i];
            hist_maxc[i] = fmax(hist_maxc[i], maxc[i]);
        }
        if (i < n_nodes) {
            hist_slot[i] = Xc[i];
            Vmax[i] = fmax(Vmax[i], fabs(Xc[i]));
        }
    }
    if (accept) {
        if (i < n_ext) Vout_row[i] = use_new ? Xc[i] : X[i];
        if (i < n_vsrc) Iout_row[i] = zero_current ? 0.0 : Ivs[i];
    }
}

static double bits_to_double(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

// ---------------------------------------------------------------------------
// predictor coefficients (adaptive.py:94-178)
// ---------------------------------------------------------------------------

struct Pred {
    double a[3];
    double err;
};

static Pred predictor_coeffs(const double dt_hist[4], int history_count, double new_dt, int max_order) {
    int order = std::min(history_count - 1, max_order);
    order = std::max(order, 0);
    const double cum0 = 0.0, cum1 = dt_hist[0];
    (void)cum0;
    const double tau1 = -(new_dt + cum1) / new_dt;
    const double tau2 = -(new_dt + dt_hist[0] + dt_hist[1]) / new_dt;
    Pred p{};
    if (order == 0) {
        p.a[0] = 1.0; p.a[1] = 0.0; p.a[2] = 0.0;
        p.err = 1.0;
    } else if (order == 1) {
        const double r1 = new_dt / std::max(dt_hist[0], 1e-30);
        p.a[0] = 1.0 + r1; p.a[1] = -r1; p.a[2] = 0.0;
        p.err = -r1 * (1 + r1) / 2;
    } else {
        const double tau0 = -1.0;
        double d0 = (tau0 - tau1) * (tau0 - tau2);
        double d1 = (tau1 - tau0) * (tau1 - tau2);
        double d2 = (tau2 - tau0) * (tau2 - tau1);
        if (std::fabs(d0) < 1e-30) d0 = 1e-30;
        if (std::fabs(d1) < 1e-30) d1 = 1e-30;
        if (std::fabs(d2) < 1e-30) d2 = 1e-30;
        p.a[0] = (0 - tau1) * (0 - tau2) / d0;
        p.a[1] = (0 - tau0) * (0 - tau2) / d1;
        p.a[2] = (0 - tau0) * (0 - tau1) / d2;
        p.err = -tau0 * tau1 * tau2 / 6;
    }
    return p;
}

// ---------------------------------------------------------------------------
// Resumable transient session: configuration, device state and the host-side
// step controller of one transient run on a circuit.
// ---------------------------------------------------------------------------

struct TranSession {
    Circuit* c = nullptr;
    // configuration (vgb_transient cfg layout)
    double t_stop = 0, max_dt = 0, min_dt = 0, reltol = 0, abstol = 0, vntol = 0, lte_ratio = 0, redo_factor = 0;
    double grow_factor = 0, tran_ft = 0, gshunt_init = 0, gshunt_target = 0;
    int gshunt_steps = 0, warmup_steps = 0, max_consec = 0, method = 2, n_ext = 0, max_steps = 0, tran_itl = 20;
    bool fixed = false;
    NROpts o;
    // device state
    DevBuf<double> X, Xc, Qp, Qp2, dQp, dQn, Vpred, Vmax, hmaxc, floor_, vs, is, Ivs, hist, Vout, Iout;
    std::vector<double> tout;
    // controller state
    double t = 0.0, dt = 0.0, dt_hist[4] = {0, 0, 0, 0};
    int head = 0, history_count = 1, warmup_count = 0, consecutive = 0;
    int step_idx = 1, fixed_i = 0, fixed_n = 0;
    long long total_nr = 0;
    int rejected = 0, nr_fail_count = 0;
    double min_dt_used = 0, max_dt_used = 0;
    double device_ms = 0;
    long long launches0 = 0;
    bool done = false;

    void setup(Circuit* cc, const double* cfg, const double* X0, const double* Q0, const double* I0,
               const double* maxc0);
    int advance(int max_accepted);
    int n_x() const { return c->n_nodes + c->n_vsrc; }
};

void TranSession::setup(Circuit* cc, const double* cfg, const double* X0, const double* Q0, const double* I0,
                        const double* maxc0) {
    c = cc;
    t_stop = cfg[0];
    dt = cfg[1];
    max_dt = cfg[2]; min_dt = cfg[3];
    reltol = cfg[4]; abstol = cfg[5]; vntol = cfg[6];
    lte_ratio = cfg[7]; redo_factor = cfg[8]; grow_factor = cfg[9]; tran_ft = cfg[10];
    const double nr_damping = cfg[11];
    gshunt_init = cfg[12]; gshunt_target = cfg[13];
    gshunt_steps = (int)cfg[14]; warmup_steps = (int)cfg[15];
    max_consec = (int)cfg[16];
    fixed = cfg[17] != 0.0;
    method = (int)cfg[18];
    n_ext = (int)cfg[19];
    max_steps = (int)cfg[20];
    tran_itl = (int)cfg[21];
    VGB_REQUIRE(n_ext >= 1 && n_ext <= c->n_nodes, "n_external out of range");
    VGB_REQUIRE(max_steps >= 1, "max_steps must be >= 1");
    VGB_REQUIRE(dt > 0 && t_stop >= 0, "bad time parameters");
    VGB_REQUIRE(method >= 0 && method <= 2, "method must be 0 (BE), 1 (trap) or 2 (gear2)");
    VGB_REQUIRE(tran_itl >= 1, "tran_itl must be >= 1");
    VGB_REQUIRE(X0 != nullptr, "X0 is required");
    cudaStream_t s = c->stream;
    const int n_nodes = c->n_nodes, n_unk = c->n_unk, n_vsrc = c->n_vsrc;
    const int nx = n_x();
    const int nvo = std::max(n_vsrc, 1);
    X.alloc(nx);
    Xc.alloc(nx);
    const size_t nu = std::max(n_unk, 1);
    Qp.alloc(nu); Qp2.alloc(nu); dQp.alloc(nu); dQn.alloc(nu); hmaxc.alloc(nu); floor_.alloc(nu);
    Vpred.alloc(n_nodes); Vmax.alloc(n_nodes);
    vs.alloc(std::max(n_vsrc, 1)); is.alloc(std::max(c->n_isrc, 1)); Ivs.alloc(nvo);
    hist.alloc(4 * (size_t)n_nodes);
    Vout.alloc((size_t)max_steps * n_ext);
    Iout.alloc((size_t)max_steps * nvo);
    Qp2.zero(s); dQp.zero(s); hist.zero(s); Vout.zero(s); Iout.zero(s); is.zero(s); vs.zero(s);
    VGB_CUDA(cudaMemcpyAsync(X.p, X0, nx * sizeof(double), cudaMemcpyHostToDevice, s));
    if (Q0) VGB_CUDA(cudaMemcpyAsync(Qp.p, Q0, n_unk * sizeof(double), cudaMemcpyHostToDevice, s));
    else Qp.zero(s);
    if (maxc0) VGB_CUDA(cudaMemcpyAsync(hmaxc.p, maxc0, n_unk * sizeof(double), cudaMemcpyHostToDevice, s));
    else hmaxc.zero(s);
    // V_history[0] = X0[:n_total]; V_max_historic = |X0|
    std::vector<double> vmax0(n_nodes);
    for (int i = 0; i < n_nodes; ++i) vmax0[i] = std::fabs(X0[i]);
    VGB_CUDA(cudaMemcpyAsync(hist.p, X0, n_nodes * sizeof(double), cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpyAsync(Vmax.p, vmax0.data(), n_nodes * sizeof(double), cudaMemcpyHostToDevice, s));
    // initial outputs (index 0)
    tout.assign(max_steps, 0.0);
    VGB_CUDA(cudaMemcpyAsync(Vout.p, X0, n_ext * sizeof(double), cudaMemcpyHostToDevice, s));
    if (I0 && n_vsrc && !fixed)
        VGB_CUDA(cudaMemcpyAsync(Iout.p, I0, n_vsrc * sizeof(double), cudaMemcpyHostToDevice, s));
    // the host copies above read pageable memory that the caller may free
    VGB_CUDA(cudaStreamSynchronize(s));

    o.reltol = reltol;
    o.abstol = abstol;
    o.vntol = vntol;
    o.damping = nr_damping;
    o.max_step = 1e30;
    for (double& d : dt_hist) d = dt;
    min_dt_used = max_dt_used = dt;
    if (fixed) {
        fixed_n = std::min((int)(t_stop / dt), max_steps - 1);
        if (fixed_n < 1) fixed_n = 1;
    }
    launches0 = c->launches;
}

// Run until max_accepted more steps are accepted (0 = to the end of the run).
int TranSession::advance(int max_accepted) {
    if (done) return 0;
    cudaStream_t s = c->stream;
    const int n_nodes = c->n_nodes, n_unk = c->n_unk, n_vsrc = c->n_vsrc;
    const int nx = n_x();
    const int nvo = std::max(n_vsrc, 1);
    const int tb = 256;
    const int grid_x = ceil_div(std::max(nx, 1), tb);
    int accepted_now = 0;
    VGB_CUDA(cudaMemsetAsync(&c->d_status.p->dev_err, 0, sizeof(int), s));
    cudaEvent_t ev0, ev1;
    VGB_CUDA(cudaEventCreate(&ev0));
    VGB_CUDA(cudaEventCreate(&ev1));
    VGB_CUDA(cudaEventRecord(ev0, s));
    const auto limit_hit = [&]() { return max_accepted > 0 && accepted_now >= max_accepted; };

    if (fixed) {
        // constant-step coefficients (full_mna.py:1236-1253)
        const double inv = 1.0 / dt;
        Coeffs k;
        k.c0 = inv; k.c1 = -inv;
        if (method == 1) { k.c0 = 2 * inv; k.c1 = -2 * inv; k.d1 = -1.0; }
        else if (method == 2) { k.c0 = 1.5 * inv; k.c1 = -2.0 * inv; k.c2 = 0.5 * inv; }
        DefaultVecs dv = defaults_for(*c, abstol, s);
        while (fixed_i < fixed_n && !limit_hit()) {
            const int i = fixed_i;
            const double t_next = ((double)i + 1.0) * dt;
            launch_eval_sources(c->vsrc_wave, n_vsrc, t_next, vs.p, s);
            launch_eval_sources(c->isrc_wave, c->n_isrc, t_next, is.p, s);
            VGB_CUDA(cudaMemcpyAsync(Xc.p, X.p, nx * sizeof(double), cudaMemcpyDeviceToDevice, s));
            NRResult r = nr_loop(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, dv.floor_abstol, k, o, tran_itl, s);
            total_nr += r.iterations;
            if (!r.converged) nr_fail_count++;
            launch_status_reset(c->d_status.p, s);
            build_system(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, k, dv.floor_abstol, reltol, vntol,
                         c->d_csr_vals.p, c->d_f.p, c->d_Q.p, c->d_maxc.p, c->d_fres.p, s);
            launch_vsrc_current(c->d_fres.p, c->d_vsrc_p.p, Ivs.p, n_vsrc, s);
            launch_dqdt(c->d_Q.p, Qp.p, dQp.p, Qp2.p, k.c0, k.c1, k.d1, k.c2, dQn.p, n_unk, s);
            const int slot = ((i + 1) % 4);
            commit_kernel<<<grid_x, tb, 0, s>>>(n_nodes, nx, n_unk, n_ext, n_vsrc, 1, 1, 0, Xc.p, X.p,
                                                 c->d_Q.p, Qp.p, dQn.p, dQp.p, Qp2.p, hist.p + (size_t)slot * n_nodes,
                                                 Vmax.p, c->d_maxc.p, hmaxc.p, Ivs.p,
                                                 Vout.p + (size_t)(i + 1) * n_ext, Iout.p + (size_t)(i + 1) * nvo);
            tout[i + 1] = t_next;
            // sources (2), status reset, vsource current, dQ/dt, commit
            c->launches += (n_vsrc ? 1 : 0) + (c->n_isrc ? 1 : 0) + 4;
            fixed_i++;
            accepted_now++;
        }
        step_idx = fixed_i + 1;
        if (fixed_i >= fixed_n) done = true;
    } else {
        const int max_order = 2, max_history = 4;
        while (t < t_stop && step_idx < max_steps && !limit_hit()) {
            const double dt_cur = dt;
            Coeffs k;
            double err_integ;
            const double inv = 1.0 / dt_cur;
            if (method == 0) { k.c0 = inv; k.c1 = -inv; err_integ = -0.5; }
            else if (method == 1) { k.c0 = 2 * inv; k.c1 = -2 * inv; k.d1 = -1.0; err_integ = 1.0 / 24.0; }
            else {
                const double dt_prev = dt_hist[0];
                const double w = dt_prev > 0 ? dt_cur / dt_prev : 1.0;
                const double wp1 = 1.0 + w;
                k.c0 = (1.0 + 2.0 * w) / (wp1 * dt_cur);
                k.c1 = -wp1 / dt_cur;
                k.c2 = (w * w) / (wp1 * dt_cur);
                err_integ = -2.0 / 9.0;
            }
            const double t_next = t + dt_cur;
            launch_eval_sources(c->vsrc_wave, n_vsrc, t_next, vs.p, s);
            launch_eval_sources(c->isrc_wave, c->n_isrc, t_next, is.p, s);
            const bool can_predict = warmup_count >= warmup_steps && history_count >= 2;
            const Pred pr = predictor_coeffs(dt_hist, history_count, dt_cur, max_order);
            const int order = std::max(std::min(history_count - 1, max_order), 0);
            double a0 = pr.a[0], a1 = order >= 1 ? pr.a[1] : 0.0, a2 = order >= 2 ? pr.a[2] : 0.0;
            const double* h0 = hist.p + (size_t)((head + 0) % 4) * n_nodes;
            const double* h1 = hist.p + (size_t)((head + 1) % 4) * n_nodes;
            const double* h2 = hist.p + (size_t)((head + 2) % 4) * n_nodes;
            predict_kernel<<<grid_x, tb, 0, s>>>(n_nodes, nx, n_unk, X.p, Xc.p, Vpred.p, h0, h1, h2, a0, a1, a2,
                                                  can_predict ? 1 : 0, hmaxc.p, reltol, abstol, floor_.p);
            double ramp = gshunt_steps > 0 ? std::min(std::max((double)step_idx / gshunt_steps, 0.0), 1.0) : 1.0;
            k.gshunt = gshunt_init + ramp * (gshunt_target - gshunt_init);
            NRResult r = nr_loop(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, floor_.p, k, o, tran_itl, s);
            total_nr += r.iterations;
            // post-NR rebuild (solver_factories.py:689-713) + LTE
            launch_status_reset(c->d_status.p, s);
            build_system(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, k, floor_.p, reltol, vntol, c->d_csr_vals.p,
                         c->d_f.p, c->d_Q.p, c->d_maxc.p, c->d_fres.p, s);
            launch_vsrc_current(c->d_fres.p, c->d_vsrc_p.p, Ivs.p, n_vsrc, s);
            launch_dqdt(c->d_Q.p, Qp.p, dQp.p, Qp2.p, k.c0, k.c1, k.d1, k.c2, dQn.p, n_unk, s);
            const double kl = err_integ / (err_integ - pr.err);
            lte_kernel<<<ceil_div(n_nodes, tb), tb, 0, s>>>(n_nodes, Xc.p, Vpred.p, Vmax.p, kl, reltol, abstol,
                                                             c->d_status.p);
            VGB_CUDA(cudaMemcpyAsync(c->h_status, c->d_status.p, sizeof(NRStatus), cudaMemcpyDeviceToHost, s));
            VGB_CUDA(cudaStreamSynchronize(s));
            const double lte_norm = bits_to_double(c->h_status->lte_norm);
            const int lte_order = std::min(history_count - 1, max_order);
            double factor = std::pow(lte_ratio / std::max(lte_norm, 1e-10), 1.0 / (lte_order + 1));
            factor = std::min(std::max(factor, 0.1), grow_factor);
            const double dt_lte = dt_cur * factor;

            const bool nr_failed = !r.converged;
            if (nr_failed) nr_fail_count++;
            const bool at_min_dt = dt_cur <= min_dt;
            const bool nr_failed_at_min = nr_failed && at_min_dt;
            const bool lte_reject = (dt_cur / dt_lte > redo_factor) && can_predict && r.converged;
            const bool nr_reject = nr_failed && !at_min_dt;
            const bool force_accept = consecutive >= max_consec;
            const bool reject = (lte_reject || nr_reject) && !force_accept;
            const bool accept = !reject;
            consecutive = accept ? 0 : (lte_reject ? consecutive + 1 : consecutive);
            const double dt_from_lte = can_predict ? dt_lte : dt_cur;
            const double dt_nr_halved = std::max(dt_cur * tran_ft, min_dt);
            const double last_good = history_count > 0 ? dt_hist[0] : min_dt * 16.0;
            const double dt_recovery = std::max(last_good / 8.0, min_dt * 2.0);
            double new_dt = nr_failed ? (at_min_dt ? dt_recovery : dt_nr_halved) : dt_from_lte;
            new_dt = std::min(std::max(new_dt, min_dt), max_dt);
            new_dt = std::min(new_dt, t_stop - t_next);

            const bool use_new = accept && !nr_failed_at_min;
            int new_head = head;
            if (use_new) new_head = (head + 3) % 4;
            commit_kernel<<<grid_x, tb, 0, s>>>(
                n_nodes, nx, n_unk, n_ext, n_vsrc, use_new ? 1 : 0, accept ? 1 : 0, nr_failed_at_min ? 1 : 0,
                Xc.p, X.p, c->d_Q.p, Qp.p, dQn.p, dQp.p, Qp2.p, hist.p + (size_t)new_head * n_nodes, Vmax.p,
                c->d_maxc.p, hmaxc.p, Ivs.p, Vout.p + (size_t)step_idx * n_ext, Iout.p + (size_t)step_idx * nvo);
            // sources, predictor, status reset, vsource current, dQ/dt, LTE, commit
            c->launches += (n_vsrc ? 1 : 0) + (c->n_isrc ? 1 : 0) + 6;
            if (use_new) {
                head = new_head;
                for (int q = 3; q > 0; --q) dt_hist[q] = dt_hist[q - 1];
                dt_hist[0] = dt_cur;
                history_count = std::min(history_count + 1, max_history);
                warmup_count++;
            }
            if (accept) {
                tout[step_idx] = t_next;
                t = t_next;
                step_idx++;
                accepted_now++;
                min_dt_used = std::min(min_dt_used, dt_cur);
                max_dt_used = std::max(max_dt_used, dt_cur);
            }
            if (reject) rejected++;
            dt = new_dt;
        }
        if (!(t < t_stop && step_idx < max_steps)) done = true;
    }
    VGB_CUDA(cudaEventRecord(ev1, s));
    VGB_CUDA(cudaEventSynchronize(ev1));
    float ms = 0.f;
    VGB_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    device_ms += ms;
    return accepted_now;
}

} // namespace vgb

using namespace vgb;

namespace {

template <class F>
int tran_guarded(TranSession* ts, F&& f) {
    if (!ts || !ts->c) return VGB_ERR_INVALID;
    try {
        f();
        return VGB_OK;
    } catch (const Error& e) {
        ts->c->last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        ts->c->last_error = e.what();
        return VGB_ERR_INVALID;
    }
}

void read_outputs(TranSession& ts, double* times, double* V_out, double* I_out) {
    cudaStream_t s = ts.c->stream;
    const int n = ts.step_idx;
    const int nvo = std::max(ts.c->n_vsrc, 1);
    if (V_out)
        VGB_CUDA(cudaMemcpyAsync(V_out, ts.Vout.p, (size_t)n * ts.n_ext * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (I_out) VGB_CUDA(cudaMemcpyAsync(I_out, ts.Iout.p, (size_t)n * nvo * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    if (times) std::memcpy(times, ts.tout.data(), n * sizeof(double));
}

void fill_stats(const TranSession& ts, double* stats) {
    stats[0] = ts.step_idx;
    stats[1] = ts.rejected;
    stats[2] = (double)ts.total_nr;
    stats[3] = ts.min_dt_used;
    stats[4] = ts.max_dt_used;
    stats[5] = ts.device_ms;
    stats[6] = ts.nr_fail_count;
    stats[7] = (double)(ts.c->launches - ts.launches0);
}

} // namespace

extern "C" int vgb_tran_create(void* h, const double* cfg, const double* X0, const double* Q0, const double* I0,
                               const double* maxc0, void** out) {
    Circuit* c = static_cast<Circuit*>(h);
    if (!c || !cfg || !out) return VGB_ERR_INVALID;
    *out = nullptr;
    TranSession* ts = new TranSession();
    ts->c = c;
    const int rc = tran_guarded(ts, [&] {
        if (!c->finalized) throw Error(VGB_ERR_STATE, "circuit is not finalized");
        ts->setup(c, cfg, X0, Q0, I0, maxc0);
    });
    if (rc != VGB_OK) {
        delete ts;
        return rc;
    }
    *out = ts;
    return VGB_OK;
}

extern "C" int vgb_tran_advance(void* tr, int max_accepted, int* accepted, int* done) {
    TranSession* ts = static_cast<TranSession*>(tr);
    return tran_guarded(ts, [&] {
        VGB_REQUIRE(max_accepted >= 0, "max_accepted must be >= 0");
        const int n = ts->advance(max_accepted);
        if (accepted) *accepted = n;
        if (done) *done = ts->done ? 1 : 0;
    });
}

extern "C" int vgb_tran_read(void* tr, double* times, double* V_out, double* I_out, double* stats) {
    TranSession* ts = static_cast<TranSession*>(tr);
    return tran_guarded(ts, [&] {
        read_outputs(*ts, times, V_out, I_out);
        if (stats) fill_stats(*ts, stats);
    });
}

extern "C" int vgb_tran_state(void* tr, double* X, double* Q) {
    TranSession* ts = static_cast<TranSession*>(tr);
    return tran_guarded(ts, [&] {
        cudaStream_t s = ts->c->stream;
        if (X) VGB_CUDA(cudaMemcpyAsync(X, ts->X.p, ts->n_x() * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (Q) VGB_CUDA(cudaMemcpyAsync(Q, ts->Qp.p, ts->c->n_unk * sizeof(double), cudaMemcpyDeviceToHost, s));
        VGB_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int vgb_tran_destroy(void* tr) {
    TranSession* ts = static_cast<TranSession*>(tr);
    if (!ts) return VGB_ERR_INVALID;
    delete ts;
    return VGB_OK;
}

extern "C" int vgb_transient(void* h, const double* cfg, const double* X0, const double* Q0, const double* I0,
                             const double* maxc0, double* times, double* V_out, double* I_out, double* stats) {
    void* tr = nullptr;
    int rc = vgb_tran_create(h, cfg, X0, Q0, I0, maxc0, &tr);
    if (rc != VGB_OK) return rc;
    rc = vgb_tran_advance(tr, 0, nullptr, nullptr);
    if (rc == VGB_OK) rc = vgb_tran_read(tr, times, V_out, I_out, stats);
    vgb_tran_destroy(tr);
    return rc;
}
