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
#include "vgb_stepctl.cuh"

namespace vgb {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

__global__ void dqdt_kernel(const double* Q, const double* Qp, const double* dQp, const double* Qp2,
                            const double* k, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = k[0] * Q[i] + k[1] * Qp[i] + k[2] * dQp[i] + k[3] * Qp2[i];
}

void launch_dqdt(const double* Q, const double* Qp, const double* dQp, const double* Qp2, const double* kdev,
                 double* out, int n, cudaStream_t s) {
    if (n) dqdt_kernel<<<ceil_div(n, 256), 256, 0, s>>>(Q, Qp, dQp, Qp2, kdev, out, n);
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
__device__ __forceinline__ void commit_kernel_body(int n_nodes, int n_x, int n_unk, int n_ext, int n_vsrc, int use_new, int accept,
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

__global__ void commit_kernel(int n_nodes, int n_x, int n_unk, int n_ext, int n_vsrc, int use_new, int accept,
                              int zero_current, const double* Xc, double* X, const double* Q, double* Qp,
                              const double* dQ, double* dQp, double* Qp2, double* hist_slot, double* Vmax,
                              const double* maxc, double* hist_maxc, const double* Ivs, double* Vout_row,
                              double* Iout_row) {
    commit_kernel_body(n_nodes, n_x, n_unk, n_ext, n_vsrc, use_new, accept, zero_current, Xc, X, Q, Qp, dQ, dQp, Qp2,
                       hist_slot, Vmax, maxc, hist_maxc, Ivs, Vout_row, Iout_row);
}

static double bits_to_double(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

// ---------------------------------------------------------------------------
// Device-resident step loop (the transient graph).  The controller state of a
// session lives in device memory; one-thread kernels run ctl_plan, the Newton
// convergence decision and ctl_finish between the batched kernels.  The whole
// loop is one CUDA graph: an outer while-node over steps whose body holds an
// inner while-node over Newton iterations.  Both loops are bounded on the
// device (tran_itl iterations; guard_cap step attempts), whatever the inputs.
// ---------------------------------------------------------------------------

struct TranDev {
    // configuration (field names as in TranSession, for ctl_plan / ctl_finish)
    double t_stop, max_dt, min_dt, lte_ratio, redo_factor, grow_factor, tran_ft, gshunt_init, gshunt_target;
    int gshunt_steps, warmup_steps, max_consec, method, max_steps, tran_itl, fixed, fixed_n;
    // controller state
    double t, dt, dt_hist[4];
    int head, history_count, warmup_count, consecutive, step_idx, fixed_i;
    long long total_nr;
    int rejected, nr_fail_count, done;
    double min_dt_used, max_dt_used;
    // the step in progress
    StepPlan plan;
    StepCommit commit;
    int nr_it, nr_conv;
    // loop control of one run
    int accepted_now, limit, guard, guard_cap, stop_reason;
};

enum { TRAN_STOP_NONE = 0, TRAN_STOP_TIMEOUT = 1, TRAN_STOP_GUARD = 2 };

// Plan of the step (coefficients into k); arms the Newton loop.
__global__ void tran_step_begin_kernel(TranDev* T, double* k, cudaGraphConditionalHandle h_nr) {
    T->plan = ctl_plan(*T);
    for (int q = 0; q < 5; ++q) k[q] = T->plan.k[q];
    T->nr_it = 0;
    T->nr_conv = 0;
    cudaGraphSetConditional(h_nr, 1u);
}

// X_init from the predictor (adaptive): predict_kernel with the plan in device memory
__global__ void tran_predict_kernel(int n_nodes, int n_x, int n_unk, const double* X, double* Xc, double* Vpred,
                                    const double* hist, const TranDev* T, const double* hist_maxc, double reltol,
                                    double abstol, double* floor_) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const StepPlan& p = T->plan;
    if (i < n_nodes) {
        const double vp = p.pa[0] * hist[(size_t)p.slot[0] * n_nodes + i] +
                          p.pa[1] * hist[(size_t)p.slot[1] * n_nodes + i] +
                          p.pa[2] * hist[(size_t)p.slot[2] * n_nodes + i];
        Vpred[i] = vp;
        Xc[i] = p.can_predict ? vp : X[i];
    } else if (i < n_x) {
        Xc[i] = X[i];
    }
    if (i < n_unk) floor_[i] = hist_maxc ? fmax(hist_maxc[i] * reltol, abstol) : abstol;
}

__global__ void tran_copy_kernel(int n, const double* src, double* dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

// Newton convergence decision after one iteration (the host loop's test in nr_loop)
__global__ void tran_nr_decide_kernel(TranDev* T, const NRStatus* S, cudaGraphConditionalHandle h_nr) {
    const int i = T->nr_it;
    bool stop = false;
    if (S->dev_err & DEV_ERR_TIMEOUT) {
        T->stop_reason = TRAN_STOP_TIMEOUT;
        stop = true;
    } else if (S->nonfinite) {
        stop = true;  // the residual left the finite range: not converged
    } else if (S->res_ok && (i == 0 || S->delta_ok)) {
        T->nr_conv = 1;
        stop = true;
    }
    T->nr_it = i + 1;
    if (T->nr_it >= T->tran_itl) stop = true;
    cudaGraphSetConditional(h_nr, stop ? 0u : 1u);
}

// LTE norm: lte_kernel with the coefficient from the plan
__global__ void tran_lte_kernel(int n_nodes, const double* Vnew, const double* Vpred, const double* Vmax,
                                const TranDev* T, double reltol, double abstol, NRStatus* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double k = T->plan.kl;
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

// ctl_finish on the device state, then the loop condition of the step graph.
__global__ void tran_step_end_kernel(TranDev* T, const NRStatus* S, double* tdev, cudaGraphConditionalHandle h_out) {
    const double lte_norm = __longlong_as_double((long long)S->lte_norm);
    T->commit = ctl_finish(*T, T->plan, lte_norm, T->nr_it, T->nr_conv != 0, tdev);
    T->accepted_now += T->commit.accept;
    T->guard++;
    if (!T->done && T->guard >= T->guard_cap) T->stop_reason = TRAN_STOP_GUARD;
    const bool more = !T->done && T->stop_reason == TRAN_STOP_NONE && !(T->limit > 0 && T->accepted_now >= T->limit);
    cudaGraphSetConditional(h_out, more ? 1u : 0u);
}

// Accept / reject commit (full_mna.py:2078-2147) with the controller's decision
__global__ void tran_commit_kernel(int n_nodes, int n_x, int n_unk, int n_ext, int n_vsrc, int nvo, const TranDev* T,
                                   const double* Xc, double* X, const double* Q, double* Qp, const double* dQ,
                                   double* dQp, double* Qp2, double* hist, double* Vmax, const double* maxc,
                                   double* hist_maxc, const double* Ivs, double* Vout, double* Iout) {
    const StepCommit& m = T->commit;
    commit_kernel_body(n_nodes, n_x, n_unk, n_ext, n_vsrc, m.use_new, m.accept, m.zero_current, Xc, X, Q, Qp, dQ,
                       dQp, Qp2, hist + (size_t)m.slot * n_nodes, Vmax, maxc, hist_maxc, Ivs,
                       Vout + (size_t)m.row * n_ext, Iout + (size_t)m.row * nvo);
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
    // the step loop as one CUDA graph (used unless the circuit disables it or profiles phases)
    DevBuf<TranDev> d_td;
    TranDev* h_td = nullptr;  // pinned
    DevBuf<double> tdev;      // accepted step times, written by the device controller
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int graph_epoch = -1;
    bool graph_unavailable = false;  // capture or instantiation failed once: host-driven loop from then on
    long long per_iter_launches = 0, per_step_launches = 0;

    void setup(Circuit* cc, const double* cfg, const double* X0, const double* Q0, const double* I0,
               const double* maxc0);
    int advance(int max_accepted);
    int advance_graph(int max_accepted);
    void build_graph();
    void release_graph();
    int n_x() const { return c->n_nodes + c->n_vsrc; }
    ~TranSession() {
        release_graph();
        if (h_td) cudaFreeHost(h_td);
    }
};

void TranSession::release_graph() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr;
    graph = nullptr;
}

// Capture the step loop: outer while-node (steps) { step begin, sources, initial
// guess, inner while-node (Newton iterations) { nr_iteration, decision },
// post-Newton rebuild, LTE, step end, commit }.
void TranSession::build_graph() {
    release_graph();
    cudaStream_t s = c->stream;
    const int n_nodes = c->n_nodes, n_unk = c->n_unk, n_vsrc = c->n_vsrc;
    const int nx = n_x();
    const int nvo = std::max(n_vsrc, 1);
    const int tb = 256;
    const int grid_x = ceil_div(std::max(nx, 1), tb);
    VGB_CUDA(cudaStreamSynchronize(s));
    mf_prepare_capture(*c);
    const DefaultVecs dv = defaults_for(*c, abstol, s);
    VGB_CUDA(cudaStreamSynchronize(s));
    const double* fl = fixed ? dv.floor_abstol : floor_.p;
    TranDev* T = d_td.p;
    cudaStream_t cs1 = nullptr, cs2 = nullptr;
    VGB_CUDA(cudaStreamCreateWithFlags(&cs1, cudaStreamNonBlocking));
    VGB_CUDA(cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking));
    const long long l0 = c->launches;
    bool cap1 = false, cap2 = false;
    try {
        VGB_CUDA(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle h_out, h_nr;
        VGB_CUDA(cudaGraphConditionalHandleCreate(&h_out, graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams po = {};
        po.type = cudaGraphNodeTypeConditional;
        po.conditional.handle = h_out;
        po.conditional.type = cudaGraphCondTypeWhile;
        po.conditional.size = 1;
        cudaGraphNode_t n_out;
        VGB_CUDA(cudaGraphAddNode(&n_out, graph, nullptr, nullptr, 0, &po));
        cudaGraph_t body = po.conditional.phGraph_out[0];
        VGB_CUDA(cudaGraphConditionalHandleCreate(&h_nr, body, 0, 0));
        // step begin: coefficients, sources at t_next, initial Newton guess
        VGB_CUDA(cudaStreamBeginCaptureToGraph(cs1, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        cap1 = true;
        tran_step_begin_kernel<<<1, 1, 0, cs1>>>(T, c->d_coeffs.p, h_nr);
        launch_eval_sources_dev(c->vsrc_wave, n_vsrc, &T->plan.t_next, vs.p, cs1);
        launch_eval_sources_dev(c->isrc_wave, c->n_isrc, &T->plan.t_next, is.p, cs1);
        if (fixed)
            tran_copy_kernel<<<grid_x, tb, 0, cs1>>>(nx, X.p, Xc.p);
        else
            tran_predict_kernel<<<grid_x, tb, 0, cs1>>>(n_nodes, nx, n_unk, X.p, Xc.p, Vpred.p, hist.p, T, hmaxc.p,
                                                        reltol, abstol, floor_.p);
        c->launches += 2 + (n_vsrc ? 1 : 0) + (c->n_isrc ? 1 : 0);
        // the Newton loop: a while-node nested in the step body
        cudaStreamCaptureStatus cst;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        VGB_CUDA(cudaStreamGetCaptureInfo(cs1, &cst, nullptr, nullptr, &deps, nullptr, &nd));
        cudaGraphNodeParams pn = {};
        pn.type = cudaGraphNodeTypeConditional;
        pn.conditional.handle = h_nr;
        pn.conditional.type = cudaGraphCondTypeWhile;
        pn.conditional.size = 1;
        cudaGraphNode_t n_nr;
        VGB_CUDA(cudaGraphAddNode(&n_nr, body, deps, nullptr, nd, &pn));
        cudaGraph_t nr_body = pn.conditional.phGraph_out[0];
        VGB_CUDA(cudaStreamUpdateCaptureDependencies(cs1, &n_nr, nullptr, 1, cudaStreamSetCaptureDependencies));
        // post-Newton rebuild (solver_factories.py:689-713), LTE, step control, commit
        launch_status_reset(c->d_status.p, cs1);
        build_system(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, fl, reltol, vntol, c->d_csr_vals.p, c->d_f.p,
                     c->d_Q.p, c->d_maxc.p, c->d_fres.p, cs1);
        launch_vsrc_current(c->d_fres.p, c->d_vsrc_p.p, Ivs.p, n_vsrc, cs1);
        launch_dqdt(c->d_Q.p, Qp.p, dQp.p, Qp2.p, c->d_coeffs.p, dQn.p, n_unk, cs1);
        if (!fixed)
            tran_lte_kernel<<<ceil_div(n_nodes, tb), tb, 0, cs1>>>(n_nodes, Xc.p, Vpred.p, Vmax.p, T, reltol, abstol,
                                                                  c->d_status.p);
        tran_step_end_kernel<<<1, 1, 0, cs1>>>(T, c->d_status.p, tdev.p, h_out);
        tran_commit_kernel<<<grid_x, tb, 0, cs1>>>(n_nodes, nx, n_unk, n_ext, n_vsrc, nvo, T, Xc.p, X.p, c->d_Q.p,
                                                   Qp.p, dQn.p, dQp.p, Qp2.p, hist.p, Vmax.p, c->d_maxc.p, hmaxc.p,
                                                   Ivs.p, Vout.p, Iout.p);
        c->launches += 1 + (n_vsrc ? 1 : 0) + (n_unk ? 1 : 0) + (fixed ? 0 : 1) + 2;
        VGB_CUDA(cudaGetLastError());
        cap1 = false;
        VGB_CUDA(cudaStreamEndCapture(cs1, &body));
        per_step_launches = c->launches - l0;
        // one Newton iteration and its convergence decision
        const long long l1 = c->launches;
        VGB_CUDA(cudaStreamBeginCaptureToGraph(cs2, nr_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        cap2 = true;
        nr_iteration(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, fl, o, cs2, false);
        tran_nr_decide_kernel<<<1, 1, 0, cs2>>>(T, c->d_status.p, h_nr);
        VGB_CUDA(cudaGetLastError());
        cap2 = false;
        VGB_CUDA(cudaStreamEndCapture(cs2, &nr_body));
        per_iter_launches = c->launches - l1 + 1;
        VGB_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
    } catch (...) {
        cudaGraph_t g = nullptr;
        if (cap1) cudaStreamEndCapture(cs1, &g);
        if (cap2) cudaStreamEndCapture(cs2, &g);
        cudaStreamDestroy(cs1);
        cudaStreamDestroy(cs2);
        c->launches = l0;
        release_graph();
        throw;
    }
    cudaStreamDestroy(cs1);
    cudaStreamDestroy(cs2);
    c->launches = l0;  // captures launch nothing; advance_graph counts the replays
    graph_epoch = c->config_epoch;
}

// One run of the step graph: the host controller state goes down, the graph
// runs until `max_accepted` more steps are accepted (0: to the end), the state
// comes back.  One synchronisation per call, none per step or Newton iteration.
int TranSession::advance_graph(int max_accepted) {
    cudaStream_t s = c->stream;
    if (!gexec || graph_epoch != c->config_epoch) build_graph();
    TranDev& h = *h_td;
    h = TranDev{};
    h.t_stop = t_stop; h.max_dt = max_dt; h.min_dt = min_dt; h.lte_ratio = lte_ratio; h.redo_factor = redo_factor;
    h.grow_factor = grow_factor; h.tran_ft = tran_ft; h.gshunt_init = gshunt_init; h.gshunt_target = gshunt_target;
    h.gshunt_steps = gshunt_steps; h.warmup_steps = warmup_steps; h.max_consec = max_consec; h.method = method;
    h.max_steps = max_steps; h.tran_itl = tran_itl; h.fixed = fixed ? 1 : 0; h.fixed_n = fixed_n;
    h.t = t; h.dt = dt;
    for (int q = 0; q < 4; ++q) h.dt_hist[q] = dt_hist[q];
    h.head = head; h.history_count = history_count; h.warmup_count = warmup_count; h.consecutive = consecutive;
    h.step_idx = step_idx; h.fixed_i = fixed_i;
    h.total_nr = total_nr; h.rejected = rejected; h.nr_fail_count = nr_fail_count;
    h.min_dt_used = min_dt_used; h.max_dt_used = max_dt_used;
    h.limit = max_accepted;
    h.guard_cap = 16 * max_steps + 1000;  // step attempts of one run, a bound the controller never reaches
    VGB_CUDA(cudaMemcpyAsync(d_td.p, h_td, sizeof(TranDev), cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemsetAsync(&c->d_status.p->dev_err, 0, sizeof(int), s));
    const int step0 = step_idx;
    cudaEvent_t ev0, ev1;
    VGB_CUDA(cudaEventCreate(&ev0));
    VGB_CUDA(cudaEventCreate(&ev1));
    VGB_CUDA(cudaEventRecord(ev0, s));
    VGB_CUDA(cudaGraphLaunch(gexec, s));
    VGB_CUDA(cudaEventRecord(ev1, s));
    VGB_CUDA(cudaMemcpyAsync(h_td, d_td.p, sizeof(TranDev), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    VGB_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    device_ms += ms;
    const TranDev& d = *h_td;
    c->launches += 1 + (d.total_nr - total_nr) * per_iter_launches + (long long)d.guard * per_step_launches;
    if (d.step_idx > step0)
        VGB_CUDA(cudaMemcpy(tout.data() + step0, tdev.p + step0, (size_t)(d.step_idx - step0) * sizeof(double),
                            cudaMemcpyDeviceToHost));
    t = d.t; dt = d.dt;
    for (int q = 0; q < 4; ++q) dt_hist[q] = d.dt_hist[q];
    head = d.head; history_count = d.history_count; warmup_count = d.warmup_count; consecutive = d.consecutive;
    step_idx = d.step_idx; fixed_i = d.fixed_i;
    total_nr = d.total_nr; rejected = d.rejected; nr_fail_count = d.nr_fail_count;
    min_dt_used = d.min_dt_used; max_dt_used = d.max_dt_used;
    done = d.done != 0;
    if (d.stop_reason == TRAN_STOP_TIMEOUT) throw Error(VGB_ERR_TIMEOUT, "sparse LU dependency wait timed out");
    if (d.stop_reason == TRAN_STOP_GUARD)
        throw Error(VGB_ERR_STATE, "transient step loop reached its bound on step attempts");
    return d.accepted_now;
}

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
    // an adaptive run with nothing to do (t_stop = 0 or max_steps = 1) is done at once
    done = !fixed && !(t < t_stop && step_idx < max_steps);
    // device controller state of the step graph
    d_td.alloc(1);
    VGB_CUDA(cudaMallocHost((void**)&h_td, sizeof(TranDev)));
    tdev.alloc(max_steps);
    tdev.zero(s);
    VGB_CUDA(cudaStreamSynchronize(s));
    launches0 = c->launches;
}

// Run until max_accepted more steps are accepted (0 = to the end of the run).
int TranSession::advance(int max_accepted) {
    if (done) return 0;
    if (c->tran_graph && !c->profile && !graph_unavailable) {
        try {
            return advance_graph(max_accepted);
        } catch (const Error&) {
            // a failure while building the graph (no executable graph yet) leaves the device
            // untouched: run the same kernels from the host loop instead; a failure during a
            // run of the graph is the run's error
            if (gexec) throw;
            graph_unavailable = true;
            (void)cudaGetLastError();  // clear the (non-sticky) error of the failed graph call
            c->last_error.clear();
        }
    }
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

    // the host-driven loop: the same controller (ctl_plan / ctl_finish) on the host,
    // one status read back per Newton iteration and one LTE read back per step
    const DefaultVecs dv = defaults_for(*c, abstol, s);
    while (!done && !limit_hit()) {
        const StepPlan p = ctl_plan(*this);
        Coeffs k;
        k.c0 = p.k[0];
        k.c1 = p.k[1];
        k.d1 = p.k[2];
        k.c2 = p.k[3];
        k.gshunt = p.k[4];
        launch_eval_sources(c->vsrc_wave, n_vsrc, p.t_next, vs.p, s);
        launch_eval_sources(c->isrc_wave, c->n_isrc, p.t_next, is.p, s);
        const double* fl = fixed ? dv.floor_abstol : floor_.p;
        if (fixed) {
            VGB_CUDA(cudaMemcpyAsync(Xc.p, X.p, nx * sizeof(double), cudaMemcpyDeviceToDevice, s));
        } else {
            const double* h0 = hist.p + (size_t)p.slot[0] * n_nodes;
            const double* h1 = hist.p + (size_t)p.slot[1] * n_nodes;
            const double* h2 = hist.p + (size_t)p.slot[2] * n_nodes;
            predict_kernel<<<grid_x, tb, 0, s>>>(n_nodes, nx, n_unk, X.p, Xc.p, Vpred.p, h0, h1, h2, p.pa[0],
                                                  p.pa[1], p.pa[2], p.can_predict, hmaxc.p, reltol, abstol, floor_.p);
            c->launches += 1;
        }
        NRResult r = nr_loop(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, fl, k, o, tran_itl, s);
        // post-NR rebuild (solver_factories.py:689-713), LTE
        launch_status_reset(c->d_status.p, s);
        build_system(*c, Xc.p, vs.p, is.p, Qp.p, dQp.p, Qp2.p, fl, reltol, vntol, c->d_csr_vals.p, c->d_f.p,
                     c->d_Q.p, c->d_maxc.p, c->d_fres.p, s);
        launch_vsrc_current(c->d_fres.p, c->d_vsrc_p.p, Ivs.p, n_vsrc, s);
        launch_dqdt(c->d_Q.p, Qp.p, dQp.p, Qp2.p, c->d_coeffs.p, dQn.p, n_unk, s);
        double lte_norm = 0.0;
        if (!fixed) {
            lte_kernel<<<ceil_div(n_nodes, tb), tb, 0, s>>>(n_nodes, Xc.p, Vpred.p, Vmax.p, p.kl, reltol, abstol,
                                                             c->d_status.p);
            VGB_CUDA(cudaMemcpyAsync(c->h_status, c->d_status.p, sizeof(NRStatus), cudaMemcpyDeviceToHost, s));
            VGB_CUDA(cudaStreamSynchronize(s));
            lte_norm = bits_to_double(c->h_status->lte_norm);
            c->launches += 1;
        }
        const StepCommit m = ctl_finish(*this, p, lte_norm, r.iterations, r.converged, tout.data());
        commit_kernel<<<grid_x, tb, 0, s>>>(
            n_nodes, nx, n_unk, n_ext, n_vsrc, m.use_new, m.accept, m.zero_current, Xc.p, X.p, c->d_Q.p, Qp.p,
            dQn.p, dQp.p, Qp2.p, hist.p + (size_t)m.slot * n_nodes, Vmax.p, c->d_maxc.p, hmaxc.p, Ivs.p,
            Vout.p + (size_t)m.row * n_ext, Iout.p + (size_t)m.row * nvo);
        // sources, status reset, vsource current, dQ/dt, commit
        c->launches += (n_vsrc ? 1 : 0) + (c->n_isrc ? 1 : 0) + 4;
        accepted_now += m.accept;
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
