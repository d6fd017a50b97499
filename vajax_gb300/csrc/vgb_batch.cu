// Batched transient of many replicas of one small circuit: Monte-Carlo and
// process/temperature corners, or served jobs that share a sparsity pattern.
//
// The reference runs corners one after another (vajax/analysis/engine.py:
// 2274-2320), each through its own transient loop (full_mna.py:1198-1441
// fixed step, :1792-2196 adaptive).  Here every replica runs its own loop
// with its own Newton iterations, time step, rejections and outputs, as it
// would alone, but all replicas advance together in one persistent kernel:
//
//  * one cooperative launch, at most one CTA per SM, loops over "ticks";
//  * a tick is one device evaluation of every replica that needs one
//    (evaluation items spread evenly over the whole grid, lanes running the
//    same device of 32 consecutive replicas, so a warp mostly follows one
//    branch path and no SM holds more evaluation warps than it must), a grid
//    barrier, then one warp per replica that assembles its dense Jacobian
//    and residual in shared memory, factorises (LU with partial pivoting)
//    and solves, applies the Newton update and decides, or, after
//    convergence, finishes the step (charges, branch currents, LTE,
//    accept/reject, next dt, commit, outputs) and plans the next one, then a
//    second grid barrier;
//  * per-replica masks: a replica that converged, was rejected or is done
//    takes no further work from the others' iterations;
//  * values are batch-interleaved ([k][replica]) where the evaluation reads
//    and writes them, replica-contiguous where one warp owns them;
//  * the model outputs keep the resistive and reactive Jacobians apart, so an
//    evaluation at the point where the next Newton iteration starts (every
//    fixed step; adaptive steps without a prediction) serves both: the
//    post-convergence rebuild of one step and the first iteration of the next
//    share one evaluation, which leaves every result unchanged.
//
// Every loop is bounded: ticks by a cap derived from max_steps and tran_itl,
// barriers by a poll limit that sets an error flag and stops the kernel.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "vgb_core.h"
#include "vgb_math.cuh"
#include "vgb_models_gen.cuh"
#include "vgb_sources.cuh"
#include "vgb_stepctl.cuh"

namespace vgb {

constexpr int BATCH_MAX_N = 48;       // n_aug limit: each warp's dense system lives in shared memory
constexpr int BATCH_THREADS = 256;
constexpr int BATCH_MAX_GROUPS = 16;
constexpr unsigned BARRIER_POLLS = 1u << 26;
constexpr int COOP_WARPS = 8;  // warps that share one cooperative evaluation: the whole CTA, two per SM sub-partition

// Replica states between ticks: INIT (uic start: charges from the evaluation
// at X0), START (given initial state: step 1 from X0), NR (a Newton
// iteration at Xc), POST (Newton ended: finish the step at Xc), DONE.
enum : int { RS_INIT = 0, RS_START = 1, RS_NR = 2, RS_POST = 3, RS_DONE = 4 };

struct BGroup {
    int model, n_dev, nn, nj, np;
    const int* node_map;     // [nn][n_dev] circuit node of each model node
    const double* shared;    // [np]
    const int* vidx;         // [np] -1 shared, else column of `varying`
    const double* varying;   // [n_var][n_dev][n_rep]
    const double* temps;     // [n_dev][n_rep] or null
    double temp_shared;
    long long cbase;         // first contribution slot of the group
    long long item0;         // first evaluation item of the group
    long long cu0, cu1;      // its cooperative units [cu0, cu1) (empty: one warp per item warp)
    double* cache;           // cooperative groups: [NCACHE][n_dev][n_rep] parameter-only values
};

// Per-replica controller state (field names as ctl_plan / ctl_finish expect).
struct BRep {
    double t_stop, max_dt, min_dt, lte_ratio, redo_factor, grow_factor, tran_ft, gshunt_init, gshunt_target;
    int gshunt_steps, warmup_steps, max_consec, method, max_steps, tran_itl, fixed, fixed_n;
    double t, dt, dt_hist[4];
    int head, history_count, warmup_count, consecutive, step_idx, fixed_i;
    long long total_nr;
    int rejected, nr_fail_count, done;
    double min_dt_used, max_dt_used;
    StepPlan plan;
    int state, nr_it, nr_conv, need_eval;
    int pivot_err;
    double k[5];  // Newton coefficients of the step in progress
};

struct BatchArgs {
    int n_rep, n_nodes, n_unk, n_vsrc, n_isrc, n_aug, n_x, n_ext, nvo, nnz;
    int n_groups;
    long long n_items, n_contrib;
    long long n_coop_units;  // item warps evaluated by a group of COOP_WARPS warps
    long long coop_stride;   // doubles of shared memory per group (exchange slots x 32 lanes)
    // assembly gather lists staged in shared memory at the start of the kernel
    // (when they fit): counts and the byte offset of the staged area
    int n_csr_src, n_res_src, stage;
    long long stage_off;
    // doubles of gather scratch in each warp's workspace (0: gather from global)
    int ws_sc;
    double gmin, reltol, abstol, vntol, damping;
    const BGroup* groups;
    // pattern and gather lists (one replica)
    const int* csr_row; const int* indices;
    const int* csr_ptr; const int* csr_jr; const int* csr_jq;
    const double* csr_const; const unsigned char* csr_diag;
    const int* res_ptr; const int* res_rr; const int* res_rq;
    const int* nb_ptr; const int* nb_idx; const int* ni_ptr; const int* ni_idx;
    const int* vsrc_p; const int* vsrc_n;
    const unsigned char* conv_mask;
    // sources (template kinds/offsets/counts, per-replica data [n_rep][len])
    const int* vs_kind; const int* vs_off; const int* vs_cnt; const double* vs_data; int vs_len;
    const int* is_kind; const int* is_off; const int* is_cnt; const double* is_data; int is_len;
    // state
    double* X;        // [n_x][n_rep]   committed solution
    double* Xc;       // [n_x][n_rep]   Newton iterate (evaluation point)
    double* contrib;  // [n_contrib][n_rep]
    double* Qp; double* Qp2; double* dQp; double* hmaxc; double* floor_;   // [n_rep][n_unk]
    double* Vpred; double* Vmax; double* hist;                               // [n_rep][n_nodes], [n_rep][4][n_nodes]
    double* vs; double* is;                                                 // [n_rep][n_vsrc], [n_rep][n_isrc]
    BRep* rep;
    // outputs
    double* tout; double* Vout; double* Iout;  // [n_rep][max_steps], [n_rep][max_steps][n_ext], [..][nvo]
    int max_steps;
    // control
    unsigned* bar_count; unsigned* bar_gen; int* active; int* err;
    long long max_ticks;
    long long* ticks_out;
    // SM clock cycles summed over ticks: [0..3] each phase of a tick as CTA 0's
    // thread 0 sees it (evaluation, wait at the first barrier, per-replica
    // step, wait at the second barrier); [4..7] replica 0's assembly, LU and
    // solve, Newton update and test, step finish and plan; [8..11] inside
    // those: the assembly's Jacobian and its residual rows, the LU's
    // factorisation and its substitutions
    long long* phase_cycles;
};

// ---------------------------------------------------------------------------
// grid barrier (the launch is cooperative: every CTA is resident)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void grid_barrier(const BatchArgs& a) {
    __syncthreads();
    if (gridDim.x == 1) return;  // one CTA: the block barrier is the grid barrier
    if (threadIdx.x == 0) {
        volatile unsigned* gen = a.bar_gen;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(a.bar_count, 1u) == gridDim.x - 1) {
            *a.bar_count = 0;
            __threadfence();
            atomicAdd(a.bar_gen, 1u);
        } else {
            unsigned it = 0;
            while (*gen == g) {
                if (++it > BARRIER_POLLS) {
                    atomicOr(a.err, DEV_ERR_TIMEOUT);
                    break;
                }
                if (it > 32) __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// evaluation of one item (group g, device d, replica r)
// ---------------------------------------------------------------------------

struct BParam {
    const BGroup g;
    int d, r, n_rep;
    __device__ __forceinline__ double operator()(int k) const {
        const int v = __ldg(g.vidx + k);
        return v < 0 ? __ldg(g.shared + k) : __ldg(g.varying + ((size_t)v * g.n_dev + d) * n_rep + r);
    }
};

// The per-instance cache of a cooperative model: the values of its body that
// depend on parameters and temperature only, computed once per run
// (batch_cache_kernel) and read by every evaluation.
struct CacheW {
    double* c;
    size_t sd, o;
    __device__ __forceinline__ void operator()(int k, double v) const { c[(size_t)k * sd + o] = v; }
};
struct CacheR {
    const double* c;
    size_t sd, o;
    __device__ __forceinline__ double operator()(int k) const { return __ldg(c + (size_t)k * sd + o); }
    __device__ __forceinline__ bool b(int k) const {
        return __double_as_longlong(__ldg(c + (size_t)k * sd + o)) != 0;
    }
};

// Models with a generated cache program (HasCache) read their parameter-only
// values from the per-instance cache in the one-warp path too.

template <class M>
__device__ __noinline__ void eval_item(const BatchArgs& a, const BGroup& g, int d, int r) {
    double V[M::NN];
#pragma unroll
    for (int t = 0; t < M::NN; ++t)
        V[t] = __ldcg(a.Xc + (size_t)__ldg(g.node_map + (size_t)t * g.n_dev + d) * a.n_rep + r);
    const double T = g.temps ? __ldg(g.temps + (size_t)d * a.n_rep + r) : g.temp_shared;
    double rr[M::NN], rq[M::NN], jr[M::NJ > 0 ? M::NJ : 1], jq[M::NJ > 0 ? M::NJ : 1];
    BParam P{g, d, r, a.n_rep};
    if constexpr (HasCache<M>::value) {
        const CacheR C{g.cache, (size_t)g.n_dev * a.n_rep, (size_t)d * a.n_rep + r};
        M::eval_cached(P, C, T, V, rr, rq, jr, jq);
    } else {
        M::eval(P, T, V, rr, rq, jr, jq);
    }
    // layout of a group: [2 NJ + 2 NN][n_dev]: jr, jq, rr, rq
    double* base = a.contrib + (size_t)g.cbase * a.n_rep;
    const size_t sd = (size_t)g.n_dev * a.n_rep;
    const size_t o = (size_t)d * a.n_rep + r;
#pragma unroll
    for (int k = 0; k < M::NJ; ++k) {
        __stcg(base + k * sd + o, jr[k]);
        __stcg(base + (M::NJ + k) * sd + o, jq[k]);
    }
#pragma unroll
    for (int q = 0; q < M::NN; ++q) {
        __stcg(base + (2 * M::NJ + q) * sd + o, rr[q]);
        __stcg(base + (2 * M::NJ + M::NN + q) * sd + o, rq[q]);
    }
}

// Output sink of a cooperative evaluation: output i of the [jr | jq | rr | rq]
// layout of instance (d, r).
struct CoopOut {
    double* base;
    size_t sd, o;
    __device__ __forceinline__ void operator()(int i, double v) const { __stcg(base + (size_t)i * sd + o, v); }
};

// One thread per instance (d, r) of a cooperative group: the cache program.
template <class M>
__global__ void __launch_bounds__(128) batch_cache_kernel(BGroup g, int n_rep) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)g.n_dev * n_rep) return;
    const int d = (int)(i / n_rep), r = (int)(i - (long long)d * n_rep);
    const double T = g.temps ? __ldg(g.temps + (size_t)d * n_rep + r) : g.temp_shared;
    BParam P{g, d, r, n_rep};
    M::cache(P, T, CacheW{g.cache, (size_t)g.n_dev * n_rep, (size_t)d * n_rep + r});
}

// One item warp evaluated by the COOP_WARPS warps of a group (this warp is
// part w).  Lanes without an instance (padding, or a replica that needs no
// evaluation) run the straight-line body on instance (0, 0) and store
// nothing, so that every warp of the group passes every barrier.
template <class M>
__device__ __noinline__ void eval_coop_item(const BatchArgs& a, const BGroup& g, int d, int r, bool act, int w,
                                            vgb_xs_t xs, int bar) {
    // every warp of the group runs one part, and every part passes the group's barriers
    static_assert(M::COOP_W == COOP_WARPS, "the model's cooperative body is split for another group size");
    double V[M::NN];
#pragma unroll
    for (int t = 0; t < M::NN; ++t)
        V[t] = __ldcg(a.Xc + (size_t)__ldg(g.node_map + (size_t)t * g.n_dev + d) * a.n_rep + r);
    const double T = g.temps ? __ldg(g.temps + (size_t)d * a.n_rep + r) : g.temp_shared;
    BParam P{g, d, r, a.n_rep};
    const CacheR C{g.cache, (size_t)g.n_dev * a.n_rep, (size_t)d * a.n_rep + r};
    const CoopOut out{a.contrib + (size_t)g.cbase * a.n_rep, (size_t)g.n_dev * a.n_rep, (size_t)d * a.n_rep + r};
    M::coop(w, P, C, T, V, xs, act, out, bar);
}

// Item warps (32 consecutive items: one device of 32 consecutive replicas)
// are dealt round-robin over the CTAs, so every SM holds as few evaluation
// warps as the batch allows.  Item warps of a model with a cooperative body
// go to groups of COOP_WARPS warps (the whole CTA, two warps per SM
// sub-partition), dealt round-robin over the CTAs; the rest to single warps.
__device__ void eval_phase(const BatchArgs& a) {
    const int lane = threadIdx.x & 31;
    if (a.n_coop_units) {
        extern __shared__ double batch_smem[];
        const int warp = threadIdx.x >> 5;
        const int grp = warp / COOP_WARPS, w = warp % COOP_WARPS;
        const int ngrp = (blockDim.x >> 5) / COOP_WARPS;
        const vgb_xs_t xs = vgb_xs_base(batch_smem + (size_t)grp * a.coop_stride + lane);
        for (long long u = blockIdx.x + (long long)gridDim.x * grp; u < a.n_coop_units;
             u += (long long)gridDim.x * ngrp) {
            int gi = 0;
            while (gi + 1 < a.n_groups && !(u >= a.groups[gi].cu0 && u < a.groups[gi].cu1)) ++gi;
            const BGroup g = a.groups[gi];
            const long long loc = (u - g.cu0) * 32 + lane;
            int d = (int)(loc / a.n_rep);
            int r = (int)(loc - (long long)d * a.n_rep);
            bool act = d < g.n_dev;
            if (act) act = *(volatile int*)&a.rep[r].need_eval != 0;
            if (!act) d = r = 0;
            // the same decision in every warp of the group (each lane's flag is)
            if (!__any_sync(0xffffffffu, act)) continue;
            switch (g.model) {
#define VGB_COOP_CASE(ID, STRUCT) \
    case ID: eval_coop_item<STRUCT>(a, g, d, r, act, w, xs, 1 + grp); break;
                VGB_COOP_LIST(VGB_COOP_CASE)
#undef VGB_COOP_CASE
                default: break;
            }
        }
    }
    const long long n_iw = (a.n_items + 31) / 32;
    const long long step = (long long)gridDim.x * (blockDim.x >> 5);
    // one-warp items start at the CTA's last warps, which hold no cooperative group
    // when the batch has fewer cooperative units than groups: they run beside it
    const int wr = (int)(blockDim.x >> 5) - 1 - (int)(threadIdx.x >> 5);
    for (long long iw = (long long)wr * gridDim.x + blockIdx.x; iw < n_iw; iw += step) {
        const long long it = iw * 32 + lane;
        if (it >= a.n_items) continue;
        int gi = 0;
        while (gi + 1 < a.n_groups && it >= a.groups[gi + 1].item0) ++gi;
        const BGroup g = a.groups[gi];
        if (g.cu1 > g.cu0) continue;  // evaluated cooperatively
        const long long loc = it - g.item0;
        const int d = (int)(loc / a.n_rep);
        const int r = (int)(loc - (long long)d * a.n_rep);
        if (d >= g.n_dev) continue;  // padding to a warp boundary
        if (!*(volatile int*)&a.rep[r].need_eval) continue;
        switch (g.model) {
#define VGB_BATCH_CASE(ID, STRUCT) \
    case ID: eval_item<STRUCT>(a, g, d, r); break;
            VGB_MODEL_LIST(VGB_BATCH_CASE)
#undef VGB_BATCH_CASE
            default: break;
        }
    }
}

// ---------------------------------------------------------------------------
// per-replica work, one warp
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Per-warp workspace in shared memory: the dense Newton matrix (column
// major), the residual / right-hand side / update, and the charges, largest
// contributions and resistive residuals of the node rows.
struct WarpWS {
    double* M; double* f; double* Q; double* maxc; double* fres;
    BRep* rep;  // the replica's controller state for the tick (read once, written back at its end)
    double* sc; // the assembly's gathered contributions (ws_scratch doubles), or null
};

constexpr size_t BREP_DOUBLES = (sizeof(BRep) + 7) / 8;
constexpr int WS_SCRATCH_MAX = 1024;  // doubles of gather scratch per warp, at most

// Gather scratch per warp: every Jacobian contribution, or every resistive and
// reactive residual contribution, of one replica; 0 (no scratch) when larger
// than WS_SCRATCH_MAX.
__host__ __device__ inline int ws_scratch(int n_csr_src, int n_res_src) {
    const int need = n_csr_src > 2 * n_res_src ? n_csr_src : 2 * n_res_src;
    return need <= WS_SCRATCH_MAX ? need : 0;
}

__host__ __device__ inline size_t ws_doubles(int n_aug, int n_unk, int scratch) {
    return (size_t)n_aug * n_aug + n_aug + 3 * (size_t)(n_unk > 0 ? n_unk : 1) + BREP_DOUBLES + scratch;
}

__device__ __forceinline__ WarpWS warp_ws(const BatchArgs& a) {
    extern __shared__ double batch_smem[];
    const size_t n = a.n_aug, nu = a.n_unk > 0 ? a.n_unk : 1;
    const int sc = a.ws_sc;
    double* base = batch_smem + (threadIdx.x >> 5) * ws_doubles(a.n_aug, a.n_unk, sc);
    double* rep = base + n * n + n + 3 * nu;
    return WarpWS{base, base + n * n, base + n * n + n, base + n * n + n + nu, base + n * n + n + 2 * nu,
                  reinterpret_cast<BRep*>(rep), sc ? rep + BREP_DOUBLES : nullptr};
}

// Warp-cooperative copy of a controller state (32-bit words).
__device__ __forceinline__ void copy_brep(BRep* dst, const BRep* src, int lane) {
    static_assert(sizeof(BRep) % 4 == 0, "BRep is copied as 32-bit words");
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    for (int i = lane; i < (int)(sizeof(BRep) / 4); i += 32) d[i] = s[i];
}

// Source waveforms of replica r at time t (lanes over sources).
__device__ void replica_sources(const BatchArgs& a, int r, double t, int lane) {
    for (int k = lane; k < a.n_vsrc; k += 32)
        a.vs[(size_t)r * a.n_vsrc + k] = eval_source(a.vs_kind[k], a.vs_data + (size_t)r * a.vs_len + a.vs_off[k],
                                                     a.vs_cnt[k], t);
    for (int k = lane; k < a.n_isrc; k += 32)
        a.is[(size_t)r * a.n_isrc + k] = eval_source(a.is_kind[k], a.is_data + (size_t)r * a.is_len + a.is_off[k],
                                                     a.is_cnt[k], t);
}

// NaN -> 0 and the running max of |v| on the bit patterns: integer work, not
// the FP64 pipe, which one warp reaches only once per 64 cycles.  Same values
// as nan0(x) and fmax(m, fabs(v)) for m >= 0 and v not NaN.
__device__ __forceinline__ double nan0_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? 0.0 : x;
}
__device__ __forceinline__ double max_abs_bits(double m, double v) {
    const unsigned long long bm = (unsigned long long)__double_as_longlong(m);
    const unsigned long long bv = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return __longlong_as_double((long long)(bv > bm ? bv : bm));
}

// Contribution of gather entry idx of replica r.  Another SM may have
// written it in this tick: read it from L2, unless the grid is one CTA.
__device__ __forceinline__ double cval(const BatchArgs& a, int idx, int r) {
    const double* p = a.contrib + (size_t)idx * a.n_rep + r;
    return gridDim.x == 1 ? *p : __ldcg(p);
}

// Assembly at Xc with coefficients k (mna_builder.py:759-1076, the same sums
// in the same order as assemble_kernel): dense column-major M (if jac), f,
// Q, maxc, fres in the warp's workspace; returns res_ok (residual test) and
// sets *nonfinite.
__device__ __noinline__ bool replica_assemble(const BatchArgs& a, const WarpWS& w, int r, const double* k,
                                              const double* floor_, bool jac, bool* nonfinite, int lane) {
    const int n = a.n_aug;
    const double* Xr = a.Xc;  // [n_x][n_rep]
    const double c0 = k[0], c1 = k[1], d1 = k[2], c2 = k[3], gshunt = k[4];
    const bool prof = r == 0 && lane == 0;
    const long long t0 = prof ? clock64() : 0;
    if (jac) {
        for (int t = lane; t < n * n; t += 32) w.M[t] = 0.0;
        if (w.sc) {
            // every contribution's jr + c0 jq over the lanes (eight loads of each lane in flight
            // at once), then each entry's sum in its own order from shared memory: a supply
            // rail's entry no longer waits on its chain of loads
            const int ncs = a.n_csr_src;
            for (int t0 = lane; t0 < ncs; t0 += 256) {
                double jr[8], jq[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (t0 + 32 * u < ncs) {
                        jr[u] = cval(a, a.csr_jr[t0 + 32 * u], r);
                        jq[u] = cval(a, a.csr_jq[t0 + 32 * u], r);
                    }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (t0 + 32 * u < ncs) w.sc[t0 + 32 * u] = nan0_bits(jr[u] + c0 * jq[u]);
            }
        }
        __syncwarp();
        for (int e = lane; e < a.nnz; e += 32) {
            double s = 0.0;
            const int q1 = a.csr_ptr[e + 1];
            if (w.sc) {
                for (int q = a.csr_ptr[e]; q < q1; ++q) s += w.sc[q];
            } else {
                for (int q = a.csr_ptr[e]; q < q1; q += 8) {  // every load of a chunk in flight at once
                    double jr[8], jq[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                        if (q + t < q1) {
                            jr[t] = cval(a, a.csr_jr[q + t], r);
                            jq[t] = cval(a, a.csr_jq[q + t], r);
                        }
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                        if (q + t < q1) s += nan0_bits(jr[t] + c0 * jq[t]);
                }
            }
            if (a.csr_diag[e]) s += a.gmin + gshunt;
            s += a.csr_const[e];
            w.M[a.csr_row[e] + (size_t)a.indices[e] * n] = s;
        }
        __syncwarp();
    }
    const long long t1 = prof ? clock64() : 0;
    bool ok = true, nf = false;
    const int nrs = a.n_res_src;
    if (w.sc) {  // the residual contributions over the lanes, as for the Jacobian
        __syncwarp();
        for (int t0 = lane; t0 < nrs; t0 += 256) {
            double rv[8], qv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (t0 + 32 * u < nrs) {
                    rv[u] = cval(a, a.res_rr[t0 + 32 * u], r);
                    qv[u] = cval(a, a.res_rq[t0 + 32 * u], r);
                }
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (t0 + 32 * u < nrs) {
                    w.sc[t0 + 32 * u] = nan0_bits(rv[u]);
                    w.sc[nrs + t0 + 32 * u] = nan0_bits(qv[u]);
                }
        }
        __syncwarp();
    }
    for (int row = lane; row < n; row += 32) {
        double fn, tol;
        if (row < a.n_unk) {
            double fr = 0.0, q = 0.0, mc = 0.0;
            const int e1 = a.res_ptr[row + 1];
            if (w.sc) {
                for (int e = a.res_ptr[row]; e < e1; ++e) {
                    const double v = w.sc[e];
                    fr += v;
                    mc = max_abs_bits(mc, v);
                    q += w.sc[nrs + e];
                }
            } else {
                for (int e = a.res_ptr[row]; e < e1; e += 8) {  // every load of a chunk in flight at once
                    double rv[8], qv[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                        if (e + t < e1) {
                            rv[t] = cval(a, a.res_rr[e + t], r);
                            qv[t] = cval(a, a.res_rq[e + t], r);
                        }
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                        if (e + t < e1) {
                            const double v = nan0_bits(rv[t]);
                            fr += v;
                            mc = max_abs_bits(mc, v);
                            q += nan0_bits(qv[t]);
                        }
                }
            }
            for (int e = a.ni_ptr[row]; e < a.ni_ptr[row + 1]; ++e) {
                const int kk = a.ni_idx[e];
                double v = kk > 0 ? a.is[(size_t)r * a.n_isrc + kk - 1] : -a.is[(size_t)r * a.n_isrc - kk - 1];
                v = nan0_bits(v);
                fr += v;
                mc = max_abs_bits(mc, v);
            }
            w.fres[row] = fr;
            for (int e = a.nb_ptr[row]; e < a.nb_ptr[row + 1]; ++e) {
                const int kk = a.nb_idx[e];
                fr += kk > 0 ? Xr[(size_t)(a.n_nodes + kk - 1) * a.n_rep + r]
                             : -Xr[(size_t)(a.n_nodes - kk - 1) * a.n_rep + r];
            }
            const size_t o = (size_t)r * a.n_unk + row;
            fn = fr + c0 * q + c1 * a.Qp[o] + d1 * a.dQp[o] + c2 * a.Qp2[o] +
                 (a.gmin + gshunt) * Xr[(size_t)(row + 1) * a.n_rep + r];
            w.Q[row] = q;
            w.maxc[row] = mc;
            tol = fmax(mc * a.reltol, floor_ ? floor_[o] : a.abstol);
        } else {
            const int kk = row - a.n_unk;
            fn = Xr[(size_t)a.vsrc_p[kk] * a.n_rep + r] - Xr[(size_t)a.vsrc_n[kk] * a.n_rep + r] -
                 a.vs[(size_t)r * a.n_vsrc + kk];
            tol = a.vntol;
        }
        w.f[row] = fn;
        if (!isfinite(fn)) nf = true;
        if (a.conv_mask[row] == 1 && !(fabs(fn) < tol)) ok = false;
    }
    __syncwarp();
    *nonfinite = __any_sync(0xffffffffu, nf);
    const bool all_ok = __all_sync(0xffffffffu, ok);
    if (prof && jac) {
        a.phase_cycles[8] += t1 - t0;
        a.phase_cycles[9] += clock64() - t1;
    }
    return all_ok;
}

// Dense LU with partial pivoting (largest |M(i,k)|, ties to the smaller row)
// and the solve of M x = b in place of b, all in shared memory.  The
// diagonal keeps the reciprocal of each pivot, so that the dependent chain of
// the back substitution has no division.  The rank-1 update of each step is
// spread over the lanes element by element (an n = 9 system takes one or two
// FP64 instructions per lane a step instead of one per trailing column), and
// the pivot search and pivot checks are integer work on the bit patterns.
// Returns 1 + the first column whose pivot was zero or not finite (replaced
// by 1e-30), or 0.  `prof` (replica 0, lane 0) accumulates the cycles of the
// factorisation and of the substitutions.
__device__ __noinline__ int replica_lu_solve(int n, double* M, double* b, int lane, long long* prof) {
    int bad = 0;
    const long long t0 = prof ? clock64() : 0;
    for (int k = 0; k < n; ++k) {
        int p;
        if (n - k <= 32) {
            // the column fits the warp: three reductions (high word, low word, first index)
            const int i = k + lane;
            const bool valid = i < n;
            unsigned long long key = 0;
            if (valid) {
                key = (unsigned long long)__double_as_longlong(M[i + (size_t)k * n]) & 0x7fffffffffffffffull;
                if (key > 0x7ff0000000000000ull) key = 0;  // NaN counts as 0
            }
            const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
            const unsigned mh = __reduce_max_sync(0xffffffffu, valid ? hi : 0u);
            const unsigned ml = __reduce_max_sync(0xffffffffu, valid && hi == mh ? lo : 0u);
            p = (int)__reduce_min_sync(0xffffffffu, valid && hi == mh && lo == ml ? (unsigned)i : 0xffffffffu);
        } else {
            unsigned long long best = 0;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                const unsigned long long bits = (unsigned long long)__double_as_longlong(M[i + (size_t)k * n]) &
                                                0x7fffffffffffffffull;  // |M(i,k)|
                const unsigned long long key = bits > 0x7ff0000000000000ull ? 0ull : bits;  // NaN counts as 0
                if (bi == n || key > best) { best = key; bi = i; }
            }
            for (int o = 16; o; o >>= 1) {
                const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (oi < n && (bi == n || ob > best || (ob == best && oi < bi))) { best = ob; bi = oi; }
            }
            p = bi;
        }
        if (p != k) {
            for (int j = lane; j < n; j += 32) {
                const double t = M[k + (size_t)j * n];
                M[k + (size_t)j * n] = M[p + (size_t)j * n];
                M[p + (size_t)j * n] = t;
            }
            if (lane == 0) {
                const double t = b[k];
                b[k] = b[p];
                b[p] = t;
            }
        }
        __syncwarp();
        double piv = M[k + (size_t)k * n];
        const unsigned long long pb = (unsigned long long)__double_as_longlong(piv) & 0x7fffffffffffffffull;
        if (pb == 0ull || pb >= 0x7ff0000000000000ull) {  // zero, infinite or NaN
            piv = 1e-30;
            if (!bad) bad = k + 1;
        }
        const double rinv = vgb_rcp(piv);  // on the chain of dependent pivot steps: the short reciprocal
        __syncwarp();
        if (lane == 0) M[k + (size_t)k * n] = rinv;  // the diagonal keeps 1 / pivot
        for (int i = k + 1 + lane; i < n; i += 32) M[i + (size_t)k * n] *= rinv;
        __syncwarp();
        const int m = n - k - 1;
        for (int t = lane; t < m * m; t += 32) {
            const int jj = t / m, ii = t - jj * m;
            const int i = k + 1 + ii, j = k + 1 + jj;
            M[i + (size_t)j * n] -= M[i + (size_t)k * n] * M[k + (size_t)j * n];
        }
        __syncwarp();
    }
    const long long t1 = prof ? clock64() : 0;
    for (int k = 0; k < n; ++k) {
        const double yk = b[k];
        for (int i = k + 1 + lane; i < n; i += 32) b[i] -= M[i + (size_t)k * n] * yk;
        __syncwarp();
    }
    for (int k = n - 1; k >= 0; --k) {
        if (lane == 0) b[k] *= M[k + (size_t)k * n];
        __syncwarp();
        const double xk = b[k];
        for (int i = lane; i < k; i += 32) b[i] -= M[i + (size_t)k * n] * xk;
        __syncwarp();
    }
    if (prof) {
        prof[0] += t1 - t0;
        prof[1] += clock64() - t1;
    }
    return bad;
}

// One Newton iteration of replica r at Xc with the current contributions
// (solver_factories.py:230-325): assemble, solve J delta = -f, convergence
// tests, update.  Afterwards the replica needs an evaluation at the new Xc.
__device__ void replica_nr(const BatchArgs& a, const WarpWS& w, int r, BRep& s, int lane) {
    const int n = a.n_aug;
    const double* fl = s.fixed ? nullptr : a.floor_;
    bool nonfinite = false;
    const long long c0 = clock64();
    const bool res_ok = replica_assemble(a, w, r, s.k, fl, true, &nonfinite, lane);
    double* b = w.f;
    for (int i = lane; i < n; i += 32) b[i] = -b[i];
    __syncwarp();
    const long long c1 = clock64();
    const int bad = replica_lu_solve(n, w.M, b, lane, r == 0 && lane == 0 ? a.phase_cycles + 10 : nullptr);
    const long long c2 = clock64();
    // delta test (before the update) and the damped update
    bool dok = true;
    double max_dv = 0.0;
    for (int i = lane; i < n; i += 32) {
        const double d = b[i];
        const bool is_v = i < a.n_unk;
        const double conv = is_v ? d * a.damping : d;
        const double tol = fmax(fabs(a.Xc[(size_t)(i + 1) * a.n_rep + r]) * a.reltol, is_v ? a.vntol : a.abstol);
        if (!(fabs(conv) < tol)) dok = false;
        if (is_v) max_dv = fmax(max_dv, fabs(d) != fabs(d) ? INFINITY : fabs(d));
    }
    const bool delta_ok = __all_sync(0xffffffffu, dok);
    max_dv = warp_max(max_dv);
    const double scale = fmin(1.0, 1e30 / fmax(max_dv, 1e-30));
    for (int i = lane; i < n; i += 32) {
        double* x = a.Xc + (size_t)(i + 1) * a.n_rep + r;
        *x += i < a.n_unk ? b[i] * scale * a.damping : b[i];
    }
    const int it = s.nr_it;
    const int itl = s.tran_itl;
    __syncwarp();
    const bool conv = !nonfinite && res_ok && (it == 0 || delta_ok);
    const bool stop = nonfinite || conv || it + 1 >= itl;
    if (lane == 0) {
        if (bad) s.pivot_err = 1;
        if (conv) s.nr_conv = 1;
        s.nr_it = it + 1;
        if (stop) s.state = RS_POST;
        s.need_eval = 1;
    }
    __syncwarp();
    if (r == 0 && lane == 0) {
        const long long c3 = clock64();
        a.phase_cycles[4] += c1 - c0;
        a.phase_cycles[5] += c2 - c1;
        a.phase_cycles[6] += c3 - c2;
    }
}

// Plan of the next step (coefficients, sources at t_next, initial guess).
// Returns true when the initial guess is the point of the last evaluation
// (so the first Newton iteration reuses its contributions).
__device__ bool replica_plan(const BatchArgs& a, int r, BRep& s, bool last_eval_at_X, int lane) {
    StepPlan p;
    if (lane == 0) p = ctl_plan(s);
    for (int q = 0; q < 5; ++q) p.k[q] = __shfl_sync(0xffffffffu, p.k[q], 0);
    p.t_next = __shfl_sync(0xffffffffu, p.t_next, 0);
    p.kl = __shfl_sync(0xffffffffu, p.kl, 0);
    for (int q = 0; q < 3; ++q) {
        p.pa[q] = __shfl_sync(0xffffffffu, p.pa[q], 0);
        p.slot[q] = __shfl_sync(0xffffffffu, p.slot[q], 0);
    }
    p.can_predict = __shfl_sync(0xffffffffu, p.can_predict, 0);
    if (lane == 0) {
        s.plan = p;
        for (int q = 0; q < 5; ++q) s.k[q] = p.k[q];
        s.nr_it = 0;
        s.nr_conv = 0;
        s.state = RS_NR;
    }
    replica_sources(a, r, p.t_next, lane);
    const bool fixed = s.fixed != 0;
    const bool predict = !fixed && p.can_predict;
    for (int i = lane; i < a.n_x; i += 32) {
        const size_t xi = (size_t)i * a.n_rep + r;
        double v = a.X[xi];
        if (!fixed && i < a.n_nodes) {
            const double* h = a.hist + (size_t)r * 4 * a.n_nodes;
            const double vp = p.pa[0] * h[(size_t)p.slot[0] * a.n_nodes + i] +
                              p.pa[1] * h[(size_t)p.slot[1] * a.n_nodes + i] +
                              p.pa[2] * h[(size_t)p.slot[2] * a.n_nodes + i];
            a.Vpred[(size_t)r * a.n_nodes + i] = vp;
            if (predict) v = vp;
        }
        a.Xc[xi] = v;
    }
    if (!fixed)
        for (int i = lane; i < a.n_unk; i += 32) {
            const size_t o = (size_t)r * a.n_unk + i;
            a.floor_[o] = fmax(a.hmaxc[o] * a.reltol, a.abstol);
        }
    __syncwarp();
    return !predict && last_eval_at_X;
}

// The step after Newton (full_mna.py:1931-2147): rebuild at the converged
// point, branch currents, dQ/dt, LTE, accept/reject, commit and outputs.
// Returns true when the replica continues with another step.
__device__ bool replica_finish_step(const BatchArgs& a, const WarpWS& w, int r, BRep& s, bool* reuse, int lane) {
    const int nu = a.n_unk, nn = a.n_nodes;
    bool nonfinite = false;
    const double* fl = s.fixed ? nullptr : a.floor_;
    replica_assemble(a, w, r, s.k, fl, false, &nonfinite, lane);
    const double* Q = w.Q;
    const double* fres = w.fres;
    // LTE norm (adaptive.py:221-264)
    double lte = 0.0;
    if (!s.fixed) {
        const double kl = s.plan.kl;
        for (int i = lane; i < nn; i += 32) {
            const double vn = a.Xc[(size_t)i * a.n_rep + r];
            const double vp = a.Vpred[(size_t)r * nn + i];
            const double l = (vn - vp) * kl;
            const double vcur = fmax(fabs(vn), fabs(vp));
            const double vs = fmax(a.Vmax[(size_t)r * nn + i], vcur);
            double v = fabs(l) / (a.reltol * vs + a.abstol);
            if (v != v) v = INFINITY;
            lte = fmax(lte, v);
        }
        lte = warp_max(lte);
    }
    __syncwarp();
    StepCommit m;
    if (lane == 0) m = ctl_finish(s, s.plan, lte, s.nr_it, s.nr_conv != 0, a.tout + (size_t)r * a.max_steps);
    m.use_new = __shfl_sync(0xffffffffu, m.use_new, 0);
    m.accept = __shfl_sync(0xffffffffu, m.accept, 0);
    m.zero_current = __shfl_sync(0xffffffffu, m.zero_current, 0);
    m.row = __shfl_sync(0xffffffffu, m.row, 0);
    m.slot = __shfl_sync(0xffffffffu, m.slot, 0);
    const int done = __shfl_sync(0xffffffffu, s.done, 0);
    const double k0 = s.k[0], k1 = s.k[1], k2 = s.k[2], k3 = s.k[3];
    // commit (full_mna.py:2078-2147)
    if (m.accept) {
        double* vrow = a.Vout + ((size_t)r * a.max_steps + m.row) * a.n_ext;
        for (int i = lane; i < a.n_ext; i += 32)
            vrow[i] = m.use_new ? a.Xc[(size_t)i * a.n_rep + r] : a.X[(size_t)i * a.n_rep + r];
        double* irow = a.Iout + ((size_t)r * a.max_steps + m.row) * a.nvo;
        for (int k = lane; k < a.n_vsrc; k += 32) {
            const int p = a.vsrc_p[k];
            irow[k] = m.zero_current ? 0.0 : (p > 0 ? -fres[p - 1] : 0.0);
        }
    }
    if (m.use_new) {
        for (int i = lane; i < a.n_x; i += 32) a.X[(size_t)i * a.n_rep + r] = a.Xc[(size_t)i * a.n_rep + r];
        for (int i = lane; i < nu; i += 32) {
            const size_t o = (size_t)r * nu + i;
            const double dq = k0 * Q[i] + k1 * a.Qp[o] + k2 * a.dQp[o] + k3 * a.Qp2[o];
            a.Qp2[o] = a.Qp[o];
            a.Qp[o] = Q[i];
            a.dQp[o] = dq;
            a.hmaxc[o] = fmax(a.hmaxc[o], w.maxc[i]);
        }
        for (int i = lane; i < nn; i += 32) {
            const double xc = a.Xc[(size_t)i * a.n_rep + r];
            a.hist[((size_t)r * 4 + m.slot) * nn + i] = xc;
            a.Vmax[(size_t)r * nn + i] = fmax(a.Vmax[(size_t)r * nn + i], fabs(xc));
        }
    }
    __syncwarp();
    if (done) {
        if (lane == 0) {
            s.state = RS_DONE;
            s.need_eval = 0;
        }
        __syncwarp();
        return false;
    }
    // the last evaluation was at Xc; after an accepted step X == Xc
    *reuse = replica_plan(a, r, s, m.use_new != 0, lane);
    return true;
}

// The uic start: charges and branch currents from the evaluation at X0
// (the engine's initial condition), then the plan of the first step.
__device__ bool replica_init(const BatchArgs& a, const WarpWS& w, int r, BRep& s, int lane) {
    const int nu = a.n_unk;
    bool nonfinite = false;
    replica_sources(a, r, 0.0, lane);
    __syncwarp();
    const double kz[5] = {0, 0, 0, 0, 0};
    replica_assemble(a, w, r, kz, nullptr, false, &nonfinite, lane);
    for (int i = lane; i < nu; i += 32) {
        const size_t o = (size_t)r * nu + i;
        a.Qp[o] = w.Q[i];
        a.hmaxc[o] = 0.0;
    }
    if (!s.fixed) {
        double* irow = a.Iout + (size_t)r * a.max_steps * a.nvo;
        for (int k = lane; k < a.n_vsrc; k += 32) {
            const int p = a.vsrc_p[k];
            irow[k] = p > 0 ? -w.fres[p - 1] : 0.0;
        }
    }
    __syncwarp();
    return replica_plan(a, r, s, true, lane);
}

__device__ void replica_tick_body(const BatchArgs& a, const WarpWS& w, int r, BRep& s, int lane) {
    const int state = s.state;
    if (state == RS_DONE) return;
    __syncwarp();
    if (lane == 0) s.need_eval = 0;
    __syncwarp();
    bool reuse = true;
    if (state == RS_INIT) {
        reuse = replica_init(a, w, r, s, lane);
    } else if (state == RS_START) {
        reuse = replica_plan(a, r, s, true, lane);  // the evaluation of this tick was at X0
    } else if (state == RS_POST) {
        const long long c0 = clock64();
        const bool more = replica_finish_step(a, w, r, s, &reuse, lane);
        if (r == 0 && lane == 0) a.phase_cycles[7] += clock64() - c0;
        if (!more) return;
    }
    __syncwarp();
    if (!reuse) {
        if (lane == 0) s.need_eval = 1;
        __syncwarp();
        return;
    }
    // RS_NR: the contributions in hand are those of Xc
    replica_nr(a, w, r, s, lane);
}

// One tick of replica r.  Its controller state lives in the warp's shared
// workspace for the tick: every field the step reads (Newton coefficients,
// counters, the plan) would otherwise be a dependent global load, each an L2
// round trip since lane 0 rewrote the line in the previous tick.
__device__ __noinline__ void replica_tick(const BatchArgs& a, int r, int lane) {
    BRep* gs = a.rep + r;
    if (gs->state == RS_DONE) return;
    const WarpWS w = warp_ws(a);
    copy_brep(w.rep, gs, lane);
    __syncwarp();
    replica_tick_body(a, w, r, *w.rep, lane);
    __syncwarp();
    copy_brep(gs, w.rep, lane);
    __syncwarp();
}

// Bytes of the staged gather lists, each array 16-byte aligned, in the order
// stage_pattern lays them out.
__host__ __device__ inline size_t stage_bytes(int nnz, int ncs, int nu, int nrs) {
    auto al = [](size_t b) { return (b + 15) & ~(size_t)15; };
    return al(4 * (size_t)(nnz + 1)) + 2 * al(4 * (size_t)ncs) + 2 * al(4 * (size_t)nnz) + al(8 * (size_t)nnz) +
           al((size_t)nnz) + al(4 * (size_t)(nu + 1)) + 2 * al(4 * (size_t)nrs);
}

// The assembly's gather lists (the same for every replica and tick) copied
// into this CTA's shared memory; `s` gets pointers to the copies.  Each
// contribution's gather is then one global load (the value) instead of a
// chain of three.
__device__ void stage_pattern(const BatchArgs& a, BatchArgs& s) {
    extern __shared__ double batch_smem[];
    unsigned char* base = reinterpret_cast<unsigned char*>(batch_smem) + a.stage_off;
    auto al = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const int nnz = a.nnz, ncs = a.n_csr_src, nu = a.n_unk > 0 ? a.n_unk : 0, nrs = a.n_res_src;
    auto take = [&](size_t bytes) { unsigned char* p = base; base += al(bytes); return p; };
    int* csr_ptr = (int*)take(4 * (size_t)(nnz + 1));
    int* csr_jr = (int*)take(4 * (size_t)ncs);
    int* csr_jq = (int*)take(4 * (size_t)ncs);
    int* csr_row = (int*)take(4 * (size_t)nnz);
    int* indices = (int*)take(4 * (size_t)nnz);
    double* csr_const = (double*)take(8 * (size_t)nnz);
    unsigned char* csr_diag = take((size_t)nnz);
    int* res_ptr = (int*)take(4 * (size_t)(nu + 1));
    int* res_rr = (int*)take(4 * (size_t)nrs);
    int* res_rq = (int*)take(4 * (size_t)nrs);
    for (int i = threadIdx.x; i <= nnz; i += blockDim.x) csr_ptr[i] = a.csr_ptr[i];
    for (int i = threadIdx.x; i < ncs; i += blockDim.x) {
        csr_jr[i] = a.csr_jr[i];
        csr_jq[i] = a.csr_jq[i];
    }
    for (int i = threadIdx.x; i < nnz; i += blockDim.x) {
        csr_row[i] = a.csr_row[i];
        indices[i] = a.indices[i];
        csr_const[i] = a.csr_const[i];
        csr_diag[i] = a.csr_diag[i];
    }
    for (int i = threadIdx.x; i <= nu; i += blockDim.x) res_ptr[i] = a.res_ptr[i];
    for (int i = threadIdx.x; i < nrs; i += blockDim.x) {
        res_rr[i] = a.res_rr[i];
        res_rq[i] = a.res_rq[i];
    }
    __syncthreads();
    s.csr_ptr = csr_ptr; s.csr_jr = csr_jr; s.csr_jq = csr_jq; s.csr_row = csr_row; s.indices = indices;
    s.csr_const = csr_const; s.csr_diag = csr_diag; s.res_ptr = res_ptr; s.res_rr = res_rr; s.res_rq = res_rq;
}

__global__ void __launch_bounds__(BATCH_THREADS, 1) batch_kernel(BatchArgs a) {
    const int lane = threadIdx.x & 31;
    // the replica step reads the gather lists from this CTA's shared memory when they are staged
    BatchArgs ra = a;
    if (a.stage) stage_pattern(a, ra);
    const int warps = blockDim.x >> 5;
    // replicas dealt round-robin over the CTAs, like the evaluation warps
    const int gw = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
    const int nw = gridDim.x * warps;
    const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
    long long cyc[4] = {0, 0, 0, 0};
    for (long long tick = 0; tick < a.max_ticks; ++tick) {
        const long long c0 = clock64();
        eval_phase(a);
        const long long c1 = clock64();
        grid_barrier(a);
        const long long c2 = clock64();
        int mine = 0;
        for (int r = gw; r < a.n_rep; r += nw) {
            replica_tick(ra, r, lane);
            __syncwarp();
            mine += a.rep[r].state != RS_DONE;
        }
        if (lane == 0 && mine) atomicAdd(&a.active[tick & 1], mine);
        if (blockIdx.x == 0 && threadIdx.x == 0) a.active[(tick + 1) & 1] = 0;
        const long long c3 = clock64();
        grid_barrier(a);
        if (timer) {
            cyc[0] += c1 - c0;
            cyc[1] += c2 - c1;
            cyc[2] += c3 - c2;
            cyc[3] += clock64() - c3;
            for (int q = 0; q < 4; ++q) a.phase_cycles[q] = cyc[q];
        }
        const int left = *(volatile int*)&a.active[tick & 1];
        const int err = *(volatile int*)a.err;
        if (left == 0 || err) {
            if (blockIdx.x == 0 && threadIdx.x == 0) *a.ticks_out = tick + 1;
            return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.ticks_out = a.max_ticks;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static bool model_has_coop(int model) {
    switch (model) {
#define VGB_COOP_ID(ID, STRUCT) \
    case ID: return true;
        VGB_COOP_LIST(VGB_COOP_ID)
#undef VGB_COOP_ID
        default: return false;
    }
}

static int model_ncache(int model) {
    switch (model) {
#define VGB_COOP_NC(ID, STRUCT) \
    case ID: return STRUCT::NCACHE;
        VGB_COOP_LIST(VGB_COOP_NC)
#undef VGB_COOP_NC
        default: return 0;
    }
}

static void launch_cache(const BGroup& g, int n_rep, cudaStream_t s) {
    const long long n = (long long)g.n_dev * n_rep;
    const int blocks = (int)((n + 127) / 128);
    switch (g.model) {
#define VGB_COOP_LAUNCH(ID, STRUCT) \
    case ID: batch_cache_kernel<STRUCT><<<blocks, 128, 0, s>>>(g, n_rep); break;
        VGB_COOP_LIST(VGB_COOP_LAUNCH)
#undef VGB_COOP_LAUNCH
        default: break;
    }
}

struct Batch {
    Circuit* c = nullptr;
    int n_rep = 0;
    std::string last_error;
    std::vector<BGroup> groups;             // device pointers filled on upload
    std::vector<std::vector<int>> vidx;     // per group [np]
    std::vector<std::vector<double>> vvals; // per group [n_var][n_dev][n_rep]
    std::vector<std::vector<double>> temps; // per group [n_dev][n_rep] or empty
    std::vector<double> vs_data, is_data;   // [n_rep][len]
    // device
    DevBuf<BGroup> d_groups;
    DevBuf<int> d_csr_row, d_indices, d_csr_ptr, d_csr_jr, d_csr_jq, d_res_ptr, d_res_rr, d_res_rq;
    DevBuf<int> d_nb_ptr, d_nb_idx, d_ni_ptr, d_ni_idx, d_vsrc_p, d_vsrc_n;
    DevBuf<int> d_vs_kind, d_vs_off, d_vs_cnt, d_is_kind, d_is_off, d_is_cnt;
    DevBuf<double> d_csr_const, d_vs_data, d_is_data;
    DevBuf<unsigned char> d_csr_diag, d_conv_mask;
    std::vector<DevBuf<int>> d_node_map, d_vidx;
    std::vector<DevBuf<double>> d_shared, d_varying, d_temps, d_cache;
    long long n_contrib = 0, n_items = 0, n_coop_units = 0;
    int coop = 1;  // cooperative evaluation: 0 never, 1 when its item warps fit one per SM, 2 always
    double run_ms = 0.0;
    long long ticks = 0;
    long long phase_cycles[12] = {0};
};

static void batch_require(bool ok, const std::string& m) {
    if (!ok) throw Error(VGB_ERR_INVALID, m);
}

// The dynamic shared memory a batch launch may take beside the kernel's static
// shared memory.  The kernel's maximum is raised to that bound once per
// device and never lowered: batches sized differently run from several host
// threads, and a per-launch setting could shrink the limit between another
// thread's setting and its launch.
static size_t batch_smem_limit(int smem_optin) {
    static std::mutex mu;
    static std::vector<size_t> done;
    int dev = 0;
    VGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (!done[dev]) {
        cudaFuncAttributes fa{};
        VGB_CUDA(cudaFuncGetAttributes(&fa, batch_kernel));
        const size_t lim = (size_t)smem_optin > fa.sharedSizeBytes ? (size_t)smem_optin - fa.sharedSizeBytes : 0;
        VGB_CUDA(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim));
        done[dev] = lim;
    }
    return done[dev];
}

// Host-side set-up: checks, the gather lists mapped onto the batch
// contribution layout, per-replica parameters from the template.  Uploads
// nothing (batch_run does), so the checks run without a GPU.
static void batch_build(Batch& b) {
    Circuit& c = *b.c;
    if (!c.analyzed) {
        build_pattern(c);
        build_sparse_symbolic(c);
        c.analyzed = true;
    }
    batch_require(c.n_aug >= 1 && c.n_aug <= BATCH_MAX_N, "batched transient: n_aug = " + std::to_string(c.n_aug) +
                                                              " is outside 1.." + std::to_string(BATCH_MAX_N));
    batch_require(c.noi_idx.empty(), "batched transient: circuits with NOI nodes are not supported");
    batch_require((int)c.groups.size() <= BATCH_MAX_GROUPS, "batched transient: too many model groups");
    const int R = b.n_rep;
    // contribution layout per group: [2 NJ + 2 NN][n_dev] (jr, jq, rr, rq); the
    // template's gather entries ([NJ + 2 NN][n_dev]: jac, rr, rq) map onto it
    std::vector<long long> tbase(c.groups.size()), bbase(c.groups.size());
    long long nb = 0, items = 0;
    b.groups.assign(c.groups.size(), BGroup{});
    for (size_t g = 0; g < c.groups.size(); ++g) {
        const Group& G = c.groups[g];
        tbase[g] = G.contrib_base;
        bbase[g] = nb;
        nb += (long long)(2 * G.nj + 2 * G.nn) * G.n_dev;
        BGroup& B = b.groups[g];
        B.model = G.model;
        B.n_dev = G.n_dev;
        B.nn = G.nn;
        B.nj = G.nj;
        B.np = G.np;
        B.temp_shared = G.temp_shared;
        B.cbase = bbase[g];
        B.item0 = items;
        items += ((long long)G.n_dev * R + 31) / 32 * 32;
        B.cu0 = B.cu1 = 0;
    }
    b.n_contrib = nb;
    b.n_items = items;
    batch_require(nb * (long long)R < (1LL << 31), "batched transient: too many contribution slots");
    b.vidx.assign(c.groups.size(), {});
    b.vvals.assign(c.groups.size(), {});
    b.temps.assign(c.groups.size(), {});
    for (size_t g = 0; g < c.groups.size(); ++g) {
        const Group& G = c.groups[g];
        b.vidx[g] = G.vidx;
        const int nv = G.n_dev ? (int)(G.varying.size() / G.n_dev) : 0;
        b.vvals[g].assign((size_t)nv * G.n_dev * R, 0.0);
        for (int v = 0; v < nv; ++v)
            for (int d = 0; d < G.n_dev; ++d)
                for (int r = 0; r < R; ++r)
                    b.vvals[g][((size_t)v * G.n_dev + d) * R + r] = G.varying[(size_t)v * G.n_dev + d];
        if (!G.temps.empty()) {
            b.temps[g].assign((size_t)G.n_dev * R, 0.0);
            for (int d = 0; d < G.n_dev; ++d)
                for (int r = 0; r < R; ++r) b.temps[g][(size_t)d * R + r] = G.temps[d];
        }
    }
    b.vs_data.assign((size_t)R * c.vsrc_wave.data.size(), 0.0);
    for (int r = 0; r < R; ++r)
        std::copy(c.vsrc_wave.data.begin(), c.vsrc_wave.data.end(),
                  b.vs_data.begin() + (size_t)r * c.vsrc_wave.data.size());
    b.is_data.assign((size_t)R * c.isrc_wave.data.size(), 0.0);
    for (int r = 0; r < R; ++r)
        std::copy(c.isrc_wave.data.begin(), c.isrc_wave.data.end(),
                  b.is_data.begin() + (size_t)r * c.isrc_wave.data.size());
}

static void batch_upload_pattern(Batch& b) {
    Circuit& c = *b.c;
    std::vector<long long> tbase(c.groups.size());
    for (size_t g = 0; g < c.groups.size(); ++g) tbase[g] = c.groups[g].contrib_base;
    auto locate = [&](int idx, int& g, int& slot, int& d) {
        for (g = (int)c.groups.size() - 1; g > 0 && idx < tbase[g]; --g) {}
        const Group& G = c.groups[g];
        const long long loc = idx - tbase[g];
        slot = (int)(loc / G.n_dev);
        d = (int)(loc % G.n_dev);
    };
    std::vector<int> csr_ptr(c.nnz + 1, 0), csr_jr, csr_jq;
    for (int e = 0; e < c.nnz; ++e) {
        for (int q = c.csr_src_ptr[e]; q < c.csr_src_ptr[e + 1]; ++q) {
            int g, slot, d;
            locate(c.csr_src[q], g, slot, d);
            const Group& G = c.groups[g];
            batch_require(slot < G.nj, "batched transient: unexpected Jacobian gather entry");
            csr_jr.push_back((int)(b.groups[g].cbase + (long long)slot * G.n_dev + d));
            csr_jq.push_back((int)(b.groups[g].cbase + (long long)(G.nj + slot) * G.n_dev + d));
        }
        csr_ptr[e + 1] = (int)csr_jr.size();
    }
    std::vector<int> res_rr, res_rq;
    for (size_t q = 0; q < c.res_src.size(); ++q) {
        int g, slot, d;
        locate(c.res_src[q], g, slot, d);
        const Group& G = c.groups[g];
        batch_require(slot >= G.nj && slot < G.nj + G.nn, "batched transient: unexpected residual gather entry");
        res_rr.push_back((int)(b.groups[g].cbase + (long long)(G.nj + slot) * G.n_dev + d));
        locate(c.rq_src[q], g, slot, d);
        const Group& H = c.groups[g];
        res_rq.push_back((int)(b.groups[g].cbase + (long long)(H.nj + slot) * H.n_dev + d));
    }
    std::vector<int> csr_row(c.nnz);
    for (int row = 0; row < c.n_aug; ++row)
        for (int e = c.indptr[row]; e < c.indptr[row + 1]; ++e) csr_row[e] = row;
    b.d_csr_row.upload(csr_row);
    b.d_indices.upload(c.indices);
    b.d_csr_ptr.upload(csr_ptr);
    b.d_csr_jr.upload(csr_jr);
    b.d_csr_jq.upload(csr_jq);
    b.d_csr_const.upload(c.csr_const);
    b.d_csr_diag.upload(c.csr_diag);
    b.d_res_ptr.upload(c.res_src_ptr);
    b.d_res_rr.upload(res_rr);
    b.d_res_rq.upload(res_rq);
    b.d_nb_ptr.upload(c.nb_ptr);
    b.d_nb_idx.upload(c.nb_idx);
    b.d_ni_ptr.upload(c.ni_ptr);
    b.d_ni_idx.upload(c.ni_idx);
    b.d_vsrc_p.upload(c.vsrc_p);
    b.d_vsrc_n.upload(c.vsrc_n);
    b.d_conv_mask.upload(c.conv_mask);
    b.d_vs_kind.upload(c.vsrc_wave.kind);
    b.d_vs_off.upload(c.vsrc_wave.off);
    b.d_vs_cnt.upload(c.vsrc_wave.cnt);
    b.d_is_kind.upload(c.isrc_wave.kind);
    b.d_is_off.upload(c.isrc_wave.off);
    b.d_is_cnt.upload(c.isrc_wave.cnt);
    const size_t ng = c.groups.size();
    b.d_node_map.resize(ng);
    b.d_vidx.resize(ng);
    b.d_shared.resize(ng);
    b.d_varying.resize(ng);
    b.d_temps.resize(ng);
    for (size_t g = 0; g < ng; ++g) {
        b.d_node_map[g].upload(c.groups[g].node_map);
        b.d_shared[g].upload(c.groups[g].shared);
    }
}

static void batch_run(Batch& b, const double* cfg, const double* X0, const double* Q0, const double* I0,
                      const double* maxc0, double* times, double* V_out, double* I_out, double* stats) {
    Circuit& c = *b.c;
    const int R = b.n_rep;
    const int n_nodes = c.n_nodes, nu = c.n_unk, nv = c.n_vsrc, ni = c.n_isrc, n = c.n_aug;
    const int nx = n_nodes + nv;
    const int nvo = std::max(nv, 1);
    const double t_stop = cfg[0], dt = cfg[1];
    const int n_ext = (int)cfg[19], max_steps = (int)cfg[20], itl = (int)cfg[21];
    const bool fixed = cfg[17] != 0.0;
    const int method = (int)cfg[18];
    batch_require(n_ext >= 1 && n_ext <= n_nodes, "n_external out of range");
    batch_require(max_steps >= 1, "max_steps must be >= 1");
    batch_require(dt > 0 && t_stop >= 0, "bad time parameters");
    batch_require(method >= 0 && method <= 2, "method must be 0 (BE), 1 (trap) or 2 (gear2)");
    batch_require(itl >= 1, "tran_itl must be >= 1");
    batch_require(X0 != nullptr, "X0 is required");
    cudaStream_t s = c.stream;
    if (!b.d_csr_ptr.p) batch_upload_pattern(b);
    for (size_t g = 0; g < c.groups.size(); ++g) {
        b.d_vidx[g].upload(b.vidx[g]);
        b.d_varying[g].upload(b.vvals[g]);
        if (!b.temps[g].empty()) b.d_temps[g].upload(b.temps[g]);
        else b.d_temps[g].release();
        BGroup& B = b.groups[g];
        B.node_map = b.d_node_map[g].p;
        B.shared = b.d_shared[g].p;
        B.vidx = b.d_vidx[g].p;
        B.varying = b.d_varying[g].p;
        B.temps = b.temps[g].empty() ? nullptr : b.d_temps[g].p;
    }
    // cooperative units: the item warps of the models that have a cooperative
    // body, when their exchange slots fit in shared memory beside nothing else
    int dev = 0;
    VGB_CUDA(cudaGetDevice(&dev));
    int sms = 0, per_sm = 0, smem_optin = 0;
    VGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    VGB_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // dynamic shared memory left beside the kernel's static shared memory
    const size_t smem_limit = batch_smem_limit(smem_optin);
    // per-warp gather scratch only when the workspaces still fit with it
    int ws_sc = ws_scratch((int)b.d_csr_jr.n, (int)b.d_res_rr.n);
    if (sizeof(double) * ws_doubles(n, nu, ws_sc) * (BATCH_THREADS / 32) > smem_limit) ws_sc = 0;
    const size_t ws_bytes = sizeof(double) * ws_doubles(n, nu, ws_sc) * (BATCH_THREADS / 32);
    batch_require(ws_bytes <= smem_limit, "batched transient: the circuit's dense Newton matrix does not fit in shared memory");
    const long long coop_stride = 32LL * VGB_COOP_SLOTS_MAX;
    const size_t coop_bytes = sizeof(double) * coop_stride * (BATCH_THREADS / 32 / COOP_WARPS);
    // FP64 issue on GB300 is an SM-wide budget (about one warp-instruction per
    // 19 cycles) that one warp can use only a third of (one per 64 cycles):
    // eight warps sharing an instance finish it 2.5x sooner than one warp, but
    // the if-converted body holds more instructions, so the cooperative
    // evaluation pays only while no SM holds more than one group's work.
    long long units = 0;
    for (const BGroup& B : b.groups)
        if (model_has_coop(B.model)) units += ((long long)B.n_dev * R + 31) / 32;
    const bool coop = b.coop && coop_bytes <= smem_limit && (units <= sms || b.coop == 2);
    b.n_coop_units = 0;
    b.d_cache.resize(c.groups.size());
    for (size_t g = 0; g < c.groups.size(); ++g) {
        BGroup& B = b.groups[g];
        B.cu0 = B.cu1 = b.n_coop_units;
        B.cache = nullptr;
        if (model_has_coop(B.model) && B.n_dev > 0) {
            if (coop) {
                B.cu1 = B.cu0 + ((long long)B.n_dev * R + 31) / 32;
                b.n_coop_units = B.cu1;
            }
            // the cache serves the one-warp evaluation as well
            b.d_cache[g].alloc((size_t)model_ncache(B.model) * B.n_dev * R);
            B.cache = b.d_cache[g].p;
            launch_cache(B, R, c.stream);  // ordered before the persistent kernel on the same stream
        }
    }
    VGB_CUDA(cudaGetLastError());
    b.d_groups.upload(b.groups);
    b.d_vs_data.upload(b.vs_data);
    b.d_is_data.upload(b.is_data);
    // state, batch-interleaved where the evaluation reads it
    DevBuf<double> X, Xc, contrib, Qp, Qp2, dQp, hmaxc, floor_, Vpred, Vmax, hist, vs, is;
    DevBuf<double> tout, Vout, Iout;
    DevBuf<BRep> rep;
    DevBuf<unsigned> bar;
    DevBuf<int> ctl;
    DevBuf<long long> ticks, pcyc;
    std::vector<double> hX((size_t)nx * R), hhist((size_t)R * 4 * n_nodes, 0.0), hVmax((size_t)R * n_nodes);
    std::vector<double> hQp((size_t)R * std::max(nu, 1), 0.0), hmx((size_t)R * std::max(nu, 1), 0.0);
    std::vector<double> hVout((size_t)R * max_steps * n_ext, 0.0), hIout((size_t)R * max_steps * nvo, 0.0);
    for (int r = 0; r < R; ++r) {
        const double* x0 = X0 + (size_t)r * nx;
        for (int i = 0; i < nx; ++i) hX[(size_t)i * R + r] = x0[i];
        for (int i = 0; i < n_nodes; ++i) {
            hhist[(size_t)r * 4 * n_nodes + i] = x0[i];
            hVmax[(size_t)r * n_nodes + i] = std::fabs(x0[i]);
        }
        for (int i = 0; i < n_ext; ++i) hVout[(size_t)r * max_steps * n_ext + i] = x0[i];
        if (Q0)
            for (int i = 0; i < nu; ++i) hQp[(size_t)r * nu + i] = Q0[(size_t)r * nu + i];
        if (maxc0)
            for (int i = 0; i < nu; ++i) hmx[(size_t)r * nu + i] = maxc0[(size_t)r * nu + i];
        if (Q0 && I0 && nv && !fixed)
            for (int k = 0; k < nv; ++k) hIout[(size_t)r * max_steps * nvo + k] = I0[(size_t)r * nv + k];
    }
    X.upload(hX);
    Xc.upload(hX);
    hist.upload(hhist);
    Vmax.upload(hVmax);
    Qp.upload(hQp);
    hmaxc.upload(hmx);
    Vout.upload(hVout);
    Iout.upload(hIout);
    const size_t nuR = (size_t)R * std::max(nu, 1);
    contrib.alloc((size_t)b.n_contrib * R);
    Qp2.alloc(nuR); dQp.alloc(nuR); floor_.alloc(nuR);
    Qp2.zero(s); dQp.zero(s); floor_.zero(s);
    Vpred.alloc((size_t)R * n_nodes);
    Vpred.zero(s);
    vs.alloc((size_t)R * std::max(nv, 1));
    is.alloc((size_t)R * std::max(ni, 1));
    vs.zero(s); is.zero(s);
    tout.alloc((size_t)R * max_steps);
    tout.zero(s);
    // controller state, as TranSession::setup
    std::vector<BRep> hr(R);
    for (int r = 0; r < R; ++r) {
        BRep& q = hr[r];
        std::memset(&q, 0, sizeof(BRep));
        q.t_stop = t_stop; q.max_dt = cfg[2]; q.min_dt = cfg[3]; q.lte_ratio = cfg[7]; q.redo_factor = cfg[8];
        q.grow_factor = cfg[9]; q.tran_ft = cfg[10]; q.gshunt_init = cfg[12]; q.gshunt_target = cfg[13];
        q.gshunt_steps = (int)cfg[14]; q.warmup_steps = (int)cfg[15]; q.max_consec = (int)cfg[16];
        q.method = method; q.max_steps = max_steps; q.tran_itl = itl; q.fixed = fixed ? 1 : 0;
        q.t = 0.0; q.dt = dt;
        for (double& d : q.dt_hist) d = dt;
        q.head = 0; q.history_count = 1; q.step_idx = 1;
        q.min_dt_used = q.max_dt_used = dt;
        if (fixed) {
            q.fixed_n = std::min((int)(t_stop / dt), max_steps - 1);
            if (q.fixed_n < 1) q.fixed_n = 1;
        }
        q.done = (!fixed && !(q.t < q.t_stop && q.step_idx < q.max_steps)) ? 1 : 0;
        q.state = q.done ? RS_DONE : (Q0 ? RS_START : RS_INIT);
        q.need_eval = q.done ? 0 : 1;
    }
    rep.upload(hr);
    bar.alloc(2);
    bar.zero(s);
    ctl.alloc(3);  // active[2], err
    ctl.zero(s);
    ticks.alloc(1);
    ticks.zero(s);
    pcyc.alloc(12);
    pcyc.zero(s);
    VGB_CUDA(cudaStreamSynchronize(s));

    BatchArgs a{};
    a.n_rep = R; a.n_nodes = n_nodes; a.n_unk = nu; a.n_vsrc = nv; a.n_isrc = ni; a.n_aug = n; a.n_x = nx;
    a.n_ext = n_ext; a.nvo = nvo; a.nnz = c.nnz; a.n_groups = (int)c.groups.size();
    a.n_items = b.n_items; a.n_contrib = b.n_contrib;
    a.gmin = c.gmin; a.reltol = cfg[4]; a.abstol = cfg[5]; a.vntol = cfg[6]; a.damping = cfg[11];
    a.groups = b.d_groups.p;
    a.csr_row = b.d_csr_row.p; a.indices = b.d_indices.p;
    a.csr_ptr = b.d_csr_ptr.p; a.csr_jr = b.d_csr_jr.p; a.csr_jq = b.d_csr_jq.p;
    a.csr_const = b.d_csr_const.p; a.csr_diag = b.d_csr_diag.p;
    a.res_ptr = b.d_res_ptr.p; a.res_rr = b.d_res_rr.p; a.res_rq = b.d_res_rq.p;
    a.nb_ptr = b.d_nb_ptr.p; a.nb_idx = b.d_nb_idx.p; a.ni_ptr = b.d_ni_ptr.p; a.ni_idx = b.d_ni_idx.p;
    a.vsrc_p = b.d_vsrc_p.p; a.vsrc_n = b.d_vsrc_n.p; a.conv_mask = b.d_conv_mask.p;
    a.vs_kind = b.d_vs_kind.p; a.vs_off = b.d_vs_off.p; a.vs_cnt = b.d_vs_cnt.p; a.vs_data = b.d_vs_data.p;
    a.vs_len = (int)c.vsrc_wave.data.size();
    a.is_kind = b.d_is_kind.p; a.is_off = b.d_is_off.p; a.is_cnt = b.d_is_cnt.p; a.is_data = b.d_is_data.p;
    a.is_len = (int)c.isrc_wave.data.size();
    a.X = X.p; a.Xc = Xc.p; a.contrib = contrib.p;
    a.Qp = Qp.p; a.Qp2 = Qp2.p; a.dQp = dQp.p; a.hmaxc = hmaxc.p; a.floor_ = floor_.p;
    a.Vpred = Vpred.p; a.Vmax = Vmax.p; a.hist = hist.p; a.vs = vs.p; a.is = is.p;
    a.rep = rep.p;
    a.tout = tout.p; a.Vout = Vout.p; a.Iout = Iout.p; a.max_steps = max_steps;
    a.bar_count = bar.p; a.bar_gen = bar.p + 1; a.active = ctl.p; a.err = ctl.p + 2;
    a.max_ticks = (long long)(16LL * max_steps + 1000) * (itl + 2);
    a.ticks_out = ticks.p;
    a.phase_cycles = pcyc.p;
    a.n_coop_units = b.n_coop_units;
    a.coop_stride = coop_stride;
    // the exchange slots of the evaluation phase and the per-warp workspaces of
    // the replica phase share the dynamic shared memory (grid barriers between);
    // the staged gather lists follow, for the whole launch
    const size_t phase_bytes = (std::max(ws_bytes, b.n_coop_units ? coop_bytes : (size_t)0) + 15) & ~(size_t)15;
    a.n_csr_src = (int)b.d_csr_jr.n;
    a.n_res_src = (int)b.d_res_rr.n;
    const size_t sbytes = stage_bytes(c.nnz, a.n_csr_src, std::max(nu, 0), a.n_res_src);
    a.ws_sc = ws_sc;
    a.stage = (sbytes <= 48 * 1024 && phase_bytes + sbytes <= smem_limit) ? 1 : 0;
    a.stage_off = (long long)phase_bytes;
    const size_t smem = phase_bytes + (a.stage ? sbytes : 0);
    VGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, BATCH_THREADS, smem));
    batch_require(per_sm >= 1, "batched transient: the kernel does not fit on an SM");
    // about two warps of work per CTA, at most one CTA per SM (a cooperative launch)
    const long long want_warps = std::max<long long>((b.n_items + 31) / 32, (long long)R);
    int grid = (int)std::min<long long>((long long)sms, (want_warps + 1) / 2);
    grid = std::max(grid, 1);
    void* args[] = {&a};
    cudaEvent_t e0, e1;
    VGB_CUDA(cudaEventCreate(&e0));
    VGB_CUDA(cudaEventCreate(&e1));
    VGB_CUDA(cudaEventRecord(e0, s));
    const cudaError_t le =
        cudaLaunchCooperativeKernel((void*)batch_kernel, dim3(grid), dim3(BATCH_THREADS), args, smem, s);
    VGB_CUDA(cudaEventRecord(e1, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (le != cudaSuccess) throw Error(VGB_ERR_CUDA, std::string("batched transient launch: ") + cudaGetErrorString(le));
    VGB_CUDA(cudaGetLastError());
    b.run_ms = ms;
    int hctl[3];
    VGB_CUDA(cudaMemcpy(hctl, ctl.p, sizeof(hctl), cudaMemcpyDeviceToHost));
    VGB_CUDA(cudaMemcpy(&b.ticks, ticks.p, sizeof(long long), cudaMemcpyDeviceToHost));
    VGB_CUDA(cudaMemcpy(b.phase_cycles, pcyc.p, sizeof(b.phase_cycles), cudaMemcpyDeviceToHost));
    if (hctl[2] & DEV_ERR_TIMEOUT) throw Error(VGB_ERR_TIMEOUT, "batched transient: grid barrier timed out");
    // results, replica-major
    VGB_CUDA(cudaMemcpy(hr.data(), rep.p, sizeof(BRep) * R, cudaMemcpyDeviceToHost));
    if (times) VGB_CUDA(cudaMemcpy(times, tout.p, sizeof(double) * (size_t)R * max_steps, cudaMemcpyDeviceToHost));
    if (V_out)
        VGB_CUDA(cudaMemcpy(V_out, Vout.p, sizeof(double) * (size_t)R * max_steps * n_ext, cudaMemcpyDeviceToHost));
    if (I_out)
        VGB_CUDA(cudaMemcpy(I_out, Iout.p, sizeof(double) * (size_t)R * max_steps * nvo, cudaMemcpyDeviceToHost));
    if (stats)
        for (int r = 0; r < R; ++r) {
            const BRep& q = hr[r];
            double* st = stats + (size_t)r * 8;
            st[0] = q.step_idx;
            st[1] = q.rejected;
            st[2] = (double)q.total_nr;
            st[3] = q.min_dt_used;
            st[4] = q.max_dt_used;
            st[5] = ms;
            st[6] = q.nr_fail_count;
            st[7] = q.pivot_err;
        }
    int unfinished = 0;
    for (const BRep& q : hr) unfinished += q.state != RS_DONE;
    if (unfinished)
        throw Error(VGB_ERR_STATE, "batched transient: " + std::to_string(unfinished) +
                                       " replica(s) did not finish within the tick bound");
}

} // namespace vgb

using namespace vgb;

template <class F>
static int batch_guard(Batch* b, F&& fn) {
    try {
        fn();
        return VGB_OK;
    } catch (const Error& e) {
        if (b) b->last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        if (b) b->last_error = e.what();
        return VGB_ERR_INVALID;
    }
}

extern "C" {

int vgb_batch_create(void* h, int n_rep, void** out) {
    Circuit* c = static_cast<Circuit*>(h);
    if (!c || !out || n_rep < 1) {
        if (c) c->last_error = "vgb_batch_create: a circuit, an output handle and n_rep >= 1 are required";
        return VGB_ERR_INVALID;
    }
    auto* b = new Batch();
    b->c = c;
    b->n_rep = n_rep;
    const int code = batch_guard(b, [&] { batch_build(*b); });
    if (code != VGB_OK) {
        c->last_error = b->last_error;
        delete b;
        return code;
    }
    *out = b;
    return VGB_OK;
}

int vgb_batch_destroy(void* bh) {
    delete static_cast<Batch*>(bh);
    return VGB_OK;
}

const char* vgb_batch_last_error(void* bh) {
    Batch* b = static_cast<Batch*>(bh);
    return b ? b->last_error.c_str() : "null batch handle";
}

int vgb_batch_set_group(void* bh, int group, int n_varying, const int* varying_idx, const double* values,
                        const double* temperatures) {
    Batch* b = static_cast<Batch*>(bh);
    if (!b) return VGB_ERR_INVALID;
    return batch_guard(b, [&] {
        Circuit& c = *b->c;
        batch_require(group >= 0 && group < (int)c.groups.size(), "group out of range");
        const Group& G = c.groups[group];
        batch_require(n_varying >= 0 && n_varying <= G.np, "n_varying out of range");
        batch_require(n_varying == 0 || (varying_idx && values), "varying_idx and values are required");
        std::vector<int> vidx(G.np, -1);
        for (int v = 0; v < n_varying; ++v) {
            batch_require(varying_idx[v] >= 0 && varying_idx[v] < G.np, "varying parameter index out of range");
            batch_require(vidx[varying_idx[v]] < 0, "varying parameter listed twice");
            vidx[varying_idx[v]] = v;
        }
        const size_t nvals = (size_t)n_varying * G.n_dev * b->n_rep;
        b->vidx[group] = vidx;
        if (nvals) b->vvals[group].assign(values, values + nvals);
        else b->vvals[group].clear();
        if (temperatures) b->temps[group].assign(temperatures, temperatures + (size_t)G.n_dev * b->n_rep);
        else b->temps[group].clear();
    });
}

int vgb_batch_set_sources(void* bh, int is_current, const double* data) {
    Batch* b = static_cast<Batch*>(bh);
    if (!b) return VGB_ERR_INVALID;
    return batch_guard(b, [&] {
        Circuit& c = *b->c;
        const Sources& S = is_current ? c.isrc_wave : c.vsrc_wave;
        std::vector<double>& dst = is_current ? b->is_data : b->vs_data;
        if (S.data.empty()) return;
        batch_require(data != nullptr, "data is required");
        dst.assign(data, data + (size_t)b->n_rep * S.data.size());
    });
}

int vgb_batch_transient(void* bh, const double* cfg, const double* X0, const double* Q0, const double* I0,
                        const double* maxc0, double* times, double* V_out, double* I_out, double* stats) {
    Batch* b = static_cast<Batch*>(bh);
    if (!b) return VGB_ERR_INVALID;
    return batch_guard(b, [&] {
        batch_require(cfg != nullptr, "cfg is required");
        batch_run(*b, cfg, X0, Q0, I0, maxc0, times, V_out, I_out, stats);
    });
}

int vgb_batch_set_coop(void* bh, int enable) {
    Batch* b = static_cast<Batch*>(bh);
    if (!b) return VGB_ERR_INVALID;
    if (enable < 0 || enable > 2) {
        b->last_error = "vgb_batch_set_coop: 0 (never), 1 (when it fits one group per SM) or 2 (always)";
        return VGB_ERR_INVALID;
    }
    b->coop = enable;
    return VGB_OK;
}

int vgb_batch_info(void* bh, double* out) {
    Batch* b = static_cast<Batch*>(bh);
    if (!b || !out) return VGB_ERR_INVALID;
    out[0] = b->run_ms;
    out[1] = (double)b->ticks;
    out[2] = (double)b->n_items;
    out[3] = (double)b->n_contrib;
    for (int q = 0; q < 8; ++q) out[4 + q] = (double)b->phase_cycles[q];
    out[12] = (double)b->n_coop_units;
    for (int q = 8; q < 12; ++q) out[5 + q] = (double)b->phase_cycles[q];
    return VGB_OK;
}

}  // extern "C"
