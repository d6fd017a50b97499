// Device kernels of the transient Newton path.
#include <cuda/atomic>

#include "vgb_kernels.cuh"

namespace vgb {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ int ld_acquire(const int* p) {
    return cuda::atomic_ref<const int, cuda::thread_scope_device>(*p).load(cuda::memory_order_acquire);
}
__device__ __forceinline__ void st_release(int* p, int v) {
    cuda::atomic_ref<int, cuda::thread_scope_device>(*p).store(v, cuda::memory_order_release);
}

// Bounded wait for a dependency flag.  Gives up after `limit` polls, records
// DEV_ERR_TIMEOUT and raises the abort flag so every other waiter stops too.
__device__ __forceinline__ bool wait_flag(const int* flag, int epoch, int* abort_flag, int* err, unsigned limit) {
    unsigned it = 0;
    while (ld_acquire(flag) != epoch) {
        if (*(volatile int*)abort_flag) return false;
        if (++it > limit) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            atomicExch(abort_flag, 1);
            return false;
        }
        if (it > 64) __nanosleep(64);
    }
    return true;
}

// ---------------------------------------------------------------------------
// Assembly: CSR values + residual vectors + residual convergence test.
// Reference: mna_builder.py:759-1076 (stamping and _build_residual),
// solver_factories.py:271-281 (VACASK-style residual check).
// ---------------------------------------------------------------------------

// Finish one node row or branch row from its gathered sums (shared by both assembly kernels).
__device__ __forceinline__ void finish_row(const AssembleArgs& a, int r, double fr, double q, double mc) {
    double fn;
    double tol;
    if (r < a.n_unk) {
        for (int e = a.ni_ptr[r]; e < a.ni_ptr[r + 1]; ++e) {
            int k = a.ni_idx[e];
            double v = k > 0 ? a.isrc_vals[k - 1] : -a.isrc_vals[-k - 1];
            v = nan0(v);
            fr += v;
            mc = fmax(mc, fabs(v));
        }
        a.fres[r] = fr;
        for (int e = a.nb_ptr[r]; e < a.nb_ptr[r + 1]; ++e) {
            int k = a.nb_idx[e];
            fr += k > 0 ? a.X[a.n_nodes + k - 1] : -a.X[a.n_nodes - k - 1];
        }
        fn = fr + a.c0 * q + a.c1 * a.Q_prev[r] + a.d1 * a.dQdt_prev[r] + a.c2 * a.Q_prev2[r] +
             a.gdiag * a.X[r + 1];
        a.Q[r] = q;
        a.maxc[r] = mc;
        tol = fmax(mc * a.reltol, a.res_tol_floor[r]);
    } else {
        const int k = r - a.n_unk;
        fn = a.X[a.vsrc_p[k]] - a.X[a.vsrc_n[k]] - a.vsrc_vals[k];
        tol = a.vntol;
    }
    a.f[r] = fn;
    if (!isfinite(fn)) atomicOr(&a.st->nonfinite, 1);
    if (a.conv_mask[r]) {
        double af = fabs(fn);
        if (!(af < tol)) atomicAnd(&a.st->res_ok, 0);
        atomic_max_nonneg(&a.st->max_f, af != af ? INFINITY : af);
    }
}

// One thread per CSR entry / row with a short gather list.  Entries whose
// list is long (the supply rails collect one term per connected device) are
// skipped here and summed by assemble_heavy_kernel with a whole block each.
__global__ void assemble_kernel(AssembleArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_aug = a.n_unk + a.n_vsrc;
    if (t < a.nnz) {
        const int e0 = a.csr_src_ptr[t], e1 = a.csr_src_ptr[t + 1];
        if (e1 - e0 > HEAVY_LIST) return;
        double s = 0.0;
        for (int e = e0; e < e1; ++e) s += a.contrib[a.csr_src[e]];
        if (a.csr_diag[t]) s += a.gdiag;
        s += a.csr_const[t];
        a.csr_vals[t] = s;
        return;
    }
    const int r = t - a.nnz;
    if (r >= n_aug) return;
    double fr = 0.0, q = 0.0, mc = 0.0;
    if (r < a.n_unk) {
        const int e0 = a.res_src_ptr[r], e1 = a.res_src_ptr[r + 1];
        if (e1 - e0 > HEAVY_LIST) return;
        for (int e = e0; e < e1; ++e) {
            double v = nan0(a.contrib[a.res_src[e]]);
            fr += v;
            mc = fmax(mc, fabs(v));
            q += nan0(a.contrib[a.rq_src[e]]);
        }
    }
    finish_row(a, r, fr, q, mc);
}

// One block per heavy CSR entry or heavy node row; fixed-order block reduction.
__global__ void __launch_bounds__(256) assemble_heavy_kernel(AssembleArgs a) {
    __shared__ double s_sum[256], s_q[256], s_max[256];
    const int b = blockIdx.x;
    const bool is_csr = b < a.n_heavy_csr;
    const int item = is_csr ? a.heavy_csr[b] : a.heavy_row[b - a.n_heavy_csr];
    const int e0 = is_csr ? a.csr_src_ptr[item] : a.res_src_ptr[item];
    const int e1 = is_csr ? a.csr_src_ptr[item + 1] : a.res_src_ptr[item + 1];
    double s = 0.0, q = 0.0, m = 0.0;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        if (is_csr) {
            s += a.contrib[a.csr_src[e]];
        } else {
            double v = nan0(a.contrib[a.res_src[e]]);
            s += v;
            m = fmax(m, fabs(v));
            q += nan0(a.contrib[a.rq_src[e]]);
        }
    }
    s_sum[threadIdx.x] = s;
    s_q[threadIdx.x] = q;
    s_max[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s_sum[threadIdx.x] += s_sum[threadIdx.x + o];
            s_q[threadIdx.x] += s_q[threadIdx.x + o];
            s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    if (is_csr) {
        double v = s_sum[0];
        if (a.csr_diag[item]) v += a.gdiag;
        v += a.csr_const[item];
        a.csr_vals[item] = v;
    } else {
        finish_row(a, item, s_sum[0], s_q[0], s_max[0]);
    }
}

void launch_assemble(const AssembleArgs& a, cudaStream_t s) {
    const long long total = (long long)a.nnz + a.n_unk + a.n_vsrc;
    if (total == 0) return;
    assemble_kernel<<<ceil_div(total, 256), 256, 0, s>>>(a);
    if (a.n_heavy_csr + a.n_heavy_row) assemble_heavy_kernel<<<a.n_heavy_csr + a.n_heavy_row, 256, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// Newton update (solver_factories.py:287-313)
// ---------------------------------------------------------------------------

__global__ void status_reset_kernel(NRStatus* st) {
    st->res_ok = 1;
    st->delta_ok = 1;
    st->max_f = 0;
    st->max_dv = 0;
    st->max_delta = 0;
    st->lte_norm = 0;
    st->nonfinite = 0;
}

void launch_status_reset(NRStatus* st, cudaStream_t s) { status_reset_kernel<<<1, 1, 0, s>>>(st); }

__global__ void nr_reduce_kernel(NRUpdateArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_aug) return;
    const double d = a.delta[i];
    const bool is_v = i < a.n_unk;
    const double conv = is_v ? d * a.damping : d;
    const double tol = fmax(fabs(a.X[i + 1]) * a.reltol, is_v ? a.vntol : a.abstol);
    if (!(fabs(conv) < tol)) atomicAnd(&a.st->delta_ok, 0);
    const double ad = fabs(d);
    atomic_max_nonneg(&a.st->max_delta, ad != ad ? INFINITY : ad);
    if (is_v) atomic_max_nonneg(&a.st->max_dv, ad != ad ? INFINITY : ad);
}

__global__ void nr_apply_kernel(NRUpdateArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_aug) return;
    const double d = a.delta[i];
    if (i < a.n_unk) {
        const double max_dv = __longlong_as_double((long long)a.st->max_dv);
        const double scale = fmin(1.0, a.max_step / fmax(max_dv, 1e-30));
        a.X[i + 1] += d * scale * a.damping;
    } else {
        a.X[i + 1] += d;
    }
}

void launch_nr_reduce(const NRUpdateArgs& a, cudaStream_t s) {
    if (a.n_aug) nr_reduce_kernel<<<ceil_div(a.n_aug, 256), 256, 0, s>>>(a);
}
void launch_nr_apply(const NRUpdateArgs& a, cudaStream_t s) {
    if (a.n_aug) nr_apply_kernel<<<ceil_div(a.n_aug, 256), 256, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// Static-pivot sparse LU of the block M: sync-free left-looking factorisation.
//
// Column j (in elimination order) is owned by one warp.  The warp first waits,
// lanes in parallel, until every column k in the U pattern of column j is
// final; it then stages the column (the permuted A entries) and every update
// operand L(i, k) with its target position in shared memory in one bulk
// load, and runs the sequential part, x(i) -= L(i, k) * x(k) for k ascending,
// entirely on chip.  Columns are claimed in increasing order from a global
// counter, so every dependency (k < j) is owned by a warp that is already
// running and the waits always end; each wait is bounded anyway.  Columns too
// large for the shared-memory stage run the same loop on global memory.
// ---------------------------------------------------------------------------

struct LUArgs {
    int n;
    const long long* col_ptr;
    const int* nU;
    const int* rows;
    const int* f2a;
    const long long* ustart;
    const long long* umap_ptr;
    const int* umap;
    const long long* ukl;
    const double* A;
    int* done;
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

constexpr int LU_WARPS = 4;
constexpr int CAP_X = 256;   // column entries staged per warp
constexpr int CAP_U = 512;   // update operands staged per warp
constexpr int CAP_T = 128;   // U entries staged per warp

template <typename T>
struct LUSmem {
    T x[LU_WARPS][CAP_X];
    T lv[LU_WARPS][CAP_U];
    int um[LU_WARPS][CAP_U];
    int uptr[LU_WARPS][CAP_T + 1];
};

template <typename T>
__global__ void __launch_bounds__(LU_WARPS * 32) lu_factor_kernel(LUArgs a, T* vals) {
    __shared__ LUSmem<T> sm;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    T* x = sm.x[w];
    T* lv = sm.lv[w];
    int* um = sm.um[w];
    int* uptr = sm.uptr[w];
    while (true) {
        int j = 0;
        if (lane == 0) j = atomicAdd(a.counter, 1);
        j = __shfl_sync(0xffffffffu, j, 0);
        if (j >= a.n) return;
        const long long s0 = a.col_ptr[j], s1 = a.col_ptr[j + 1];
        const int len = (int)(s1 - s0);
        const int nu = a.nU[j];
        const long long ub = a.ustart[j];
        const long long M0 = a.umap_ptr[ub], M1 = a.umap_ptr[ub + nu];
        const long long nupd = M1 - M0;
        // 1. dependencies, waited for in parallel
        bool ok = true;
        for (int t = lane; t < nu; t += 32)
            ok = ok && wait_flag(a.done + a.rows[s0 + t], a.epoch, a.abort_flag, a.err, a.spin_limit);
        ok = __all_sync(0xffffffffu, ok);
        const bool fits = len <= CAP_X && nupd <= CAP_U && nu <= CAP_T;
        if (ok && fits) {
            // 2. bulk stage: column values, update pointers, update operands
            for (int s = lane; s < len; s += 32) {
                const int e = a.f2a[s0 + s];
                x[s] = e >= 0 ? (T)a.A[e] : (T)0;
            }
            for (int t = lane; t <= nu; t += 32) uptr[t] = (int)(a.umap_ptr[ub + t] - M0);
            __syncwarp();
            for (int m = lane; m < (int)nupd; m += 32) {
                int lo = 0, hi = nu;  // largest t with uptr[t] <= m
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (uptr[mid] <= m) lo = mid; else hi = mid;
                }
                lv[m] = vals[a.ukl[ub + lo] + (m - uptr[lo])];
                um[m] = a.umap[M0 + m];
            }
            __syncwarp();
            // 3. sequential elimination on chip
            for (int t = 0; t < nu; ++t) {
                const T u = x[t];
                if (u != (T)0)
                    for (int m = uptr[t] + lane; m < uptr[t + 1]; m += 32) x[um[m]] -= lv[m] * u;
                __syncwarp();
            }
            T piv = x[nu];
            if (piv == (T)0 || !isfinite((double)piv)) {
                if (lane == 0) atomicOr(a.err, DEV_ERR_PIVOT);
                piv = (T)1e-30;
                if (lane == 0) x[nu] = piv;
                __syncwarp();
            }
            for (int s = lane; s < len; s += 32) vals[s0 + s] = s > nu ? x[s] / piv : x[s];
        } else if (ok) {
            // large column: same elimination on global memory
            for (int s = lane; s < len; s += 32) {
                const int e = a.f2a[s0 + s];
                vals[s0 + s] = e >= 0 ? (T)a.A[e] : (T)0;
            }
            __syncwarp();
            for (int t = 0; t < nu; ++t) {
                const T u = vals[s0 + t];
                const long long m0 = a.umap_ptr[ub + t], m1 = a.umap_ptr[ub + t + 1];
                const long long kL = a.ukl[ub + t];
                if (u != (T)0)
                    for (long long m = m0 + lane; m < m1; m += 32) vals[s0 + a.umap[m]] -= vals[kL + (m - m0)] * u;
                __syncwarp();
            }
            T piv = vals[s0 + nu];
            if (piv == (T)0 || !isfinite((double)piv)) {
                if (lane == 0) atomicOr(a.err, DEV_ERR_PIVOT);
                piv = (T)1e-30;
                if (lane == 0) vals[s0 + nu] = piv;
            }
            __syncwarp();
            for (long long s = s0 + nu + 1 + lane; s < s1; s += 32) vals[s] = vals[s] / piv;
        }
        __syncwarp();
        __threadfence();
        if (lane == 0) st_release(a.done + j, a.epoch);
    }
}

struct SolveArgs {
    int n;
    const long long* ptr;    // row access pointers
    const long long* pos;    // slot of each entry
    const int* col;          // dependency index of each entry
    const long long* col_ptr;
    const int* nU;
    const int* q;            // backward: B index of permuted column
    int* done;
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

// Right-hand side of the block M: b restricted to M minus the couplings to the
// singletons solved first (x_F = b_F / diag).  Also writes x_F.
template <typename T>
__global__ void lu_pre_kernel(int nM, int nF, const int* brow, const int* pre_ptr, const int* pre_e,
                              const int* pre_f, const int* f_col, const int* f_arow, const int* f_diag_e,
                              const double* A, const double* b, T* rhsM, double* xout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nM) {
        double v = b[brow[i]];
        for (int e = pre_ptr[i]; e < pre_ptr[i + 1]; ++e) {
            const int f = pre_f[e];
            v -= A[pre_e[e]] * (b[f_arow[f]] / A[f_diag_e[f]]);
        }
        rhsM[i] = (T)v;
    } else if (i < nM + nF) {
        const int f = i - nM;
        xout[f_col[f]] = b[f_arow[f]] / A[f_diag_e[f]];
    }
}

// L y = rhs (unit lower triangular), row-oriented, one warp per row.
template <typename T>
__global__ void __launch_bounds__(256) lu_fwd_kernel(SolveArgs a, const T* __restrict__ vals,
                                                     const T* __restrict__ rhs, T* y) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(a.counter, 1);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= a.n) return;
        T acc = 0;
        for (long long e = a.ptr[i] + lane; e < a.ptr[i + 1]; e += 32) {
            const int k = a.col[e];
            if (!wait_flag(a.done + k, a.epoch, a.abort_flag, a.err, a.spin_limit)) break;
            acc += vals[a.pos[e]] * ((volatile T*)y)[k];
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            y[i] = rhs[i] - acc;
            __threadfence();
            st_release(a.done + i, a.epoch);
        }
    }
}

// U x = y, rows processed from the last one upwards.
template <typename T>
__global__ void __launch_bounds__(256) lu_bwd_kernel(SolveArgs a, const T* __restrict__ vals,
                                                     const T* __restrict__ y, T* xs, double* xout) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int c = 0;
        if (lane == 0) c = atomicAdd(a.counter, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= a.n) return;
        const int i = a.n - 1 - c;
        T acc = 0;
        for (long long e = a.ptr[i] + lane; e < a.ptr[i + 1]; e += 32) {
            const int j = a.col[e];
            if (!wait_flag(a.done + j, a.epoch, a.abort_flag, a.err, a.spin_limit)) break;
            acc += vals[a.pos[e]] * ((volatile T*)xs)[j];
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            const T d = vals[a.col_ptr[i] + a.nU[i]];
            const T xi = (y[i] - acc) / d;
            xs[i] = xi;
            xout[a.q[i]] = (double)xi;
            __threadfence();
            st_release(a.done + i, a.epoch);
        }
    }
}

// Singletons solved last: x_c = (b_c - sum_j B(c, j) x_j) / B(c, c), one warp per row.
__global__ void lu_post_kernel(int nL, const int* l_col, const int* l_arow, const int* l_diag_e, const int* l_ptr,
                               const int* l_e, const int* l_x, const double* A, const double* b, double* xout) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nL) return;
    double acc = 0.0;
    for (int e = l_ptr[warp] + lane; e < l_ptr[warp + 1]; e += 32) acc += A[l_e[e]] * xout[l_x[e]];
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) xout[l_col[warp]] = (b[l_arow[warp]] - acc) / A[l_diag_e[warp]];
}

static int persistent_blocks(int per_sm) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        sms = std::max(1, sms);
    }
    return sms * per_sm;
}

static unsigned spin_limit_default() { return 1u << 24; }

void lu_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s) {
    SparseLU& L = c.lu;
    if (L.nM == 0) return;
    L.epoch++;
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
    LUArgs a{};
    a.n = L.nM;
    a.col_ptr = L.d_col_ptr.p;
    a.nU = L.d_nU.p;
    a.rows = L.d_rows.p;
    a.f2a = L.d_f2a.p;
    a.ustart = L.d_ustart.p;
    a.umap_ptr = L.d_umap_ptr.p;
    a.umap = L.d_umap.p;
    a.ukl = L.d_ukl.p;
    a.A = A;
    a.done = L.d_done.p;
    a.counter = L.d_counters.p;
    a.abort_flag = L.d_counters.p + 3;
    a.err = &c.d_status.p->dev_err;
    a.epoch = L.epoch;
    a.spin_limit = spin_limit_default();
    const int threads = LU_WARPS * 32;
    const int blocks = std::min(persistent_blocks(fp32 ? 8 : 5), ceil_div((long long)L.nM * 32, threads));
    if (fp32) lu_factor_kernel<float><<<blocks, threads, 0, s>>>(a, L.d_vals32.p);
    else lu_factor_kernel<double><<<blocks, threads, 0, s>>>(a, L.d_vals64.p);
    VGB_CUDA(cudaGetLastError());
}

template <typename T>
static void lu_solve_once(Circuit& c, const T* vals, const double* A, const double* rhs, double* x, T* rhsM, T* ybuf,
                          T* xbuf, cudaStream_t s) {
    SparseLU& L = c.lu;
    const int nM = L.nM, nF = (int)L.f_col.size(), nL = (int)L.l_col.size();
    if (nM + nF)
        lu_pre_kernel<T><<<ceil_div(nM + nF, 256), 256, 0, s>>>(nM, nF, L.d_brow.p, L.d_pre_ptr.p, L.d_pre_e.p,
                                                                L.d_pre_f.p, L.d_f_col.p, L.d_f_arow.p,
                                                                L.d_f_diag_e.p, A, rhs, rhsM, x);
    if (nM) {
        L.epoch++;
        VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
        const int blocks = std::min(persistent_blocks(8), ceil_div((long long)nM * 32, 256));
        SolveArgs f{};
        f.n = nM;
        f.ptr = L.d_lrow_ptr.p;
        f.pos = L.d_lrow_pos.p;
        f.col = L.d_lrow_col.p;
        f.col_ptr = L.d_col_ptr.p;
        f.nU = L.d_nU.p;
        f.q = L.d_q.p;
        f.done = L.d_done.p + nM;
        f.counter = L.d_counters.p + 1;
        f.abort_flag = L.d_counters.p + 3;
        f.err = &c.d_status.p->dev_err;
        f.epoch = L.epoch;
        f.spin_limit = spin_limit_default();
        lu_fwd_kernel<T><<<blocks, 256, 0, s>>>(f, vals, rhsM, ybuf);
        SolveArgs b = f;
        b.ptr = L.d_urow_ptr.p;
        b.pos = L.d_urow_pos.p;
        b.col = L.d_urow_col.p;
        b.done = L.d_done.p + 2 * (size_t)nM;
        b.counter = L.d_counters.p + 2;
        lu_bwd_kernel<T><<<blocks, 256, 0, s>>>(b, vals, ybuf, xbuf, x);
    }
    if (nL)
        lu_post_kernel<<<ceil_div((long long)nL * 32, 256), 256, 0, s>>>(nL, L.d_l_col.p, L.d_l_arow.p,
                                                                        L.d_l_diag_e.p, L.d_l_ptr.p, L.d_l_e.p,
                                                                        L.d_l_x.p, A, rhs, x);
    VGB_CUDA(cudaGetLastError());
}

// r = rhs - A x   (CSR SpMV, one warp per row)
__global__ void residual_kernel(int n, const int* indptr, const int* indices, const double* A,
                                const double* rhs, const double* x, double* r) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    double acc = 0.0;
    for (int e = indptr[warp] + lane; e < indptr[warp + 1]; e += 32) acc += A[e] * x[indices[e]];
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) r[warp] = rhs[warp] - acc;
}

__global__ void axpy_kernel(int n, const double* d, double* x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += d[i];
}

void lu_solve(Circuit& c, const double* A, const double* rhs, double* x, bool fp32, int sweeps, cudaStream_t s) {
    SparseLU& L = c.lu;
    const int n = L.n;
    if (n == 0) return;
    const int nM = std::max(L.nM, 1);
    if (!fp32) {
        double* rhsM = c.d_work.p;
        double* ybuf = c.d_work.p + nM;
        double* xbuf = c.d_work.p + 2 * (size_t)nM;
        lu_solve_once<double>(c, L.d_vals64.p, A, rhs, x, rhsM, ybuf, xbuf, s);
        return;
    }
    float* rhsM = (float*)c.d_work.p;
    float* ybuf = rhsM + nM;
    float* xbuf = ybuf + nM;
    lu_solve_once<float>(c, L.d_vals32.p, A, rhs, x, rhsM, ybuf, xbuf, s);
    double* r = c.d_work2.p;
    double* d = c.d_work2.p + n;
    for (int k = 0; k < sweeps; ++k) {
        residual_kernel<<<ceil_div((long long)n * 32, 256), 256, 0, s>>>(n, c.d_indptr.p, c.d_indices.p, A, rhs, x, r);
        lu_solve_once<float>(c, L.d_vals32.p, A, r, d, rhsM, ybuf, xbuf, s);
        axpy_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, d, x);
    }
}

// ---------------------------------------------------------------------------
// small vector kernels
// ---------------------------------------------------------------------------

__global__ void negate_kernel(const double* in, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = -in[i];
}
void launch_negate(const double* in, double* out, int n, cudaStream_t s) {
    if (n) negate_kernel<<<ceil_div(n, 256), 256, 0, s>>>(in, out, n);
}

// I_vsource = -f_resist[p-1] (mna.py:compute_vsource_current_from_kcl)
__global__ void vsrc_current_kernel(const double* fres, const int* vsrc_p, double* I, int n_vsrc) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_vsrc) return;
    const int p = vsrc_p[k];
    I[k] = p > 0 ? -fres[p - 1] : 0.0;
}
void launch_vsrc_current(const double* fres, const int* vsrc_p, double* I, int n_vsrc, cudaStream_t s) {
    if (n_vsrc) vsrc_current_kernel<<<ceil_div(n_vsrc, 128), 128, 0, s>>>(fres, vsrc_p, I, n_vsrc);
}

// Source waveforms (vajax/analysis/sources.py:31-105)
__device__ double eval_source(int kind, const double* p, int cnt, double t) {
    if (kind == SRC_DC) return p[0];
    if (kind == SRC_PULSE) {
        // val0, val1, rise, fall, width, period, delay
        const double v0 = p[0], v1 = p[1], r = p[2], f = p[3], w = p[4], per = p[5], d = p[6];
        const double tp = vgb_fmod_floor(t - d, per);
        if (t < d) return v0;
        if (tp < r) return v0 + (v1 - v0) * tp / r;
        if (tp < r + w) return v1;
        if (tp < r + w + f) return v1 - (v1 - v0) * (tp - r - w) / f;
        return v0;
    }
    if (kind == SRC_PWL) {
        // [period, t0, v0, t1, v1, ...] (times already stretched, values scaled)
        const double period = p[0];
        const int np = (cnt - 1) / 2;
        const double* tv = p + 1;
        double tt = t;
        if (period > 0) tt = vgb_fmod_floor(t, period);
        if (tt <= tv[0]) return tv[1];
        if (tt >= tv[2 * (np - 1)]) return tv[2 * (np - 1) + 1];
        int lo = 0, hi = np - 1;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (tv[2 * mid] <= tt) lo = mid; else hi = mid;
        }
        const double t0 = tv[2 * lo], t1 = tv[2 * hi], v0 = tv[2 * lo + 1], v1 = tv[2 * hi + 1];
        const double dt = t1 - t0;
        return dt == 0.0 ? v1 : v0 + (tt - t0) * (v1 - v0) / dt;
    }
    if (kind == SRC_SINE) {
        return p[0] + p[1] * sin(2.0 * 3.141592653589793 * p[2] * t + p[3]);
    }
    return 0.0;
}

__global__ void eval_sources_kernel(const int* kind, const int* off, const int* cnt, const double* data,
                                    int n, double t, double* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = eval_source(kind[k], data + off[k], cnt[k], t);
}
void launch_eval_sources(const Sources& src, int n, double t, double* out, cudaStream_t s) {
    if (n) eval_sources_kernel<<<ceil_div(n, 128), 128, 0, s>>>(src.d_kind.p, src.d_off.p, src.d_cnt.p,
                                                                src.d_data.p, n, t, out);
}

} // namespace vgb
