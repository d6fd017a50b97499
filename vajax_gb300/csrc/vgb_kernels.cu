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

__global__ void assemble_kernel(AssembleArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_aug = a.n_unk + a.n_vsrc;
    if (t < a.nnz) {
        double s = 0.0;
        const int e0 = a.csr_src_ptr[t], e1 = a.csr_src_ptr[t + 1];
        for (int e = e0; e < e1; ++e) s += a.contrib[a.csr_src[e]];
        if (a.csr_diag[t]) s += a.gdiag;
        s += a.csr_const[t];
        a.csr_vals[t] = s;
        return;
    }
    const int r = t - a.nnz;
    if (r >= n_aug) return;
    double fn;
    double tol;
    if (r < a.n_unk) {
        double fr = 0.0, q = 0.0, mc = 0.0;
        const int e0 = a.res_src_ptr[r], e1 = a.res_src_ptr[r + 1];
        for (int e = e0; e < e1; ++e) {
            double v = nan0(a.contrib[a.res_src[e]]);
            fr += v;
            mc = fmax(mc, fabs(v));
            q += nan0(a.contrib[a.rq_src[e]]);
        }
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

void launch_assemble(const AssembleArgs& a, cudaStream_t s) {
    const long long total = (long long)a.nnz + a.n_unk + a.n_vsrc;
    if (total == 0) return;
    assemble_kernel<<<ceil_div(total, 256), 256, 0, s>>>(a);
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
// Static-pivot sparse LU: sync-free left-looking factorisation.
//
// Column j (in elimination order) is owned by one warp.  Its values start as
// the permuted A entries; for each k in the U pattern of column j (ascending)
// the warp waits until column k is final, reads u = U(k, j) and applies
// x(i) -= L(i, k) * u for every row i of L(:, k) through a precomputed map of
// positions inside column j.  Columns are claimed in increasing order from a
// global counter, so every dependency (k < j) is already owned by a running
// warp and the waits always end; each wait is bounded anyway.
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
    const double* A;
    int* done;
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

template <typename T>
__global__ void __launch_bounds__(256) lu_factor_kernel(LUArgs a, T* vals) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int j = 0;
        if (lane == 0) j = atomicAdd(a.counter, 1);
        j = __shfl_sync(0xffffffffu, j, 0);
        if (j >= a.n) return;
        const long long s0 = a.col_ptr[j], s1 = a.col_ptr[j + 1];
        const int nu = a.nU[j];
        for (long long s = s0 + lane; s < s1; s += 32) {
            const int e = a.f2a[s];
            vals[s] = e >= 0 ? (T)a.A[e] : (T)0;
        }
        __syncwarp();
        const long long ub = a.ustart[j];
        bool ok = true;
        for (int t = 0; t < nu; ++t) {
            const int k = a.rows[s0 + t];
            if (lane == 0) ok = wait_flag(a.done + k, a.epoch, a.abort_flag, a.err, a.spin_limit);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            __syncwarp();
            const T u = vals[s0 + t];
            const long long kL = a.col_ptr[k] + a.nU[k] + 1;
            const long long m0 = a.umap_ptr[ub + t], m1 = a.umap_ptr[ub + t + 1];
            if (u != (T)0) {
                for (long long m = m0 + lane; m < m1; m += 32) vals[s0 + a.umap[m]] -= vals[kL + (m - m0)] * u;
            }
            __syncwarp();
        }
        T piv = vals[s0 + nu];
        if (piv == (T)0 || !isfinite((double)piv)) {
            if (lane == 0) atomicOr(a.err, DEV_ERR_PIVOT);
            piv = (T)1e-30;
            if (lane == 0) vals[s0 + nu] = piv;
        }
        for (long long s = s0 + nu + 1 + lane; s < s1; s += 32) vals[s] = vals[s] / piv;
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
    const int* brow;         // forward: A-row of permuted row
    const int* q;            // backward: original column of permuted column
    int* done;
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

// L y = P b (unit lower triangular), row-oriented, one warp per row.
template <typename T>
__global__ void __launch_bounds__(256) lu_fwd_kernel(SolveArgs a, const T* __restrict__ vals,
                                                     const double* __restrict__ b, T* y) {
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
            y[i] = (T)b[a.brow[i]] - acc;
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

static int persistent_blocks() {
    static int blocks = 0;
    if (!blocks) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = std::max(1, sms) * 4;
    }
    return blocks;
}

static unsigned spin_limit_default() { return 1u << 24; }

void lu_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s) {
    SparseLU& L = c.lu;
    if (L.n == 0) return;
    L.epoch++;
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
    LUArgs a{};
    a.n = L.n;
    a.col_ptr = L.d_col_ptr.p;
    a.nU = L.d_nU.p;
    a.rows = L.d_rows.p;
    a.f2a = L.d_f2a.p;
    a.ustart = L.d_ustart.p;
    a.umap_ptr = L.d_umap_ptr.p;
    a.umap = L.d_umap.p;
    a.A = A;
    a.done = L.d_done.p;
    a.counter = L.d_counters.p;
    a.abort_flag = L.d_counters.p + 3;
    a.err = &c.d_status.p->dev_err;
    a.epoch = L.epoch;
    a.spin_limit = spin_limit_default();
    const int blocks = std::min(persistent_blocks(), ceil_div((long long)L.n * 32, 256));
    if (fp32) lu_factor_kernel<float><<<blocks, 256, 0, s>>>(a, L.d_vals32.p);
    else lu_factor_kernel<double><<<blocks, 256, 0, s>>>(a, L.d_vals64.p);
    VGB_CUDA(cudaGetLastError());
}

template <typename T>
static void lu_solve_once(Circuit& c, const T* vals, const double* rhs, double* x, T* ybuf, T* xbuf, cudaStream_t s) {
    SparseLU& L = c.lu;
    L.epoch++;
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
    const int blocks = std::min(persistent_blocks(), ceil_div((long long)L.n * 32, 256));
    SolveArgs f{};
    f.n = L.n;
    f.ptr = L.d_lrow_ptr.p;
    f.pos = L.d_lrow_pos.p;
    f.col = L.d_lrow_col.p;
    f.col_ptr = L.d_col_ptr.p;
    f.nU = L.d_nU.p;
    f.brow = L.d_brow.p;
    f.q = L.d_q.p;
    f.done = L.d_done.p + L.n;
    f.counter = L.d_counters.p + 1;
    f.abort_flag = L.d_counters.p + 3;
    f.err = &c.d_status.p->dev_err;
    f.epoch = L.epoch;
    f.spin_limit = spin_limit_default();
    lu_fwd_kernel<T><<<blocks, 256, 0, s>>>(f, vals, rhs, ybuf);
    SolveArgs b = f;
    b.ptr = L.d_urow_ptr.p;
    b.pos = L.d_urow_pos.p;
    b.col = L.d_urow_col.p;
    b.done = L.d_done.p + 2 * (size_t)L.n;
    b.counter = L.d_counters.p + 2;
    lu_bwd_kernel<T><<<blocks, 256, 0, s>>>(b, vals, ybuf, xbuf, x);
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
    if (!fp32) {
        lu_solve_once<double>(c, L.d_vals64.p, rhs, x, (double*)c.d_work.p, (double*)c.d_work2.p, s);
        return;
    }
    float* ybuf = (float*)c.d_work.p;
    float* xbuf = ybuf + n;
    lu_solve_once<float>(c, L.d_vals32.p, rhs, x, ybuf, xbuf, s);
    double* r = c.d_work2.p;
    double* d = c.d_work2.p + n;
    for (int k = 0; k < sweeps; ++k) {
        residual_kernel<<<ceil_div((long long)n * 32, 256), 256, 0, s>>>(n, c.d_indptr.p, c.d_indices.p, A, rhs, x, r);
        lu_solve_once<float>(c, L.d_vals32.p, r, d, ybuf, xbuf, s);
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
