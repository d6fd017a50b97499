// Device kernels of the transient Newton path.
#include <cuda/atomic>

#include "vgb_kernels.cuh"
#include "vgb_math.cuh"
#include "vgb_sources.cuh"

namespace vgb {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// The same maximum, one atomic per group of lanes that reach the call together:
// the non-negative doubles compare as their bit patterns, whose maximum is
// taken exactly as the maximum of the high words and then of the low words
// among the lanes that hold it.  Tens of thousands of same-address atomics per
// Newton iteration (one per row) serialised at L2.
__device__ __forceinline__ void warp_max_nonneg(unsigned long long* addr, double v) {
    const unsigned mask = __activemask();
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(b >> 32);
    const unsigned mh = __reduce_max_sync(mask, hi);
    const unsigned ml = __reduce_max_sync(mask, hi == mh ? (unsigned)b : 0u);
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) atomicMax(addr, ((unsigned long long)mh << 32) | ml);
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
        const double c0 = a.k[0], c1 = a.k[1], d1 = a.k[2], c2 = a.k[3], gshunt = a.k[4];
        fn = fr + c0 * q + c1 * a.Q_prev[r] + d1 * a.dQdt_prev[r] + c2 * a.Q_prev2[r] + (a.gmin + gshunt) * a.X[r + 1];
        if (a.shunt_ref) fn -= gshunt * a.shunt_ref[r];
        a.Q[r] = q;
        a.maxc[r] = mc;
        tol = fmax(mc * a.reltol, a.res_tol_floor[r]);
    } else {
        const int k = r - a.n_unk;
        fn = a.X[a.vsrc_p[k]] - a.X[a.vsrc_n[k]] - a.vsrc_vals[k];
        tol = a.vntol;
    }
    a.f[r] = fn;
    // NOI rows (mask 2) are replaced by an identity row before the solve, so their
    // residual (a 1e40 conductance in PSP103) neither stops nor enters the test.
    // The flags and the maximum go out once per group of lanes here together.
    const int cm = a.conv_mask[r];
    const double af = fabs(fn);
    const bool nonfin = cm != 2 && !isfinite(fn);
    const bool bad = cm == 1 && !(af < tol);
    const unsigned mask = __activemask();
    const bool lead = (int)(threadIdx.x & 31) == __ffs(mask) - 1;
    const bool any_nonfin = __any_sync(mask, nonfin), any_bad = __any_sync(mask, bad);
    if (lead && any_nonfin) atomicOr(&a.st->nonfinite, 1);
    if (lead && any_bad) atomicAnd(&a.st->res_ok, 0);
    warp_max_nonneg(&a.st->max_f, cm == 1 ? (af != af ? INFINITY : af) : 0.0);
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
        // several entries' index and value loads in flight; the sum keeps list order
#pragma unroll 4
        for (int e = e0; e < e1; ++e) s += a.contrib[a.csr_src[e]];
        if (a.csr_diag[t]) s += a.gmin + a.k[4];
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
#pragma unroll 4
        for (int e = e0; e < e1; ++e) {
            double v = nan0(a.contrib[a.res_src[e]]);
            fr += v;
            mc = fmax(mc, fabs(v));
            q += nan0(a.contrib[a.rq_src[e]]);
        }
    }
    finish_row(a, r, fr, q, mc);
}

// Heavy CSR entries and node rows: one block per HEAVY_CHUNK-entry chunk
// reduces it with a fixed tree, then one thread per item adds its chunks in
// order, so the sums are deterministic.
constexpr int HEAVY_THREADS = 256;
__global__ void __launch_bounds__(HEAVY_THREADS) assemble_heavy_kernel(AssembleArgs a) {
    __shared__ double s_sum[HEAVY_THREADS], s_q[HEAVY_THREADS], s_max[HEAVY_THREADS];
    const int ch = blockIdx.x;
    const int it = a.hchunk_item[ch];
    const bool is_csr = it < a.n_heavy_csr;
    double s = 0.0, q = 0.0, m = 0.0;
#pragma unroll 4
    for (int e = a.hchunk_lo[ch] + threadIdx.x; e < a.hchunk_hi[ch]; e += HEAVY_THREADS) {
        if (is_csr) {
            s += a.contrib[a.csr_src[e]];
        } else {
            const double v = nan0(a.contrib[a.res_src[e]]);
            s += v;
            m = fmax(m, fabs(v));
            q += nan0(a.contrib[a.rq_src[e]]);
        }
    }
    s_sum[threadIdx.x] = s;
    s_q[threadIdx.x] = q;
    s_max[threadIdx.x] = m;
    __syncthreads();
    for (int o = HEAVY_THREADS / 2; o; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s_sum[threadIdx.x] += s_sum[threadIdx.x + o];
            s_q[threadIdx.x] += s_q[threadIdx.x + o];
            s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.hpart[ch] = s_sum[0];
        a.hpart[a.n_hchunk + ch] = s_q[0];
        a.hpart[2 * a.n_hchunk + ch] = s_max[0];
    }
}

__global__ void assemble_heavy_finish_kernel(AssembleArgs a) {
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= a.n_heavy_csr + a.n_heavy_row) return;
    double s = 0.0, q = 0.0, m = 0.0;
    for (int ch = a.hitem_ptr[it]; ch < a.hitem_ptr[it + 1]; ++ch) {
        s += a.hpart[ch];
        q += a.hpart[a.n_hchunk + ch];
        m = fmax(m, a.hpart[2 * a.n_hchunk + ch]);
    }
    if (it < a.n_heavy_csr) {
        const int item = a.heavy_csr[it];
        if (a.csr_diag[item]) s += a.gmin + a.k[4];
        s += a.csr_const[item];
        a.csr_vals[item] = s;
    } else {
        finish_row(a, a.heavy_row[it - a.n_heavy_csr], s, q, m);
    }
}

void launch_assemble(const AssembleArgs& a, cudaStream_t s) {
    const long long total = (long long)a.nnz + a.n_unk + a.n_vsrc;
    if (total == 0) return;
    assemble_kernel<<<ceil_div(total, 256), 256, 0, s>>>(a);
    if (a.n_heavy_csr + a.n_heavy_row) {
        assemble_heavy_kernel<<<a.n_hchunk, HEAVY_THREADS, 0, s>>>(a);
        assemble_heavy_finish_kernel<<<ceil_div(a.n_heavy_csr + a.n_heavy_row, 64), 64, 0, s>>>(a);
    }
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
    bool bad = false;
    double md = 0.0, mv = 0.0;
    if (i < a.n_aug) {
        const double d = a.delta[i];
        const bool is_v = i < a.n_unk;
        const double conv = is_v ? d * a.damping : d;
        const double tol = fmax(fabs(a.X[i + 1]) * a.reltol, is_v ? a.vntol : a.abstol);
        bad = !(fabs(conv) < tol);
        const double ad = fabs(d);
        md = ad != ad ? INFINITY : ad;
        if (is_v) mv = md;
    }
    // one atomic per warp (the maxima are exact, so the grouping changes nothing)
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicAnd(&a.st->delta_ok, 0);
    warp_max_nonneg(&a.st->max_delta, md);
    warp_max_nonneg(&a.st->max_dv, mv);
}

__global__ void nr_apply_kernel(NRUpdateArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_aug) return;
    const double d = a.delta[i];
    if (i < a.n_unk) {
        const double max_dv = __longlong_as_double((long long)a.st->max_dv);
        const double scale = fmin(1.0, a.max_step / fmax(max_dv, 1e-30));
        double dv = d * scale * a.damping;
        if (a.node_limit > 0.0) dv = fmin(fmax(dv, -a.node_limit), a.node_limit);
        a.X[i + 1] += dv;
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
// Static-pivot sparse LU: singletons around the multifrontal block M.
//
// B = P_r A (voltage-source transversal).  Rows of B that hold only their
// diagonal are solved first (x_F = b_F / diag), the block M is factorised by
// the multifrontal kernels (vgb_frontal.cu), and rows whose column holds only
// the diagonal are solved last from their own row.
// ---------------------------------------------------------------------------

// Right-hand side of the block M: b restricted to M minus the couplings to the
// singletons solved first (x_F = b_F / diag).  Also writes x_F.
// With the scaling of a weighted matching (rscale non-null) the block M is
// factorised as diag(r) M diag(s): its right-hand side is scaled by r here and
// its solution by s when the backward solve writes it.
template <typename T>
__global__ void lu_pre_kernel(int nM, int nF, const int* brow, const int* pre_ptr, const int* pre_e,
                              const int* pre_f, const int* f_col, const int* f_arow, const int* f_diag_e,
                              const double* A, const double* b, const double* rscale, T* rhsM, double* xout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nM) {
        const int ra = brow[i];
        double v = b[ra];
        for (int e = pre_ptr[i]; e < pre_ptr[i + 1]; ++e) {
            const int f = pre_f[e];
            v -= A[pre_e[e]] * (b[f_arow[f]] / A[f_diag_e[f]]);
        }
        if (rscale) v *= rscale[ra];
        rhsM[i] = (T)v;
    } else if (i < nM + nF) {
        const int f = i - nM;
        xout[f_col[f]] = b[f_arow[f]] / A[f_diag_e[f]];
    }
}


// Singletons solved last: x_c = (b_c - sum_j B(c, j) x_j) / B(c, c), one block
// per row (the supply-rail rows hold one entry per connected device) with a
// fixed-order tree reduction.
// The supply-rail row holds one entry per connected device (tens of thousands):
// 1024 threads, each with four entries' loads in flight per step.
constexpr int POST_THREADS = 1024;
__global__ void __launch_bounds__(POST_THREADS) lu_post_kernel(int nL, const int* l_col, const int* l_arow,
                                                              const int* l_diag_e, const int* l_ptr, const int* l_e,
                                                              const int* l_x, const double* A, const double* b,
                                                              double* xout) {
    __shared__ double part[POST_THREADS / 32];
    const int row = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc = 0.0;
#pragma unroll 4
    for (int e = l_ptr[row] + threadIdx.x; e < l_ptr[row + 1]; e += POST_THREADS) acc += A[l_e[e]] * xout[l_x[e]];
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < POST_THREADS / 32; ++w) s += part[w];
        xout[l_col[row]] = (b[l_arow[row]] - s) / A[l_diag_e[row]];
    }
}


__global__ void scale_slots_kernel(int nnz, const double* __restrict__ A, const double* __restrict__ sc,
                                   double* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nnz) out[e] = A[e] * sc[e];
}

// The block M is factorised from the scaled values when a weighted matching
// is in use (one pass over the CSR values before the factorisation).
void lu_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s) {
    SparseLU& L = c.lu;
    if (L.d_slot_scale.p && c.nnz) {
        scale_slots_kernel<<<ceil_div(c.nnz, 256), 256, 0, s>>>(c.nnz, A, L.d_slot_scale.p, L.d_scaled.p);
        VGB_CUDA(cudaGetLastError());
        A = L.d_scaled.p;
    }
    mf_factor(c, A, fp32, s);
}

template <typename T>
static void lu_solve_once(Circuit& c, const double* A, const double* rhs, double* x, T* rhsM, T* ybuf, T* xbuf,
                          cudaStream_t s) {
    SparseLU& L = c.lu;
    const int nM = L.nM, nF = (int)L.f_col.size(), nL = (int)L.l_col.size();
    if (nM + nF)
        lu_pre_kernel<T><<<ceil_div(nM + nF, 256), 256, 0, s>>>(nM, nF, L.d_brow.p, L.d_pre_ptr.p, L.d_pre_e.p,
                                                                L.d_pre_f.p, L.d_f_col.p, L.d_f_arow.p,
                                                                L.d_f_diag_e.p, A, rhs, L.d_rscale.p, rhsM, x);
    if (nM) mf_solve_t<T>(c, rhsM, ybuf, xbuf, x, s);
    if (nL)
        lu_post_kernel<<<nL, POST_THREADS, 0, s>>>(nL, L.d_l_col.p, L.d_l_arow.p,
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
        lu_solve_once<double>(c, A, rhs, x, rhsM, c.d_work.p + nM, c.d_work.p + 2 * (size_t)nM, s);
        return;
    }
    float* rhsM = (float*)c.d_work.p;
    float* ybuf = rhsM + nM;
    float* xbuf = ybuf + nM;
    lu_solve_once<float>(c, A, rhs, x, rhsM, ybuf, xbuf, s);
    double* r = c.d_work2.p;
    double* d = c.d_work2.p + n;
    for (int k = 0; k < sweeps; ++k) {
        residual_kernel<<<ceil_div((long long)n * 32, 256), 256, 0, s>>>(n, c.d_indptr.p, c.d_indices.p, A, rhs, x, r);
        lu_solve_once<float>(c, A, r, d, rhsM, ybuf, xbuf, s);
        axpy_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, d, x);
    }
}

// ---------------------------------------------------------------------------
// small vector kernels
// ---------------------------------------------------------------------------

// Newton coefficients {c0, c1, d1, c2, gshunt} in device memory, where the
// evaluation, assembly and dQ/dt kernels read them (a captured graph replays
// kernels with frozen arguments, so values that change per step live here).
__global__ void set_coeffs_kernel(double* k, double c0, double c1, double d1, double c2, double gshunt) {
    k[0] = c0;
    k[1] = c1;
    k[2] = d1;
    k[3] = c2;
    k[4] = gshunt;
}
void launch_set_coeffs(double* kdev, double c0, double c1, double d1, double c2, double gshunt, cudaStream_t s) {
    set_coeffs_kernel<<<1, 1, 0, s>>>(kdev, c0, c1, d1, c2, gshunt);
}

// NOI constraint (solver_factories.py:775-782): rows and columns of NOI unknowns
// zeroed, their diagonal set to 1 and their RHS to 0, so delta[NOI] = 0.
__global__ void noi_enforce_kernel(const int* zero, int nz, const int* diag, const int* res, int nn, double* csr,
                                   double* rhs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nz) csr[zero[t]] = 0.0;
    else if (t < nz + nn) csr[diag[t - nz]] = 1.0;
    else if (t < nz + 2 * nn) rhs[res[t - nz - nn]] = 0.0;
}
void launch_noi_enforce(const int* zero, int nz, const int* diag, const int* res, int nn, double* csr, double* rhs,
                        cudaStream_t s) {
    const int total = nz + 2 * nn;
    if (total) noi_enforce_kernel<<<ceil_div(total, 256), 256, 0, s>>>(zero, nz, diag, res, nn, csr, rhs);
}

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

// t_dev (device memory) replaces t when given: the transient graph computes the time on the device
__global__ void eval_sources_kernel(const int* kind, const int* off, const int* cnt, const double* data,
                                    int n, double t, const double* t_dev, double* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = eval_source(kind[k], data + off[k], cnt[k], t_dev ? *t_dev : t);
}
void launch_eval_sources(const Sources& src, int n, double t, double* out, cudaStream_t s) {
    if (n) eval_sources_kernel<<<ceil_div(n, 128), 128, 0, s>>>(src.d_kind.p, src.d_off.p, src.d_cnt.p,
                                                                src.d_data.p, n, t, nullptr, out);
}
void launch_eval_sources_dev(const Sources& src, int n, const double* t_dev, double* out, cudaStream_t s) {
    if (n) eval_sources_kernel<<<ceil_div(n, 128), 128, 0, s>>>(src.d_kind.p, src.d_off.p, src.d_cnt.p,
                                                                src.d_data.p, n, 0.0, t_dev, out);
}

// The device elementary functions of the generated models, one per element
// (accuracy tests of csrc/vgb_math.cuh).  fn: 0 a/b, 1 exp(a), 2 ln(a),
// 3 pow(a, b), 4 the models' safe division (a/0 = 0), 5 1/a.
__global__ void math_eval_kernel(int fn, int n, const double* __restrict__ a, const double* __restrict__ b,
                                 double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i];
    double r = 0.0;
    switch (fn) {
        case 0: r = vgb_div(x, b[i]); break;
        case 1: r = vgb_exp(x); break;
        case 2: r = vgb_log(x); break;
        case 3: r = vgb_pow(x, b[i]); break;
        case 4: r = vgb_msdiv(x, b[i]); break;
        default: r = vgb_rcp(x); break;
    }
    out[i] = r;
}

void launch_math_eval(int fn, int n, const double* a, const double* b, double* out, cudaStream_t s) {
    if (n > 0) math_eval_kernel<<<ceil_div(n, 256), 256, 0, s>>>(fn, n, a, b, out);
}

// FP64 FMA throughput of the device: every SM runs warps of eight
// independent dependent-FMA chains (the measured rate is the denominator of
// the FP64 roofline fractions the benchmark reports).
constexpr int FP64_RATE_THREADS = 512;
__global__ void __launch_bounds__(FP64_RATE_THREADS) fp64_rate_kernel(int iters, double a, double b,
                                                                      double* __restrict__ sink) {
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 12345.678) sink[blockIdx.x] = s;  // keeps the chains live; never true for these inputs
}

double measure_fp64_rate(int iters, cudaStream_t s) {
    int dev = 0, sms = 0;
    VGB_CUDA(cudaGetDevice(&dev));
    VGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* sink = nullptr;
    VGB_CUDA(cudaMalloc(&sink, sizeof(double) * sms * 2));
    cudaEvent_t e0, e1;
    VGB_CUDA(cudaEventCreate(&e0));
    VGB_CUDA(cudaEventCreate(&e1));
    fp64_rate_kernel<<<sms * 2, FP64_RATE_THREADS, 0, s>>>(iters / 8, 0.9999999, 1e-9, sink);  // warm-up
    VGB_CUDA(cudaEventRecord(e0, s));
    fp64_rate_kernel<<<sms * 2, FP64_RATE_THREADS, 0, s>>>(iters, 0.9999999, 1e-9, sink);
    VGB_CUDA(cudaEventRecord(e1, s));
    VGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    VGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    const double flops = 2.0 * 8.0 * iters * (double)sms * 2 * FP64_RATE_THREADS;
    return flops / (ms * 1e-3) / 1e9;
}

} // namespace vgb
