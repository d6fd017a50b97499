// Multifrontal static-pivot LU of the block M and its triangular solves.
//
// Numeric factorisation is one persistent, sync-free kernel over a task list
// in topological order of the assembly tree (built by the host symbolic phase):
//
//   TASK_SMALL  front of order m <= SMALL_FRONT: one CTA assembles it in shared
//               memory (A entries + children's contribution blocks), eliminates
//               its w pivots and writes the front back;
//   TASK_DIAG   large front: assemble in global memory, factor the w x w
//               diagonal block on chip;
//   TASK_PANEL  one row tile of L21 = A21 U11^-1 and one column tile of
//               U12 = L11^-1 A12;
//   TASK_SCHUR  one tile of the contribution block, C -= L21 U12.
//
// CTAs claim tasks in list order from a global counter and wait (bounded) on
// flags of earlier tasks only, so every wait ends.  Extend-add is a pull by
// the parent, one child at a time, so sums are deterministic.  Front storage
// is dense column-major: F[i + j*m].
#include <cuda/atomic>

#include "vgb_kernels.cuh"

namespace vgb {

namespace {

__device__ __forceinline__ int ld_acq(const int* p) {
    return cuda::atomic_ref<const int, cuda::thread_scope_device>(*p).load(cuda::memory_order_acquire);
}
__device__ __forceinline__ void st_rel(int* p, int v) {
    cuda::atomic_ref<int, cuda::thread_scope_device>(*p).store(v, cuda::memory_order_release);
}

__device__ bool wait_eq(const int* flag, int epoch, int* abort_flag, int* err, unsigned limit) {
    unsigned it = 0;
    while (ld_acq(flag) != epoch) {
        if (++it > limit) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            atomicExch(abort_flag, 1);
            return false;
        }
        if ((it & 255) == 0) {
            if (*(volatile int*)abort_flag) return false;
            if (it > 4096) __nanosleep(200);
        }
    }
    return true;
}

}  // namespace

struct MFArgs {
    int ns;
    const long long* fr_ptr;
    const long long* fr_off;
    const int* fr_w;
    const int* ch_ptr;
    const int* ch_idx;
    const long long* em_ptr;
    const int* em_idx;
    const long long* asm_ptr;
    const int* asm_e;
    const int* asm_pos;
    const int* fr_task0;
    const int* fr_nb;
    const int* task_type;
    const int* task_front;
    const int* task_b0;
    const int* task_b1;
    const int* sn_parent;
    const int* fr_big;
    int n_tasks;
    const double* A;
    int* flags;       // done [ns], diag [ns], fwd [ns], bwd [ns], panel [n_tasks]
    int* count;       // per front
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

constexpr int MF_THREADS = 128;
constexpr int MF_SMEM_DOUBLES = 8192;  // 64 KB

// wait for every child front of S to be complete
__device__ bool wait_children(const MFArgs& a, int S, const int* flag_base) {
    bool ok = true;
    for (int q = a.ch_ptr[S] + threadIdx.x; q < a.ch_ptr[S + 1]; q += blockDim.x)
        ok = ok && wait_eq(flag_base + a.ch_idx[q], a.epoch, a.abort_flag, a.err, a.spin_limit);
    return __syncthreads_and(ok);
}

template <typename T>
__device__ void assemble_front(const MFArgs& a, int S, T* F, int m, const T* pool, bool zero_first) {
    if (zero_first)
        for (long long t = threadIdx.x; t < (long long)m * m; t += blockDim.x) F[t] = (T)0;
    __syncthreads();
    for (long long t = a.asm_ptr[S] + threadIdx.x; t < a.asm_ptr[S + 1]; t += blockDim.x)
        F[a.asm_pos[t]] = (T)a.A[a.asm_e[t]];
    __syncthreads();
    for (int q = a.ch_ptr[S]; q < a.ch_ptr[S + 1]; ++q) {
        const int C = a.ch_idx[q];
        const int mc = (int)(a.fr_ptr[C + 1] - a.fr_ptr[C]);
        const int wc = a.fr_w[C];
        const int rc = mc - wc;
        const T* FC = pool + a.fr_off[C];
        const int* em = a.em_idx + a.em_ptr[C];
        for (int idx = threadIdx.x; idx < rc * rc; idx += blockDim.x) {
            const int i = idx % rc, j = idx / rc;
            F[em[i] + (long long)em[j] * m] += __ldcg(FC + (wc + i) + (long long)(wc + j) * mc);
        }
        __syncthreads();
    }
}

// Eliminate w pivots of an m x m column-major matrix held by the CTA (shared or global).
template <typename T>
__device__ void partial_lu(T* F, int ld, int m, int w, int* err) {
    for (int p = 0; p < w; ++p) {
        T piv = F[p + (long long)p * ld];
        if (piv == (T)0 || !isfinite((double)piv)) {
            piv = (T)1e-30;
            __syncthreads();
            if (threadIdx.x == 0) {
                F[p + (long long)p * ld] = piv;
                atomicOr(err, DEV_ERR_PIVOT);
            }
        }
        __syncthreads();
        for (int i = p + 1 + threadIdx.x; i < m; i += blockDim.x) F[i + (long long)p * ld] /= piv;
        __syncthreads();
        const int n = m - p - 1;
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
            const int i = p + 1 + idx % n, j = p + 1 + idx / n;
            F[i + (long long)j * ld] -= F[i + (long long)p * ld] * F[p + (long long)j * ld];
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(MF_THREADS) mf_factor_kernel(MFArgs a, T* pool) {
    extern __shared__ double smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_task;
    int* const done = a.flags;
    int* const diag = a.flags + a.ns;
    int* const panel = a.flags + 4 * (size_t)a.ns;
    while (true) {
        if (threadIdx.x == 0) s_task = atomicAdd(a.counter, 1);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= a.n_tasks) return;
        const int type = a.task_type[t];
        const int S = a.task_front[t];
        const int m = (int)(a.fr_ptr[S + 1] - a.fr_ptr[S]);
        const int w = a.fr_w[S];
        T* FS = pool + a.fr_off[S];
        const int P = a.sn_parent[S];
        const bool push = P >= 0 && a.fr_big[P];
        if (type == TASK_SMALL) {
            if (!wait_children(a, S, done)) continue;
            assemble_front<T>(a, S, sm, m, pool, true);
            partial_lu<T>(sm, m, m, w, a.err);
            for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) FS[idx] = sm[idx];
            if (push) {
                // contribution block straight into the (large) parent front
                const int r = m - w;
                const int mp = (int)(a.fr_ptr[P + 1] - a.fr_ptr[P]);
                T* FP = pool + a.fr_off[P];
                const int* em = a.em_idx + a.em_ptr[S];
                for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
                    const int i = idx % r, j = idx / r;
                    atomicAdd(FP + em[i] + (long long)em[j] * mp, sm[(w + i) + (w + j) * m]);
                }
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) st_rel(done + S, a.epoch);
        } else if (type == TASK_DIAG) {
            // a large front is zeroed and A-assembled before the kernel starts and its children
            // push their contribution blocks into it: once they are done it is complete
            if (!wait_children(a, S, done)) continue;
            for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x)
                sm[idx] = __ldcg(FS + idx % w + (long long)(idx / w) * m);
            __syncthreads();
            partial_lu<T>(sm, w, w, w, a.err);
            for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) FS[idx % w + (long long)(idx / w) * m] = sm[idx];
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) st_rel(diag + S, a.epoch);
        } else if (type == TASK_PANEL) {
            bool ok = true;
            if (threadIdx.x == 0) ok = wait_eq(diag + S, a.epoch, a.abort_flag, a.err, a.spin_limit);
            if (__syncthreads_or(!ok)) continue;
            const int b = a.task_b0[t];
            const int r0 = w + b * FRONT_TILE;
            const int nr = min(FRONT_TILE, m - r0);
            T* D = sm;                       // w x w diagonal block (L11 \ U11)
            T* R = sm + w * w;               // nr x w rows of A21
            T* Cc = R + FRONT_TILE * w;      // w x nr columns of A12
            for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x)
                D[idx] = __ldcg(FS + idx % w + (long long)(idx / w) * m);
            for (int idx = threadIdx.x; idx < nr * w; idx += blockDim.x) {
                const int i = idx % nr, k = idx / nr;
                R[i + k * FRONT_TILE] = __ldcg(FS + (r0 + i) + (long long)k * m);
                Cc[k + i * w] = __ldcg(FS + k + (long long)(r0 + i) * m);
            }
            __syncthreads();
            const int tid = threadIdx.x;
            if (tid < nr) {
                // row i of L21: x U11 = a
                T* x = R + tid;
                for (int k = 0; k < w; ++k) {
                    T s = x[k * FRONT_TILE];
                    for (int kk = 0; kk < k; ++kk) s -= x[kk * FRONT_TILE] * D[kk + k * w];
                    x[k * FRONT_TILE] = s / D[k + k * w];
                }
            } else if (tid >= 64 && tid < 64 + nr) {
                // column j of U12: L11 y = a (unit lower)
                T* y = Cc + (tid - 64) * w;
                for (int k = 0; k < w; ++k) {
                    T s = y[k];
                    for (int kk = 0; kk < k; ++kk) s -= D[k + kk * w] * y[kk];
                    y[k] = s;
                }
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < nr * w; idx += blockDim.x) {
                const int i = idx % nr, k = idx / nr;
                FS[(r0 + i) + (long long)k * m] = R[i + k * FRONT_TILE];
                FS[k + (long long)(r0 + i) * m] = Cc[k + i * w];
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) st_rel(panel + t, a.epoch);
        } else {  // TASK_SCHUR
            const int bi = a.task_b0[t], bj = a.task_b1[t];
            const int t0 = a.fr_task0[S];
            bool ok = true;
            if (threadIdx.x == 0) {
                ok = wait_eq(panel + t0 + 1 + bi, a.epoch, a.abort_flag, a.err, a.spin_limit);
                ok = ok && wait_eq(panel + t0 + 1 + bj, a.epoch, a.abort_flag, a.err, a.spin_limit);
            }
            if (__syncthreads_or(!ok)) continue;
            const int i0 = w + bi * FRONT_TILE, j0 = w + bj * FRONT_TILE;
            const int ni = min(FRONT_TILE, m - i0), nj = min(FRONT_TILE, m - j0);
            T* Ls = sm;                        // FRONT_TILE x w
            T* Us = sm + FRONT_TILE * w;       // w x FRONT_TILE
            for (int idx = threadIdx.x; idx < ni * w; idx += blockDim.x) {
                const int i = idx % ni, k = idx / ni;
                Ls[i + k * FRONT_TILE] = __ldcg(FS + (i0 + i) + (long long)k * m);
            }
            for (int idx = threadIdx.x; idx < nj * w; idx += blockDim.x) {
                const int k = idx % w, j = idx / w;
                Us[k + j * w] = __ldcg(FS + k + (long long)(j0 + j) * m);
            }
            __syncthreads();
            const int mp = push ? (int)(a.fr_ptr[P + 1] - a.fr_ptr[P]) : 0;
            T* FP = push ? pool + a.fr_off[P] : nullptr;
            const int* em = a.em_idx + a.em_ptr[S];
            for (int idx = threadIdx.x; idx < ni * nj; idx += blockDim.x) {
                const int i = idx % ni, j = idx / ni;
                T acc = 0;
                for (int k = 0; k < w; ++k) acc += Ls[i + k * FRONT_TILE] * Us[k + j * w];
                const long long pos = (i0 + i) + (long long)(j0 + j) * m;
                if (push) {
                    const int ci = i0 - w + i, cj = j0 - w + j;  // indices inside the contribution block
                    atomicAdd(FP + em[ci] + (long long)em[cj] * mp, __ldcg(FS + pos) - acc);
                } else {
                    FS[pos] = __ldcg(FS + pos) - acc;
                }
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) {
                const int nb = a.fr_nb[S];
                const int old = atomicAdd(a.count + S, 1);
                if (old == nb * nb - 1) {
                    __threadfence();
                    st_rel(done + S, a.epoch);
                }
            }
        }
    }
}

// A entries of the large fronts, scattered once the pool is zeroed.
template <typename T>
__global__ void mf_init_kernel(long long n, const int* __restrict__ e, const long long* __restrict__ pos,
                               const double* __restrict__ A, T* pool) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) pool[pos[i]] = (T)A[e[i]];
}

// ---------------------------------------------------------------------------
// Triangular solves over the assembly tree
// ---------------------------------------------------------------------------

struct MFSolveArgs {
    int ns;
    const long long* fr_ptr;
    const long long* fr_off;
    const int* fr_w;
    const int* fr_idx;
    const int* sn_parent;
    const int* ch_ptr;
    const int* ch_idx;
    const long long* em_ptr;
    const int* em_idx;
    const long long* cv_off;
    const int* q;          // B index of each permuted M index
    int* flags;            // fwd [ns], bwd [ns]
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

// Forward: L y = rhs.  Each front adds its children's update vectors, solves
// with its unit-lower diagonal block and passes cv = u_tail - L21 y up.
template <typename T>
__global__ void __launch_bounds__(MF_THREADS) mf_fwd_kernel(MFSolveArgs a, const T* __restrict__ pool,
                                                            const T* __restrict__ rhs, T* y, T* cv) {
    extern __shared__ double smem_raw[];
    T* u = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_S;
    int* const fdone = a.flags;
    while (true) {
        if (threadIdx.x == 0) s_S = atomicAdd(a.counter, 1);
        __syncthreads();
        const int S = s_S;
        __syncthreads();
        if (S >= a.ns) return;
        bool ok = true;
        for (int q = a.ch_ptr[S] + threadIdx.x; q < a.ch_ptr[S + 1]; q += blockDim.x)
            ok = ok && wait_eq(fdone + a.ch_idx[q], a.epoch, a.abort_flag, a.err, a.spin_limit);
        if (!__syncthreads_and(ok)) continue;
        const int m = (int)(a.fr_ptr[S + 1] - a.fr_ptr[S]);
        const int w = a.fr_w[S];
        const int* idx = a.fr_idx + a.fr_ptr[S];
        const T* F = pool + a.fr_off[S];
        for (int i = threadIdx.x; i < m; i += blockDim.x) u[i] = i < w ? rhs[idx[i]] : (T)0;
        __syncthreads();
        for (int q = a.ch_ptr[S]; q < a.ch_ptr[S + 1]; ++q) {
            const int C = a.ch_idx[q];
            const int rc = (int)(a.cv_off[C + 1] - a.cv_off[C]);
            const int* em = a.em_idx + a.em_ptr[C];
            const T* cvc = cv + a.cv_off[C];
            for (int i = threadIdx.x; i < rc; i += blockDim.x) u[em[i]] += __ldcg(cvc + i);
            __syncthreads();
        }
        for (int p = 0; p < w; ++p) {
            const T yp = u[p];
            for (int i = p + 1 + threadIdx.x; i < m; i += blockDim.x) u[i] -= F[i + (long long)p * m] * yp;
            __syncthreads();
        }
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (i < w) y[idx[i]] = u[i];
            else cv[a.cv_off[S] + (i - w)] = u[i];
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) st_rel(fdone + S, a.epoch);
    }
}

// Backward: U x = y from the root down; a front needs only its parent done
// (its tail indices are pivots of ancestors).
template <typename T>
__global__ void __launch_bounds__(MF_THREADS) mf_bwd_kernel(MFSolveArgs a, const T* __restrict__ pool,
                                                            const T* __restrict__ y, T* xs, double* xout) {
    extern __shared__ double smem_raw[];
    T* z = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_S;
    int* const bdone = a.flags + a.ns;
    while (true) {
        if (threadIdx.x == 0) s_S = atomicAdd(a.counter, 1);
        __syncthreads();
        const int c = s_S;
        __syncthreads();
        if (c >= a.ns) return;
        const int S = a.ns - 1 - c;
        const int P = a.sn_parent[S];
        bool ok = true;
        if (threadIdx.x == 0 && P >= 0) ok = wait_eq(bdone + P, a.epoch, a.abort_flag, a.err, a.spin_limit);
        if (__syncthreads_or(!ok)) continue;
        const int m = (int)(a.fr_ptr[S + 1] - a.fr_ptr[S]);
        const int w = a.fr_w[S];
        const int* idx = a.fr_idx + a.fr_ptr[S];
        const T* F = pool + a.fr_off[S];
        // stage x_tail (pivots of ancestors, written by other CTAs: read through L2)
        T* xt = z + w;
        for (int j = threadIdx.x; j < m - w; j += blockDim.x) xt[j] = __ldcg(xs + idx[w + j]);
        __syncthreads();
        // z = y_S - U12 x_tail: each warp takes pivot rows, lanes split the tail
        {
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
            for (int p = warp; p < w; p += nw) {
                T s = 0;
                for (int j = lane; j < m - w; j += 32) s += F[p + (long long)(w + j) * m] * xt[j];
                for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
                if (lane == 0) z[p] = y[idx[p]] - s;
            }
        }
        __syncthreads();
        for (int p = w - 1; p >= 0; --p) {
            const T xp = z[p] / F[p + (long long)p * m];
            __syncthreads();
            if (threadIdx.x == 0) z[p] = xp;
            for (int i = threadIdx.x; i < p; i += blockDim.x) z[i] -= F[i + (long long)p * m] * xp;
            __syncthreads();
        }
        for (int p = threadIdx.x; p < w; p += blockDim.x) {
            xs[idx[p]] = z[p];
            xout[a.q[idx[p]]] = (double)z[p];
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) st_rel(bdone + S, a.epoch);
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

static int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        sms = std::max(1, sms);
    }
    return sms;
}

static MFArgs mf_args(Circuit& c, const double* A) {
    SparseLU& L = c.lu;
    MFArgs a{};
    a.ns = L.nsn;
    a.fr_ptr = L.d_fr_ptr.p;
    a.fr_off = L.d_fr_off.p;
    a.fr_w = L.d_fr_w.p;
    a.ch_ptr = L.d_ch_ptr.p;
    a.ch_idx = L.d_ch_idx.p;
    a.em_ptr = L.d_em_ptr.p;
    a.em_idx = L.d_em_idx.p;
    a.asm_ptr = L.d_asm_ptr.p;
    a.asm_e = L.d_asm_e.p;
    a.asm_pos = L.d_asm_pos.p;
    a.fr_task0 = L.d_fr_task0.p;
    a.fr_nb = L.d_fr_nb.p;
    a.task_type = L.d_task_type.p;
    a.task_front = L.d_task_front.p;
    a.task_b0 = L.d_task_b0.p;
    a.task_b1 = L.d_task_b1.p;
    a.sn_parent = L.d_sn_parent.p;
    a.fr_big = L.d_fr_big.p;
    a.n_tasks = (int)L.task_type.size();
    a.A = A;
    a.flags = L.d_mf_flags.p;
    a.count = L.d_mf_count.p;
    a.counter = L.d_counters.p;
    a.abort_flag = L.d_counters.p + 3;
    a.err = &c.d_status.p->dev_err;
    a.spin_limit = 1u << 22;
    return a;
}

template <typename T>
static void mf_factor_t(Circuit& c, const double* A, T* pool, cudaStream_t s) {
    SparseLU& L = c.lu;
    static bool attr_set = false;
    if (!attr_set) {
        VGB_CUDA(cudaFuncSetAttribute(mf_factor_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      MF_SMEM_DOUBLES * (int)sizeof(double)));
        attr_set = true;
    }
    L.epoch++;
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
    VGB_CUDA(cudaMemsetAsync(L.d_mf_count.p, 0, std::max(L.nsn, 1) * sizeof(int), s));
    if (!L.big_asm_e.empty()) {
        // large fronts accumulate pushes from their children: zero them, then place A
        // (one memset over the span that holds them)
        VGB_CUDA(cudaMemsetAsync(pool + L.big_lo, 0, (L.big_hi - L.big_lo) * sizeof(T), s));
        const long long n = (long long)L.big_asm_e.size();
        mf_init_kernel<T><<<ceil_div(n, 256), 256, 0, s>>>(n, L.d_big_asm_e.p, L.d_big_asm_pos.p, A, pool);
    }
    MFArgs a = mf_args(c, A);
    a.epoch = L.epoch;
    const int blocks = std::min(sm_count() * 3, std::max(a.n_tasks, 1));
    mf_factor_kernel<T><<<blocks, MF_THREADS, MF_SMEM_DOUBLES * sizeof(double), s>>>(a, pool);
    VGB_CUDA(cudaGetLastError());
}

void mf_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s) {
    if (c.lu.nsn == 0) return;
    if (fp32) mf_factor_t<float>(c, A, c.lu.d_pool32.p, s);
    else mf_factor_t<double>(c, A, c.lu.d_pool64.p, s);
}

template <typename T>
void mf_solve_t(Circuit& c, const T* rhsM, T* y, T* xs, double* xout, cudaStream_t s) {
    SparseLU& L = c.lu;
    if (L.nsn == 0) return;
    const T* pool = std::is_same<T, float>::value ? (const T*)L.d_pool32.p : (const T*)L.d_pool64.p;
    T* cv = std::is_same<T, float>::value ? (T*)L.d_cv32.p : (T*)L.d_cv64.p;
    L.epoch++;
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
    MFSolveArgs a{};
    a.ns = L.nsn;
    a.fr_ptr = L.d_fr_ptr.p;
    a.fr_off = L.d_fr_off.p;
    a.fr_w = L.d_fr_w.p;
    a.fr_idx = L.d_fr_idx.p;
    a.sn_parent = L.d_sn_parent.p;
    a.ch_ptr = L.d_ch_ptr.p;
    a.ch_idx = L.d_ch_idx.p;
    a.em_ptr = L.d_em_ptr.p;
    a.em_idx = L.d_em_idx.p;
    a.cv_off = L.d_cv_off.p;
    a.q = L.d_q.p;
    a.flags = L.d_mf_flags.p + 2 * (size_t)L.nsn;
    a.counter = L.d_counters.p + 1;
    a.abort_flag = L.d_counters.p + 3;
    a.err = &c.d_status.p->dev_err;
    a.epoch = L.epoch;
    a.spin_limit = 1u << 22;
    const size_t smem = (size_t)std::max<long long>(L.mf_max_m, 1) * sizeof(T);
    const int blocks = std::min(sm_count() * 4, L.nsn);
    mf_fwd_kernel<T><<<blocks, MF_THREADS, smem, s>>>(a, pool, rhsM, y, cv);
    a.counter = L.d_counters.p + 2;
    mf_bwd_kernel<T><<<blocks, MF_THREADS, smem, s>>>(a, pool, y, xs, xout);
    VGB_CUDA(cudaGetLastError());
}

template void mf_solve_t<double>(Circuit&, const double*, double*, double*, double*, cudaStream_t);
template void mf_solve_t<float>(Circuit&, const float*, float*, float*, double*, cudaStream_t);

}  // namespace vgb
