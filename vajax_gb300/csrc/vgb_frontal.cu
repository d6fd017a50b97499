// Multifrontal static-pivot LU of the block M and its triangular solves.
//
// Numeric factorisation is one persistent, sync-free kernel over a task list
// in topological order of the assembly tree (built by the host symbolic phase):
//
//   TASK_SMALL   front of order m <= SMALL_FRONT: one CTA assembles it in shared
//                memory (A entries, then the children's contribution blocks in
//                child order), eliminates its w pivots and stores it;
//   TASK_GETRF   large front, diagonal tile k: LU of a 32 x 32 tile in the
//                registers of the CTA's warps;
//   TASK_TRSM_L  tile (i, k) below it: L(i,k) = A(i,k) U(k,k)^-1;
//   TASK_TRSM_U  tile (k, j) right of it: U(k,j) = L(k,k)^-1 A(k,j);
//   TASK_GEMM    trailing tile (i, j): A(i,j) -= L(i,k) U(k,j), except the
//                update of the next diagonal tile (k+1, k+1) of the pivot block:
//                GETRF(1) applies that one itself, and for k + 1 >= 2 it runs as
//   TASK_DUPD    DUPD_SLICES column slices of that update on separate CTAs.
//
// Large fronts are never assembled as a whole: the first task that touches a
// tile (the k = 0 task of that tile) builds it in shared memory from its A
// entries and the blocks of the children's contribution blocks that land in
// it, in child order, so every sum has a fixed order and the factorisation is
// deterministic.  A per-tile version counter orders the updates of a tile
// (GEMM k waits for version k) and marks finished L / U / diagonal tiles
// (TILE_FINAL).  CTAs claim tasks in list order from a global counter and wait
// (bounded) only on tasks earlier in the list, so every wait ends.
//
// Front storage is dense column-major, F[i + j * m], in one pool.
#include <cuda/atomic>
#include <mutex>

#include "vgb_fastdiv.cuh"
#include "vgb_kernels.cuh"

namespace vgb {

namespace {

__device__ __forceinline__ int ld_acq(const int* p) {
    return cuda::atomic_ref<const int, cuda::thread_scope_device>(*p).load(cuda::memory_order_acquire);
}
__device__ __forceinline__ void st_rel(int* p, int v) {
    cuda::atomic_ref<int, cuda::thread_scope_device>(*p).store(v, cuda::memory_order_release);
}

__device__ __forceinline__ unsigned mf_smid() {
    unsigned r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}

// Column flags of one tile task in shared memory (block scope).
__device__ __forceinline__ int ld_acq_cta(const int* p) {
    return cuda::atomic_ref<const int, cuda::thread_scope_block>(*p).load(cuda::memory_order_acquire);
}
__device__ __forceinline__ void st_rel_cta(int* p, int v) {
    cuda::atomic_ref<int, cuda::thread_scope_block>(*p).store(v, cuda::memory_order_release);
}

// Spin until *flag == value; gives up after `limit` polls (sets the timeout
// error bit and the abort flag) or when another CTA has aborted.
__device__ bool wait_eq(const int* flag, int value, int* abort_flag, int* err, unsigned limit) {
    unsigned it = 0;
    while (ld_acq(flag) != value) {
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
    const int* fr_kb;
    const int* fr_nb;
    const int* fr_tile0;
    const long long* tasm_ptr;
    const int* tasm_e;
    const int* tasm_pos;
    const long long* tch_ptr;
    const int* tch;
    const int* task_type;
    const int* task_front;
    const int* task_i;
    const int* task_j;
    const int* task_k;
    int n_tasks;
    const double* A;
    int* done;        // [ns] epoch flag: front factorised (contribution block final)
    int* count;       // [ns] final contribution tiles of a large front
    int* tver;        // [n_tiles] updates applied to a tile, or TILE_FINAL
    int* tcnt;        // [n_tiles] slices of a diagonal tile's last update applied
    int* sm_busy;     // [MF_SM_SLOTS] chain tasks running on each SM
    int* counter;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

constexpr int MF_THREADS = 512;  // tree-solve CTAs: 16 warps (80k network: 0.92 ms per solve pair, 1.02 with 8 warps, 1.28 with 4)
constexpr int LD = FRONT_TILE_LD;
constexpr int TILE_ELEMS = FRONT_TILE * FRONT_TILE_LD;
// shared memory of a factorisation CTA: one small front, or three tiles
constexpr int MF_SMEM_ELEMS = SMALL_FRONT * SMALL_FRONT;
static_assert(SMALL_FRONT <= MF_FACTOR_THREADS, "one thread per row of a small front's column");
static_assert(3 * TILE_ELEMS <= MF_SMEM_ELEMS, "three tiles must fit in the small-front buffer");
static_assert(FRONT_TILE * FRONT_TILE + FRONT_TILE <= TILE_ELEMS, "a tile area holds 32 exchanged columns and 32 reciprocals");

__device__ __forceinline__ int tile_lo(int t, int kb, int w) {
    return t < kb ? t * FRONT_TILE : w + (t - kb) * FRONT_TILE;
}
__device__ __forceinline__ int tile_hi(int t, int kb, int nb, int w, int m) {
    return t + 1 < nb ? tile_lo(t + 1, kb, w) : m;
}

// wait until every child front of S is factorised
__device__ bool wait_children(const MFArgs& a, int S) {
    bool ok = true;
    for (int q = a.ch_ptr[S] + threadIdx.x; q < a.ch_ptr[S + 1]; q += blockDim.x)
        ok = ok && wait_eq(a.done + a.ch_idx[q], a.epoch, a.abort_flag, a.err, a.spin_limit);
    return __syncthreads_and(ok);
}

// thread 0 waits on up to three flags; the whole CTA learns the outcome
__device__ bool wait3(const MFArgs& a, const int* f0, int v0, const int* f1, int v1, const int* f2, int v2) {
    bool ok = true;
    if (threadIdx.x == 0) {
        if (f0) ok = wait_eq(f0, v0, a.abort_flag, a.err, a.spin_limit);
        if (ok && f1) ok = wait_eq(f1, v1, a.abort_flag, a.err, a.spin_limit);
        if (ok && f2) ok = wait_eq(f2, v2, a.abort_flag, a.err, a.spin_limit);
    }
    return !__syncthreads_or(!ok);
}

// publish a flag after the CTA's global stores
__device__ __forceinline__ void publish(int* flag, int value) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        st_rel(flag, value);
    }
}

// ---- small fronts ------------------------------------------------------------

template <typename T>
__device__ void assemble_small(const MFArgs& a, int S, T* F, int m, const T* pool) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) F[t] = (T)0;
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
        for (int cj = warp; cj < rc; cj += nw) {
            const int dj = em[cj] * m;
            const T* src = FC + (long long)(wc + cj) * mc + wc;
            for (int ci = lane; ci < rc; ci += 32) F[em[ci] + dj] += __ldcg(src + ci);
        }
        __syncthreads();
    }
}

// Eliminate the first w pivots of an m x m column-major front in shared memory.
template <typename T>
__device__ void partial_lu_small(T* F, int m, int w, int* err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int p = 0; p < w; ++p) {
        T piv = F[p + p * m];
        if (piv == (T)0 || !isfinite((double)piv)) piv = (T)1e-30;
        // only the threads that scale the column form the reciprocal (m <= SMALL_FRONT < blockDim)
        if (p + 1 + (int)threadIdx.x < m) F[p + 1 + threadIdx.x + p * m] *= vgb_rcp(piv);
        __syncthreads();
        // a replaced pivot goes back once every thread has read it; the update below
        // does not read the diagonal element
        if (threadIdx.x == 0 && piv != F[p + p * m]) {
            F[p + p * m] = piv;
            atomicOr(err, DEV_ERR_PIVOT);
        }
        for (int j = p + 1 + warp; j < m; j += nw) {
            const T u = F[p + j * m];
            for (int i = p + 1 + lane; i < m; i += 32) F[i + j * m] -= F[i + p * m] * u;
        }
        __syncthreads();
    }
}

// ---- tiles of large fronts -----------------------------------------------------

// The tile kernels below spread each elimination step over the CTA's NWARP
// warps (two per SM sub-partition: each warp issues FP64 at a third of the
// SM's rate, so the chain of dependent elimination steps shortens with fewer
// columns per warp) and hand the step's pivot row or column between warps
// through shared memory.
constexpr int NWARP = MF_FACTOR_THREADS / 32;
constexpr int QPW = FRONT_TILE / NWARP;  // columns (or rows) per warp
static_assert((NWARP & (NWARP - 1)) == 0 && FRONT_TILE % NWARP == 0, "warps per tile: a power of two dividing 32");

// Tile rows [r0, r0+nr) x columns [c0, c0+nc) of front F (leading dimension m),
// zero-padded to 32 x 32, held in registers (lane = row, warp w has columns w,
// w + NWARP, ...).  fetch_tile only issues the loads, so a task fetches all of its
// tiles before the first shared-memory store and their L2 latencies overlap.
template <typename T>
struct TileRegs {
    T v[QPW];
};

template <typename T>
__device__ __forceinline__ void fetch_tile(TileRegs<T>& t, const T* F, long long m, int r0, int nr, int c0, int nc) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < QPW; ++q) {
        const int c = warp + NWARP * q;
        t.v[q] = (lane < nr && c < nc) ? __ldcg(F + (r0 + lane) + (c0 + c) * m) : (T)0;
    }
}

template <typename T>
__device__ __forceinline__ void put_tile(T* dst, const TileRegs<T>& t) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < QPW; ++q) dst[lane + (warp + NWARP * q) * LD] = t.v[q];
}

template <typename T>
__device__ void store_tile(T* F, const T* src, long long m, int r0, int nr, int c0, int nc) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = warp; c < nc; c += nw)
        if (lane < nr) __stcg(F + (r0 + lane) + (c0 + c) * m, src[lane + c * LD]);
}

// First touch: A entries of the tile, then the children's blocks in child order.
// A child's block lands in at most 32 rows and 32 columns of the tile.  Each warp
// adds only into the tile columns it owns (column % NWARP == warp), so no two warps
// touch one element and every element still receives its children's values in child
// order, with no block barrier between children.  The headers of up to 32 blocks
// are loaded at once (one per lane), and the next block's row and column maps are
// loaded while the current block's values are added, so a block costs about one
// L2 round trip instead of four dependent ones.
template <typename T>
__device__ void assemble_tile(const MFArgs& a, long long tile, T* dst, int r0, int c0, const T* pool) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < TILE_ELEMS; t += blockDim.x) dst[t] = (T)0;
    __syncthreads();
    for (long long t = a.tasm_ptr[tile] + threadIdx.x; t < a.tasm_ptr[tile + 1]; t += blockDim.x)
        dst[a.tasm_pos[t]] = (T)a.A[a.tasm_e[t]];
    __syncthreads();
    const long long qb = a.tch_ptr[tile];
    const int nblk = (int)((a.tch_ptr[tile + 1] - qb) / 5);
    for (int b0 = 0; b0 < nblk; b0 += 32) {
        // lane k: header of block b0 + k (source base offset, leading dimension, ranges, map offset)
        long long hbase = 0, hem = 0;
        int hmc = 0, hrlo = 0, hnr = 0, hclo = 0, hnc = 0;
        if (b0 + lane < nblk) {
            const int* h = a.tch + qb + 5LL * (b0 + lane);
            const int C = h[0];
            hrlo = h[1];
            hnr = h[2] - h[1];
            hclo = h[3];
            hnc = h[4] - h[3];
            const long long mc = a.fr_ptr[C + 1] - a.fr_ptr[C];
            const int wc = a.fr_w[C];
            hmc = (int)mc;
            hbase = a.fr_off[C] + (long long)wc * mc + wc;
            hem = a.em_ptr[C];
            if (hnr > FRONT_TILE || hnc > FRONT_TILE) {
                atomicOr(a.err, DEV_ERR_BOUNDS);
                hnr = min(hnr, FRONT_TILE);
                hnc = min(hnc, FRONT_TILE);
            }
        }
        const int nb = min(32, nblk - b0);
        // this lane's destination row and column in block k (-1: none)
        auto maps = [&](int k, int& drow, int& dcol) {
            const long long em = __shfl_sync(0xffffffffu, hem, k);
            const int rlo = __shfl_sync(0xffffffffu, hrlo, k), nr = __shfl_sync(0xffffffffu, hnr, k);
            const int clo = __shfl_sync(0xffffffffu, hclo, k), nc = __shfl_sync(0xffffffffu, hnc, k);
            drow = lane < nr ? a.em_idx[em + rlo + lane] - r0 : -1;
            dcol = lane < nc ? a.em_idx[em + clo + lane] - c0 : -1;
            if ((unsigned)drow >= (unsigned)FRONT_TILE) drow = -1;
            if ((unsigned)dcol >= (unsigned)FRONT_TILE) dcol = -1;
        };
        int drow, dcol;
        maps(0, drow, dcol);
        for (int k = 0; k < nb; ++k) {
            const long long base = __shfl_sync(0xffffffffu, hbase, k);
            const int mc = __shfl_sync(0xffffffffu, hmc, k);
            const int rlo = __shfl_sync(0xffffffffu, hrlo, k), clo = __shfl_sync(0xffffffffu, hclo, k);
            int ndrow = -1, ndcol = -1;
            if (k + 1 < nb) maps(k + 1, ndrow, ndcol);
            // the block's columns that this warp owns: at most FRONT_TILE / warps of them
            unsigned mine = __ballot_sync(0xffffffffu, dcol >= 0 && dcol % NWARP == warp);
            T v[FRONT_TILE / NWARP];
            int dc[FRONT_TILE / NWARP];
#pragma unroll
            for (int t = 0; t < FRONT_TILE / NWARP; ++t) {
                dc[t] = -1;
                v[t] = (T)0;
                if (mine) {
                    const int l = __ffs(mine) - 1;
                    mine &= mine - 1;
                    dc[t] = __shfl_sync(0xffffffffu, dcol, l);
                    if (drow >= 0) v[t] = __ldcg(pool + base + (long long)(clo + l) * mc + rlo + lane);
                }
            }
#pragma unroll
            for (int t = 0; t < FRONT_TILE / NWARP; ++t)
                if (dc[t] >= 0 && drow >= 0) dst[drow + dc[t] * LD] += v[t];
            drow = ndrow;
            dcol = ndcol;
        }
    }
    __syncthreads();
}

// Pivot of step p (checked, replaced by 1e-30 and flagged when zero) and its
// reciprocal, in every lane of the warp that owns column p.
template <typename T>
__device__ __forceinline__ void next_pivot(T& col, int p, int lane, int* err, T& r) {
    T piv = __shfl_sync(0xffffffffu, col, p);
    if (piv == (T)0 || !isfinite((double)piv)) {
        piv = (T)1e-30;
        if (lane == p) col = piv;
        if (lane == 0) atomicOr(err, DEV_ERR_PIVOT);
    }
    r = vgb_rcp(piv);  // on the chain of dependent pivot steps: the short reciprocal
}

// The elimination steps below hand each finished column (or row) from the warp
// that owns it to the others through shared memory: the owner stores it in
// xch[32 c ...] and releases flag[c]; a warp that needs it acquires the flag
// (bounded spin) and loads it.  No block barrier per step: the owner of the
// next column applies the step to that column first and publishes it at
// once, and each warp applies the step to its other columns afterwards, while
// the chain of dependent steps goes on in the next owner.  One warp issues at
// most one FP64 instruction per 64 cycles, so with a barrier per step every
// step waited for the busiest warp's updates; the per-element operations and
// their order are those of the barrier form.
__device__ __forceinline__ void col_publish(int* f) {
    __threadfence_block();
    __syncwarp();
    if ((threadIdx.x & 31) == 0) st_rel_cta(f, 1);
}
__device__ __forceinline__ void col_wait(const int* f, int* err) {
    unsigned it = 0;
    while (ld_acq_cta(f) == 0) {
        if (++it > (1u << 22)) {
            if ((threadIdx.x & 31) == 0) atomicOr(err, DEV_ERR_TIMEOUT);
            break;
        }
    }
}

// LU without pivoting of the leading n x n block of a tile.  lane = row; warp
// g owns columns g, g + NWARP, ... in registers.  xch holds the multiplier
// columns (32 x 32), flag the 32 column flags.
template <typename T>
__device__ void getrf_tile(T* t, int n, int* err, T* xch, int* flag) {
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    T a[QPW];
#pragma unroll
    for (int q = 0; q < QPW; ++q) a[q] = t[lane + (g + NWARP * q) * LD];
    if (threadIdx.x < FRONT_TILE) flag[threadIdx.x] = 0;
    __syncthreads();
    if (n > 0 && g == 0) {
        T r;
        next_pivot<T>(a[0], 0, lane, err, r);
        if (lane > 0) a[0] *= r;
        xch[lane] = a[0];
        col_publish(flag);
    }
    for (int p = 0; p + 1 < n; ++p) {
        if (g + NWARP * (QPW - 1) <= p) break;  // no column of this warp is right of p
        // multipliers L(:, p): in registers for the owner, else from its flag
        T l;
        if (g == (p & (NWARP - 1))) {
            l = a[p / NWARP];
        } else {
            col_wait(flag + p, err);
            l = xch[p * FRONT_TILE + lane];
        }
        const int p1 = p + 1;
        if (g == (p1 & (NWARP - 1))) {
            // the next pivot column first: update, pivot, multipliers, publish
            const int q1 = p1 / NWARP;
            const T u = __shfl_sync(0xffffffffu, a[q1], p);
            if (lane > p) a[q1] -= l * u;
            T r;
            next_pivot<T>(a[q1], p1, lane, err, r);
            if (lane > p1) a[q1] *= r;
            xch[p1 * FRONT_TILE + lane] = a[q1];
            col_publish(flag + p1);
        }
#pragma unroll
        for (int q = 0; q < QPW; ++q) {
            const int c = g + NWARP * q;
            if (c > p1 && c < n) {  // warp-uniform: finished columns issue no FP64 work
                const T u = __shfl_sync(0xffffffffu, a[q], p);  // U(p, c)
                if (lane > p) a[q] -= l * u;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < QPW; ++q) t[lane + (g + NWARP * q) * LD] = a[q];
    __syncthreads();
}

// x := x U^-1 with U the upper triangle (with diagonal) of the n x n tile d.
// lane = row of x; warp g owns columns g, g + NWARP, ...; xch holds the solved
// columns (32 x 32) and then the diagonal's reciprocals.
template <typename T>
__device__ void trsm_l_tile(T* x, const T* d, int n, T* xch, int* flag, int* err) {
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    T* dinv = xch + FRONT_TILE * FRONT_TILE;  // reciprocals of the diagonal, formed once in parallel
    if (threadIdx.x < n) dinv[threadIdx.x] = vgb_rcp(d[threadIdx.x + threadIdx.x * LD]);
    if (threadIdx.x < FRONT_TILE) flag[threadIdx.x] = 0;
    T a[QPW], u[QPW];
#pragma unroll
    for (int q = 0; q < QPW; ++q) {
        a[q] = x[lane + (g + NWARP * q) * LD];
        u[q] = d[lane + (g + NWARP * q) * LD];  // U(lane, c2) of this warp's columns c2, shuffled at step lane
    }
    __syncthreads();
    if (n > 0 && g == 0) {
        a[0] *= dinv[0];
        xch[lane] = a[0];
        col_publish(flag);
    }
    for (int c = 0; c + 1 < n; ++c) {
        if (g + NWARP * (QPW - 1) <= c) break;
        T xc;
        if (g == (c & (NWARP - 1))) {
            xc = a[c / NWARP];
        } else {
            col_wait(flag + c, err);
            xc = xch[c * FRONT_TILE + lane];
        }
        const int c1 = c + 1;
        if (g == (c1 & (NWARP - 1))) {
            const int q1 = c1 / NWARP;
            a[q1] -= xc * d[c + c1 * LD];
            a[q1] *= dinv[c1];
            xch[c1 * FRONT_TILE + lane] = a[q1];
            col_publish(flag + c1);
        }
#pragma unroll
        for (int q = 0; q < QPW; ++q) {
            const int c2 = g + NWARP * q;
            if (c2 > c1 && c2 < n) a[q] -= xc * __shfl_sync(0xffffffffu, u[q], c);
        }
    }
#pragma unroll
    for (int q = 0; q < QPW; ++q) x[lane + (g + NWARP * q) * LD] = a[q];
    __syncthreads();
}

// x := L^-1 x with L the unit lower triangle of the n x n tile d.  lane =
// column of x; warp g owns rows g, g + NWARP, ...; xch holds the solved rows.
template <typename T>
__device__ void trsm_u_tile(T* x, const T* d, int n, T* xch, int* flag, int* err) {
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    if (threadIdx.x < FRONT_TILE) flag[threadIdx.x] = 0;
    T a[QPW], l[QPW];
#pragma unroll
    for (int q = 0; q < QPW; ++q) {
        a[q] = x[(g + NWARP * q) + lane * LD];
        l[q] = d[(g + NWARP * q) + lane * LD];  // L(r2, lane) of this warp's rows r2, shuffled at step lane
    }
    __syncthreads();
    if (n > 0 && g == 0) {
        xch[lane] = a[0];  // row 0 is final (unit diagonal)
        col_publish(flag);
    }
    for (int r = 0; r + 1 < n; ++r) {
        if (g + NWARP * (QPW - 1) <= r) break;
        T yr;
        if (g == (r & (NWARP - 1))) {
            yr = a[r / NWARP];
        } else {
            col_wait(flag + r, err);
            yr = xch[r * FRONT_TILE + lane];
        }
        const int r1 = r + 1;
        if (g == (r1 & (NWARP - 1))) {
            const int q1 = r1 / NWARP;
            a[q1] -= d[r1 + r * LD] * yr;
            xch[r1 * FRONT_TILE + lane] = a[q1];
            col_publish(flag + r1);
        }
#pragma unroll
        for (int q = 0; q < QPW; ++q) {
            const int r2 = g + NWARP * q;
            if (r2 > r1 && r2 < n) a[q] -= __shfl_sync(0xffffffffu, l[q], r) * yr;
        }
    }
#pragma unroll
    for (int q = 0; q < QPW; ++q) x[(g + NWARP * q) + lane * LD] = a[q];
    __syncthreads();
}

// c -= l u over the first nk columns of l / rows of u (all tiles zero-padded):
// lane = row, warp w takes columns w, w + NWARP, ...
// busy (may be null): the SM's count of chain tasks computing.  A GEMM reads it
// at step 8 (the load overlaps the FMAs) and, when a chain task was computing,
// pauses at step 16 (bounded, ~8 us) so that the chain task does not share the
// SM's FP64 issue with it.
template <typename T>
__device__ void gemm_tile(T* c, const T* l, const T* u, int nk, int nj, const int* busy = nullptr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T acc[QPW];
#pragma unroll
    for (int q = 0; q < QPW; ++q) acc[q] = (T)0;
    int chain_seen = 0;
    for (int k = 0; k < nk; ++k) {
        if (busy) {
            if (k == 8) chain_seen = *(volatile const int*)busy;
            if (k == 16 && chain_seen > 0)
                for (int it = 0; it < 80 && *(volatile const int*)busy > 0; ++it) __nanosleep(100);
        }
        const T lv = l[lane + k * LD];
#pragma unroll
        for (int q = 0; q < QPW; ++q)
            if (warp + NWARP * q < nj) acc[q] += lv * u[k + (warp + NWARP * q) * LD];
    }
#pragma unroll
    for (int q = 0; q < QPW; ++q) c[lane + (warp + NWARP * q) * LD] -= acc[q];
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(MF_FACTOR_THREADS, MF_FACTOR_CTAS_MAX) mf_factor_kernel(MFArgs a, T* pool) {
    extern __shared__ double smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_task;
    __shared__ int s_col[FRONT_TILE];  // column flags of the tile kernels
    // Tasks on the chain of dependent pivot tiles (GETRF, the diagonal update
    // slices, and the TRSMs of the tiles next to the diagonal) mark their SM
    // while they compute.  A CTA on a marked SM claims nothing new for up to
    // ~20 us, so that the chain task's FP64 instructions do not queue behind a
    // second CTA's (the SM issues one FP64 warp-instruction per ~19 cycles).
    const unsigned my_sm = mf_smid();
    int* busy = my_sm < MF_SM_SLOTS ? a.sm_busy + my_sm : nullptr;
    while (true) {
        if (threadIdx.x == 0) {
            if (busy)
                for (int it = 0; it < 200 && *(volatile int*)busy > 0; ++it) __nanosleep(100);
            s_task = *(volatile int*)a.abort_flag ? a.n_tasks : atomicAdd(a.counter, 1);
        }
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= a.n_tasks) return;
        const int type = a.task_type[t];
        const int S = a.task_front[t];
        const int m = (int)(a.fr_ptr[S + 1] - a.fr_ptr[S]);
        const int w = a.fr_w[S];
        T* FS = pool + a.fr_off[S];
        if (type == TASK_SMALL) {
            if (!wait_children(a, S)) continue;
            assemble_small<T>(a, S, sm, m, pool);
            partial_lu_small<T>(sm, m, w, a.err);
            for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) __stcg(FS + idx, sm[idx]);
            publish(a.done + S, a.epoch);
            continue;
        }
        const int kb = a.fr_kb[S], nb = a.fr_nb[S];
        const long long tb = a.fr_tile0[S];
        int* tv = a.tver + tb;
        const int i = a.task_i[t], j = a.task_j[t], k = a.task_k[t];
        const int k0 = tile_lo(k, kb, w), nk = tile_hi(k, kb, nb, w, m) - k0;
        const int r0 = tile_lo(i, kb, w), nr = tile_hi(i, kb, nb, w, m) - r0;
        const int c0 = tile_lo(j, kb, w), nc = tile_hi(j, kb, nb, w, m) - c0;
        T* T0 = sm;
        T* T1 = sm + TILE_ELEMS;
        T* T2 = sm + 2 * TILE_ELEMS;
        if (type == TASK_GETRF) {
            // The last update of the diagonal tile, A(k,k) -= L(k,k-1) U(k-1,k), is on
            // the chain of dependent pivot tiles and has no GEMM task: GETRF(1) applies
            // it itself (after the first touch of tile (1, 1)), and for k >= 2 it runs
            // as DUPD_SLICES column slices on as many CTAs, whose count GETRF(k) waits
            // for.  A 32 x 32 x 32 update takes ~9 us of one SM's FP64 issue; a slice
            // takes 1 / DUPD_SLICES of that.
            const long long dk = (long long)k * nb + k;
            bool ok;
            if (k == 0) ok = wait_children(a, S);
            else if (k == 1) ok = wait3(a, tv + dk - 1, TILE_FINAL, tv + (long long)(k - 1) * nb + k, TILE_FINAL,
                                        nullptr, 0);
            else ok = wait3(a, a.tcnt + tb + dk, DUPD_SLICES, nullptr, 0, nullptr, 0);
            if (!ok) continue;
            if (threadIdx.x == 0 && busy) atomicAdd(busy, 1);
            if (k == 0) {
                assemble_tile<T>(a, tb, T2, 0, 0, pool);
            } else if (k == 1) {
                const int p0 = tile_lo(k - 1, kb, w), np = tile_hi(k - 1, kb, nb, w, m) - p0;
                TileRegs<T> lt, ut;
                fetch_tile(lt, FS, m, k0, nk, p0, np);
                fetch_tile(ut, FS, m, p0, np, k0, nk);
                put_tile(T0, lt);
                put_tile(T1, ut);
                assemble_tile<T>(a, tb + dk, T2, k0, k0, pool);  // first touch of tile (1, 1)
                __syncthreads();
                gemm_tile<T>(T2, T0, T1, np, nk);
            } else {
                TileRegs<T> dt;
                fetch_tile(dt, FS, m, k0, nk, k0, nk);
                put_tile(T2, dt);
            }
            __syncthreads();
            getrf_tile<T>(T2, nk, a.err, T0, s_col);
            store_tile<T>(FS, T2, m, k0, nk, k0, nk);
            publish(tv + dk, TILE_FINAL);
            if (k == kb - 1 && nb == kb) publish(a.done + S, a.epoch);  // no contribution block
            if (threadIdx.x == 0 && busy) atomicSub(busy, 1);
        } else if (type >= TASK_DUPD) {
            // slice of the last update of diagonal tile (i, i) = (k + 1, k + 1): its
            // columns [cs, cs + DUPD_W) of A(i,i) -= L(i,k) U(k,i); lane = row, warp =
            // column of the slice.  The sum runs in the order of gemm_tile's, so the
            // tile is bit for bit what the fused update gives.
            static_assert(DUPD_W <= NWARP, "at most one slice column per warp");
            const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
            const long long di = (long long)i * nb + i;
            if (!wait3(a, tv + (long long)i * nb + k, TILE_FINAL, tv + (long long)k * nb + i, TILE_FINAL, tv + di, k))
                continue;
            if (threadIdx.x == 0 && busy) atomicAdd(busy, 1);
            const int cs = (type - TASK_DUPD) * DUPD_W;
            const int col = wp < DUPD_W ? cs + wp : FRONT_TILE;  // column of the diagonal tile (warps past the slice: none)
            TileRegs<T> lt;
            fetch_tile(lt, FS, m, r0, nr, k0, nk);
            const T uv = (lane < nk && col < nr) ? __ldcg(FS + (k0 + lane) + (long long)(r0 + col) * m) : (T)0;
            const T cv = (lane < nr && col < nr) ? __ldcg(FS + (r0 + lane) + (long long)(r0 + col) * m) : (T)0;
            put_tile(T0, lt);
            T1[lane + wp * LD] = uv;
            __syncthreads();
            if (col < nr) {  // warp-uniform
                T acc = (T)0;
                for (int q = 0; q < nk; ++q) acc += T0[lane + q * LD] * T1[q + wp * LD];
                if (lane < nr) __stcg(FS + (r0 + lane) + (long long)(r0 + col) * m, cv - acc);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(a.tcnt + tb + di, 1);
                if (busy) atomicSub(busy, 1);
            }
        } else if (type == TASK_TRSM_L || type == TASK_TRSM_U) {
            const int* own = tv + (long long)i * nb + j;
            if (!wait3(a, tv + (long long)k * nb + k, TILE_FINAL, k > 0 ? own : nullptr, k, nullptr, 0)) continue;
            const bool chain = (type == TASK_TRSM_L ? i : j) == k + 1;  // the tile next to the diagonal
            if (chain && threadIdx.x == 0 && busy) atomicAdd(busy, 1);
            TileRegs<T> dt, xt;
            fetch_tile(dt, FS, m, k0, nk, k0, nk);
            if (k > 0) fetch_tile(xt, FS, m, r0, nr, c0, nc);
            put_tile(T0, dt);
            if (k == 0) assemble_tile<T>(a, tb + (long long)i * nb + j, T1, r0, c0, pool);
            else put_tile(T1, xt);
            __syncthreads();
            if (type == TASK_TRSM_L) trsm_l_tile<T>(T1, T0, nk, T2, s_col, a.err);
            else trsm_u_tile<T>(T1, T0, nk, T2, s_col, a.err);
            store_tile<T>(FS, T1, m, r0, nr, c0, nc);
            publish(tv + (long long)i * nb + j, TILE_FINAL);
            if (chain && threadIdx.x == 0 && busy) atomicSub(busy, 1);
        } else {  // TASK_GEMM
            int* own = tv + (long long)i * nb + j;
            if (!wait3(a, tv + (long long)i * nb + k, TILE_FINAL, tv + (long long)k * nb + j, TILE_FINAL,
                       k > 0 ? own : nullptr, k))
                continue;
            TileRegs<T> lt, ut, ct;
            fetch_tile(lt, FS, m, r0, nr, k0, nk);
            fetch_tile(ut, FS, m, k0, nk, c0, nc);
            if (k > 0) fetch_tile(ct, FS, m, r0, nr, c0, nc);
            put_tile(T0, lt);
            put_tile(T1, ut);
            if (k == 0) assemble_tile<T>(a, tb + (long long)i * nb + j, T2, r0, c0, pool);
            else put_tile(T2, ct);
            __syncthreads();
            gemm_tile<T>(T2, T0, T1, nk, nc, busy);
            store_tile<T>(FS, T2, m, r0, nr, c0, nc);
            publish(own, k + 1);
            if (k == kb - 1 && i >= kb && j >= kb && threadIdx.x == 0) {
                // a final tile of the contribution block; the last one completes the front
                const int r = nb - kb;
                if (atomicAdd(a.count + S, 1) == r * r - 1) {
                    __threadfence();
                    st_rel(a.done + S, a.epoch);
                }
            }
        }
    }
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
    const long long* fg_ptr;   // per front row: children's update entries, in child order
    const long long* fg_src;
    const int* q;          // B index of each permuted M index
    const double* cscale;  // column scaling of a weighted matching, by B index (null: none)
    const int* order;      // claim order of the fronts
    int n_small;           // fronts solved one per warp: order[0, n_small) forward, order[ns - n_small, ns) backward
    int* flags;            // fwd [ns], bwd [ns]
    int* counter;
    int* counter_small;
    int* abort_flag;
    int* err;
    int epoch;
    unsigned spin_limit;
};

// s = sum over p in [p0, p1), ascending, of F[i + p m] u[p].  A full block of 32
// pivots issues all 32 loads of the row before the first FMA, so one L2 round
// trip, not four, precedes the chain of dependent FMAs; the sum's order is
// the same either way.
template <typename T>
__device__ __forceinline__ T block_dot(const T* __restrict__ F, long long m, int i, int p0, int p1, const T* u) {
    T s = (T)0;
    if (p1 - p0 == 32) {
        T f[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) f[q] = F[i + (long long)(p0 + q) * m];
#pragma unroll
        for (int q = 0; q < 32; ++q) s += f[q] * u[p0 + q];
    } else {
#pragma unroll 8
        for (int p = p0; p < p1; ++p) s += F[i + (long long)p * m] * u[p];
    }
    return s;
}

// One warp solves a front of order m <= 32 (lane = row): forward with its
// unit-lower columns, the update vector for the parent in the same pass.
template <typename T>
__device__ void fwd_small_warp(const MFSolveArgs& a, int S, const T* __restrict__ pool, const T* __restrict__ rhs,
                               T* y, T* cv, int lane) {
    int* const fdone = a.flags;
    bool ok = true;
    for (int q = a.ch_ptr[S] + lane; q < a.ch_ptr[S + 1]; q += 32)
        ok = ok && wait_eq(fdone + a.ch_idx[q], a.epoch, a.abort_flag, a.err, a.spin_limit);
    if (!__all_sync(0xffffffffu, ok)) return;
    const int m = (int)(a.fr_ptr[S + 1] - a.fr_ptr[S]);
    const int w = a.fr_w[S];
    const int* idx = a.fr_idx + a.fr_ptr[S];
    const T* F = pool + a.fr_off[S];
    const long long* gp = a.fg_ptr + a.fr_ptr[S];
    T u = (T)0;
    if (lane < m) {
        u = lane < w ? rhs[idx[lane]] : (T)0;
#pragma unroll 4
        for (long long e = gp[lane]; e < gp[lane + 1]; ++e) u += __ldcg(cv + a.fg_src[e]);
    }
    for (int p = 0; p < w; ++p) {
        const T yp = __shfl_sync(0xffffffffu, u, p);
        if (lane > p && lane < m) u -= F[lane + (long long)p * m] * yp;
    }
    if (lane < m) {
        if (lane < w) y[idx[lane]] = u;
        else cv[a.cv_off[S] + (lane - w)] = u;
    }
    __syncwarp();
    if (lane == 0) {
        __threadfence();
        st_rel(fdone + S, a.epoch);
    }
}

// One warp solves a front of order m <= 32 (lane = row): z = y - U12 x_tail,
// then back substitution with the upper diagonal block.
template <typename T>
__device__ void bwd_small_warp(const MFSolveArgs& a, int S, const T* __restrict__ pool, const T* __restrict__ y,
                               T* xs, double* xout, int lane) {
    int* const bdone = a.flags + a.ns;
    const int P = a.sn_parent[S];
    bool ok = true;
    if (lane == 0 && P >= 0) ok = wait_eq(bdone + P, a.epoch, a.abort_flag, a.err, a.spin_limit);
    if (!__shfl_sync(0xffffffffu, ok, 0)) return;
    const int m = (int)(a.fr_ptr[S + 1] - a.fr_ptr[S]);
    const int w = a.fr_w[S];
    const int* idx = a.fr_idx + a.fr_ptr[S];
    const T* F = pool + a.fr_off[S];
    const T xt = lane < m - w ? __ldcg(xs + idx[w + lane]) : (T)0;
    T z = (T)0;
    T s = (T)0;
    for (int j = 0; j < m - w; ++j) {
        const T xj = __shfl_sync(0xffffffffu, xt, j);
        if (lane < w) s += F[lane + (long long)(w + j) * m] * xj;
    }
    if (lane < w) z = y[idx[lane]] - s;
    const T dinv = lane < w ? (T)1 / F[lane + (long long)lane * m] : (T)0;
    for (int p = w - 1; p >= 0; --p) {
        if (lane == p) z *= dinv;
        const T xp = __shfl_sync(0xffffffffu, z, p);
        if (lane < p) z -= F[lane + (long long)p * m] * xp;
    }
    if (lane < w) {
        xs[idx[lane]] = z;
        const int col = a.q[idx[lane]];
        xout[col] = a.cscale ? (double)z * a.cscale[col] : (double)z;
    }
    __syncwarp();
    if (lane == 0) {
        __threadfence();
        st_rel(bdone + S, a.epoch);
    }
}

// Forward: L y = rhs.  Each front adds its children's update vectors (child
// order), solves with its unit-lower diagonal block 32 pivots at a time (one
// warp, register shuffles) and updates the rows below with the same columns.
// Subtrees of small fronts come first, one front per warp; then the CTAs take
// the remaining fronts one at a time.
template <typename T>
__global__ void __launch_bounds__(MF_THREADS) mf_fwd_kernel(MFSolveArgs a, const T* __restrict__ pool,
                                                            const T* __restrict__ rhs, T* y, T* cv) {
    extern __shared__ double smem_raw[];
    T* u = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_S;
    int* const fdone = a.flags;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    while (true) {
        int c = 0;
        if (lane == 0) c = *(volatile int*)a.abort_flag ? a.n_small : atomicAdd(a.counter_small, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= a.n_small) break;
        fwd_small_warp<T>(a, a.order[c], pool, rhs, y, cv, lane);
    }
    __syncthreads();
    while (true) {
        if (threadIdx.x == 0) {
            const int c = *(volatile int*)a.abort_flag ? a.ns : a.n_small + atomicAdd(a.counter, 1);
            s_S = c < a.ns ? a.order[c] : a.ns;
        }
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
        {
            const long long* gp = a.fg_ptr + a.fr_ptr[S];
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                T v = i < w ? rhs[idx[i]] : (T)0;
                // several entries' index and value loads in flight; the sum keeps child order
#pragma unroll 4
                for (long long e = gp[i]; e < gp[i + 1]; ++e) v += __ldcg(cv + a.fg_src[e]);
                u[i] = v;
            }
        }
        __syncthreads();
        for (int p0 = 0; p0 < w; p0 += 32) {
            const int p1 = min(p0 + 32, w);
            if (warp == 0) {
                // lane r - p0 holds row r of the unit-lower block; its L entries are loaded up front
                const int r = p0 + lane;
                T val = r < p1 ? u[r] : (T)0;
                const int nbk = p1 - p0;
                T lrow[32];
#pragma unroll
                for (int q = 0; q < 32; ++q) lrow[q] = (r < p1 && p0 + q < r) ? F[r + (long long)(p0 + q) * m] : (T)0;
#pragma unroll
                for (int q = 0; q < 31; ++q)
                    if (q < nbk - 1) val -= lrow[q] * __shfl_sync(0xffffffffu, val, q);
                if (r < p1) u[r] = val;
            }
            __syncthreads();
            for (int i = p1 + threadIdx.x; i < m; i += blockDim.x) u[i] -= block_dot<T>(F, m, i, p0, p1, u);
            __syncthreads();
        }
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (i < w) y[idx[i]] = u[i];
            else cv[a.cv_off[S] + (i - w)] = u[i];
        }
        publish(fdone + S, a.epoch);
    }
}

// Backward: U x = y from the root down; a front needs only its parent done
// (its tail indices are pivots of ancestors).  z = y - U12 x_tail, then the
// upper diagonal block 32 pivots at a time from the bottom.
template <typename T>
__global__ void __launch_bounds__(MF_THREADS) mf_bwd_kernel(MFSolveArgs a, const T* __restrict__ pool,
                                                            const T* __restrict__ y, T* xs, double* xout) {
    extern __shared__ double smem_raw[];
    T* z = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_S;
    int* const bdone = a.flags + a.ns;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n_big = a.ns - a.n_small;
    while (true) {
        if (threadIdx.x == 0) s_S = *(volatile int*)a.abort_flag ? n_big : atomicAdd(a.counter, 1);
        __syncthreads();
        const int c = s_S;
        __syncthreads();
        if (c >= n_big) break;
        const int S = a.order[c];
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
        // z = y_S - U12 x_tail: one pivot row per thread, coalesced down each column
        {
            // P lanes over pivot rows (coalesced down each column), G groups over tail columns;
            // the G partial sums of a row are added in group order.  G is capped so that a
            // group covers at least 8 tail columns: the sum of the partial sums is a chain of
            // G dependent adds (64 cycles each), which for a one-pivot front with 512 groups
            // took longer than the rest of its solve.
            int P = 32;
            while (P > 1 && P / 2 >= w) P >>= 1;
            const int G = max(1, min(MF_THREADS / P, (m - w + 7) / 8));
            T* part = z + m;  // [G][w]
            const int pl = threadIdx.x % P, g = threadIdx.x / P;
            if (g < G)
                for (int p = pl; p < w; p += P) {
                    T s = (T)0;
#pragma unroll 4
                    for (int j = g; j < m - w; j += G) s += F[p + (long long)(w + j) * m] * xt[j];
                    part[g * w + p] = s;
                }
            __syncthreads();
            for (int p = threadIdx.x; p < w; p += blockDim.x) {
                T s = (T)0;
                for (int q = 0; q < G; ++q) s += part[q * w + p];
                z[p] = y[idx[p]] - s;
            }
        }
        __syncthreads();
        for (int p1 = w; p1 > 0; p1 -= 32) {
            const int p0 = max(p1 - 32, 0);
            if (warp == 0) {
                // lane r - p0 holds row r of the upper block (diagonal included), loaded up front
                const int r = p0 + lane;
                T val = r < p1 ? z[r] : (T)0;
                const int nbk = p1 - p0;
                T urow[32];
#pragma unroll
                for (int q = 0; q < 32; ++q)
                    urow[q] = (r < p1 && p0 + q < p1 && p0 + q > r) ? F[r + (long long)(p0 + q) * m] : (T)0;
                // every lane divides once, in parallel: x_r = (z_r - sum_{q > r} U(r,q) x_q) / U(r,r)
                const T dinv = r < p1 ? (T)1 / F[r + (long long)r * m] : (T)0;
#pragma unroll
                for (int q = 31; q >= 0; --q) {
                    if (q < nbk) {
                        if (lane == q) val *= dinv;
                        const T xp = __shfl_sync(0xffffffffu, val, q);
                        if (lane < q) val -= urow[q] * xp;
                    }
                }
                if (r < p1) z[r] = val;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < p0; i += blockDim.x) z[i] -= block_dot<T>(F, m, i, p0, p1, z);
            __syncthreads();
        }
        for (int p = threadIdx.x; p < w; p += blockDim.x) {
            xs[idx[p]] = z[p];
            const int col = a.q[idx[p]];
            xout[col] = a.cscale ? (double)z[p] * a.cscale[col] : (double)z[p];
        }
        publish(bdone + S, a.epoch);
    }
    while (true) {
        int c = 0;
        if (lane == 0) c = *(volatile int*)a.abort_flag ? a.n_small : atomicAdd(a.counter_small, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= a.n_small) break;
        bwd_small_warp<T>(a, a.order[n_big + c], pool, y, xs, xout, lane);
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

int sm_count() {
    static const int sms = [] {  // initialised once, thread-safe
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return std::max(1, n);
    }();
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
    a.fr_kb = L.d_fr_kb.p;
    a.fr_nb = L.d_fr_nb.p;
    a.fr_tile0 = L.d_fr_tile0.p;
    a.tasm_ptr = L.d_tasm_ptr.p;
    a.tasm_e = L.d_tasm_e.p;
    a.tasm_pos = L.d_tasm_pos.p;
    a.tch_ptr = L.d_tch_ptr.p;
    a.tch = L.d_tch.p;
    a.task_type = L.d_task_type.p;
    a.task_front = L.d_task_front.p;
    a.task_i = L.d_task_i.p;
    a.task_j = L.d_task_j.p;
    a.task_k = L.d_task_k.p;
    a.n_tasks = (int)L.task_type.size();
    a.A = A;
    a.done = L.d_mf_flags.p;
    a.count = L.d_mf_count.p;
    a.tver = L.d_tver.p;
    a.tcnt = L.d_tver.p + L.n_tiles;
    a.sm_busy = L.d_counters.p + 8;
    a.counter = L.d_counters.p;
    a.abort_flag = L.d_counters.p + 3;
    a.err = &c.d_status.p->dev_err;
    a.spin_limit = 1u << 22;
    return a;
}

template <typename T>
static void mf_factor_t(Circuit& c, const double* A, T* pool, cudaStream_t s) {
    SparseLU& L = c.lu;
    const int smem = MF_SMEM_ELEMS * (int)sizeof(T);
    // flags start at 0 and a finished front is marked 1 (a fixed epoch): every launch
    // resets them, so the launch replays unchanged inside a captured graph
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 4 * sizeof(int), s));
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p + 8, 0, MF_SM_SLOTS * sizeof(int), s));
    VGB_CUDA(cudaMemsetAsync(L.d_mf_flags.p, 0, std::max(L.nsn, 1) * sizeof(int), s));
    VGB_CUDA(cudaMemsetAsync(L.d_mf_count.p, 0, std::max(L.nsn, 1) * sizeof(int), s));
    if (L.n_tiles) VGB_CUDA(cudaMemsetAsync(L.d_tver.p, 0, 2 * L.n_tiles * sizeof(int), s));
    MFArgs a = mf_args(c, A);
    a.epoch = 1;
    const int blocks = std::min(sm_count() * std::min(std::max(c.tune_factor_ctas, 1), MF_FACTOR_CTAS_MAX),
                                std::max(a.n_tasks, 1));
    mf_factor_kernel<T><<<blocks, MF_FACTOR_THREADS, smem, s>>>(a, pool);
    VGB_CUDA(cudaGetLastError());
}

void mf_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s) {
    if (c.lu.nsn == 0) return;
    if (fp32) mf_factor_t<float>(c, A, c.lu.d_pool32.p, s);
    else mf_factor_t<double>(c, A, c.lu.d_pool64.p, s);
}

// bwd: z and x_tail (m) plus the partial sums of U12 x_tail ([G][w] with G = MF_THREADS / P
// groups of P lanes, P >= min(w, 32): at most (MF_THREADS / 32) w + MF_THREADS <= (MF_THREADS / 32) m
// + MF_THREADS); fwd uses m
template <typename T>
static size_t mf_solve_smem(const SparseLU& L) {
    return (size_t)((1 + MF_THREADS / 32) * std::max<long long>(L.mf_max_m, 1) + MF_THREADS) * sizeof(T);
}

// Opt the solve kernels in to more than 48 KB of dynamic shared memory (once per size).
// Circuits on several host threads (the server) may get here at once: the cache is locked.
template <typename T>
static void mf_solve_attributes(size_t smem) {
    static std::mutex mu;
    static size_t smem_set[2] = {0, 0};
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = smem_set[sizeof(T) == 4 ? 0 : 1];
    if (smem > 48 * 1024 && smem > cur) {
        VGB_REQUIRE(smem <= 200 * 1024, "front too large for the solve kernels' shared memory");
        VGB_CUDA(cudaFuncSetAttribute(mf_fwd_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        VGB_CUDA(cudaFuncSetAttribute(mf_bwd_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        cur = smem;
    }
}

// Everything the solve launches need set up outside a stream capture.
void mf_prepare_capture(Circuit& c) {
    (void)sm_count();
    if (c.lu.nsn == 0) return;
    mf_solve_attributes<double>(mf_solve_smem<double>(c.lu));
    mf_solve_attributes<float>(mf_solve_smem<float>(c.lu));
}

template <typename T>
void mf_solve_t(Circuit& c, const T* rhsM, T* y, T* xs, double* xout, cudaStream_t s) {
    SparseLU& L = c.lu;
    if (L.nsn == 0) return;
    const T* pool = std::is_same<T, float>::value ? (const T*)L.d_pool32.p : (const T*)L.d_pool64.p;
    T* cv = std::is_same<T, float>::value ? (T*)L.d_cv32.p : (T*)L.d_cv64.p;
    VGB_CUDA(cudaMemsetAsync(L.d_counters.p, 0, 8 * sizeof(int), s));
    VGB_CUDA(cudaMemsetAsync(L.d_mf_flags.p + 2 * (size_t)L.nsn, 0, 2 * (size_t)L.nsn * sizeof(int), s));
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
    a.fg_ptr = L.d_fg_ptr.p;
    a.fg_src = L.d_fg_src.p;
    a.q = L.d_q.p;
    a.cscale = L.d_cscale.p;
    a.n_small = L.n_small_solve;
    a.flags = L.d_mf_flags.p + 2 * (size_t)L.nsn;
    a.counter = L.d_counters.p + 1;
    a.abort_flag = L.d_counters.p + 3;
    a.err = &c.d_status.p->dev_err;
    a.epoch = 1;
    a.spin_limit = 1u << 22;
    const size_t smem = mf_solve_smem<T>(L);
    mf_solve_attributes<T>(smem);
    const int blocks = std::min(sm_count() * std::max(c.tune_solve_ctas, 1), L.nsn);
    a.order = L.d_fwd_order.p;
    a.counter_small = L.d_counters.p + 4;
    mf_fwd_kernel<T><<<blocks, MF_THREADS, smem, s>>>(a, pool, rhsM, y, cv);
    a.counter = L.d_counters.p + 2;
    a.counter_small = L.d_counters.p + 5;
    a.order = L.d_bwd_order.p;
    mf_bwd_kernel<T><<<blocks, MF_THREADS, smem, s>>>(a, pool, y, xs, xout);
    VGB_CUDA(cudaGetLastError());
}

template void mf_solve_t<double>(Circuit&, const double*, double*, double*, double*, cudaStream_t);
template void mf_solve_t<float>(Circuit&, const float*, float*, float*, double*, cudaStream_t);

}  // namespace vgb
