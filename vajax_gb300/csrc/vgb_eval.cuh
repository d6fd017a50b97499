// Kernel skeleton for generated device models.
//
// One thread evaluates one instance: it gathers the instance's node voltages
// through the node map, reads its parameters (shared across the group or
// per instance, struct-of-arrays), runs the generated model body and writes
// the per-instance contributions that the assembly pass gathers into the CSR
// values and the residual vectors.  No atomics: every output has exactly one
// writer, which keeps stamping deterministic.
//
// Contribution layout of a group with n instances, NJ Jacobian entries and
// NN model nodes (slot-major, so each store is coalesced across the warp):
//   slot k < NJ           : jac_resist[k] + c0 * jac_react[k]   (NaN -> 0)
//   slot NJ + r           : residual_resist[r]
//   slot NJ + NN + r      : residual_react[r]
// This mirrors the reference's per-model stamping step
// (vajax/analysis/mna_builder.py:927-966), which forms jac_r + c0*jac_c,
// masks NaN to 0 and scatter-adds into the CSR data and the dense vectors.
#pragma once

#include <type_traits>

#include "vgb_common.cuh"

namespace vgb {

struct GroupArgs {
    int n_dev;
    const int* __restrict__ node_map;     // [NN][n_dev] circuit node index, 0 = ground
    const double* __restrict__ shared;    // [NP] parameter values common to the group
    const int* __restrict__ vidx;         // [NP] -1 = shared, else column in `varying`
    const double* __restrict__ varying;   // [n_var][n_dev]
    const double* __restrict__ temperature; // [n_dev] or nullptr (use temp_shared)
    double temp_shared;
    double* __restrict__ contrib;         // [NJ + 2 NN][n_dev]
    long long batch_stride_x;             // stride of X between circuit replicas (batched mode)
    int inst_per_replica;                 // instances per replica (batched mode), else n_dev
    const double* __restrict__ cache;     // [NCACHE][n_dev] parameter-only values, or nullptr
};

// Models whose generated struct carries a cache program (codegen/coop.py):
// the values of the body that depend on parameters and temperature only are
// computed once per instance (cache_kernel) and read by every evaluation
// through eval_cached.
template <class M, class = void>
struct HasCache : std::false_type {};
template <class M>
struct HasCache<M, std::void_t<decltype(M::NCACHE)>> : std::true_type {};

// Reader / writer of one instance's cache column, [NCACHE][n] layout.
struct CacheCol {
    const double* c;
    size_t n, i;
    __device__ __forceinline__ double operator()(int k) const { return __ldg(c + (size_t)k * n + i); }
    __device__ __forceinline__ bool b(int k) const { return __double_as_longlong(__ldg(c + (size_t)k * n + i)) != 0; }
};
struct CacheColW {
    double* c;
    size_t n, i;
    __device__ __forceinline__ void operator()(int k, double v) const { c[(size_t)k * n + i] = v; }
};

// Named barrier of the warps that share one cooperative model evaluation
// (generated coop_w* members): `threads` = 32 x warps of the group, ids from 1
// (0 is __syncthreads).  Every warp of the group executes the same barriers
// in the same order: the cooperative body is straight-line code.  The
// non-aligned form counts threads one by one, so a warp still diverged after
// a library fallback inside a math function arrives correctly.
__device__ __forceinline__ void vgb_coop_bar(int id, int threads) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// The group's exchange slots: a shared-memory address (this lane's column of
// 32-double slots) and volatile accesses at constant offsets (doubles), so
// that the compiler neither forwards a warp's own store to a later load of
// the same slot (another warp may have rewritten it after a barrier) nor
// moves an access across a barrier.
typedef unsigned vgb_xs_t;
__device__ __forceinline__ vgb_xs_t vgb_xs_base(const double* p) {
    return (vgb_xs_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ double vgb_xs_ld(vgb_xs_t xs, int off) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(xs + 8u * (unsigned)off) : "memory");
    return v;
}
__device__ __forceinline__ void vgb_xs_st(vgb_xs_t xs, int off, double v) {
    asm volatile("st.shared.f64 [%0], %1;" ::"r"(xs + 8u * (unsigned)off), "d"(v) : "memory");
}
__device__ __forceinline__ bool vgb_xs_ldb(vgb_xs_t xs, int off) {
    unsigned v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(xs + 8u * (unsigned)off) : "memory");
    return v != 0u;
}
__device__ __forceinline__ void vgb_xs_stb(vgb_xs_t xs, int off, bool b) {
    asm volatile("st.shared.u32 [%0], %1;" ::"r"(xs + 8u * (unsigned)off), "r"(b ? 1u : 0u) : "memory");
}

template <class M>
struct ParamReader {
    const GroupArgs& g;
    int i;
    __device__ __forceinline__ double operator()(int k) const {
        int v = __ldg(g.vidx + k);
        return v < 0 ? __ldg(g.shared + k) : __ldg(g.varying + (size_t)v * g.n_dev + i);
    }
};

// One instance's model body: the cached one when the group has a cache.
template <class M, class PF>
__device__ __forceinline__ void eval_instance(const GroupArgs& g, int i, const PF& P, double T, const double* V,
                                              double* rr, double* rq, double* jr, double* jq) {
    if constexpr (HasCache<M>::value) {
        if (g.cache) {
            M::eval_cached(P, CacheCol{g.cache, (size_t)g.n_dev, (size_t)i}, T, V, rr, rq, jr, jq);
            return;
        }
    }
    M::eval(P, T, V, rr, rq, jr, jq);
}

// The cache program, one thread per instance.
template <class M>
__global__ void __launch_bounds__(128) cache_kernel(GroupArgs g, double* cache) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n_dev) return;
    const double T = g.temperature ? __ldg(g.temperature + i) : g.temp_shared;
    ParamReader<M> P{g, i};
    M::cache(P, T, CacheColW{cache, (size_t)g.n_dev, (size_t)i});
}

// Device evaluation is FP64-pipe bound: small blocks spread the instances over
// every SM instead of packing them onto a few.  The block size is a launch
// parameter (default 64) that the autotuner may change; EVAL_BLOCK_MAX bounds it.
constexpr int EVAL_BLOCK = 64;
constexpr int EVAL_BLOCK_MAX = 256;

template <class M>
__global__ void __launch_bounds__(EVAL_BLOCK_MAX) eval_kernel(GroupArgs g, const double* __restrict__ X,
                                                              const double* __restrict__ kdev)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n_dev) return;
    const double c0 = __ldg(kdev);  // Newton coefficient c0, in device memory
    const double* Xr = X;
    if (g.batch_stride_x) Xr = X + (long long)(i / g.inst_per_replica) * g.batch_stride_x;
    double V[M::NN];
#pragma unroll
    for (int t = 0; t < M::NN; ++t) V[t] = Xr[__ldg(g.node_map + (size_t)t * g.n_dev + i)];
    const double T = g.temperature ? __ldg(g.temperature + i) : g.temp_shared;
    double rr[M::NN], rq[M::NN], jr[M::NJ > 0 ? M::NJ : 1], jq[M::NJ > 0 ? M::NJ : 1];
    ParamReader<M> P{g, i};
    eval_instance<M>(g, i, P, T, V, rr, rq, jr, jq);
    const size_t n = g.n_dev;
#pragma unroll
    for (int k = 0; k < M::NJ; ++k) g.contrib[k * n + i] = nan0(jr[k] + c0 * jq[k]);
#pragma unroll
    for (int r = 0; r < M::NN; ++r) {
        g.contrib[(M::NJ + r) * n + i] = rr[r];
        g.contrib[(M::NJ + M::NN + r) * n + i] = rq[r];
    }
}

// Raw per-instance outputs (no c0 combination) for parity tests of the model body.
template <class M>
__global__ void __launch_bounds__(128) eval_raw_kernel(GroupArgs g, const double* __restrict__ X,
                                                       double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n_dev) return;
    double V[M::NN];
#pragma unroll
    for (int t = 0; t < M::NN; ++t) V[t] = X[__ldg(g.node_map + (size_t)t * g.n_dev + i)];
    const double T = g.temperature ? __ldg(g.temperature + i) : g.temp_shared;
    double rr[M::NN], rq[M::NN], jr[M::NJ > 0 ? M::NJ : 1], jq[M::NJ > 0 ? M::NJ : 1];
    ParamReader<M> P{g, i};
    eval_instance<M>(g, i, P, T, V, rr, rq, jr, jq);
    const size_t n = g.n_dev;
    for (int r = 0; r < M::NN; ++r) {
        out[(size_t)r * n + i] = rr[r];
        out[(size_t)(M::NN + r) * n + i] = rq[r];
    }
    for (int k = 0; k < M::NJ; ++k) {
        out[(size_t)(2 * M::NN + k) * n + i] = jr[k];
        out[(size_t)(2 * M::NN + M::NJ + k) * n + i] = jq[k];
    }
}

struct ModelEntry {
    const char* name;
    int nn, nj, np;
    const int* jrow;
    const int* jcol;
    void (*launch)(const GroupArgs&, const double* X, const double* kdev, int block, cudaStream_t s);
    void (*launch_raw)(const GroupArgs&, const double* X, double* out, cudaStream_t s);
    int ncache;  // cache values per instance, 0 without a cache program
    void (*launch_cache)(const GroupArgs&, double* cache, cudaStream_t s);
};

template <class M>
void launch_eval(const GroupArgs& g, const double* X, const double* kdev, int block, cudaStream_t s)
{
    if (g.n_dev == 0) return;
    eval_kernel<M><<<ceil_div(g.n_dev, block), block, 0, s>>>(g, X, kdev);
}

template <class M>
void launch_eval_raw(const GroupArgs& g, const double* X, double* out, cudaStream_t s)
{
    if (g.n_dev == 0) return;
    eval_raw_kernel<M><<<ceil_div(g.n_dev, 128), 128, 0, s>>>(g, X, out);
}

template <class M>
void launch_cache(const GroupArgs& g, double* cache, cudaStream_t s)
{
    if constexpr (HasCache<M>::value) {
        if (g.n_dev == 0) return;
        cache_kernel<M><<<ceil_div(g.n_dev, 128), 128, 0, s>>>(g, cache);
    }
}

template <class M>
ModelEntry make_model_entry(const char* name)
{
    int ncache = 0;
    if constexpr (HasCache<M>::value) ncache = M::NCACHE;
    return ModelEntry{name, M::NN, M::NJ, M::NP, M::JROW, M::JCOL, &launch_eval<M>, &launch_eval_raw<M>,
                      ncache, &launch_cache<M>};
}

// Defined in the generated translation unit.
const ModelEntry* model_table(int* count);

} // namespace vgb
