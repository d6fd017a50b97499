// Dense linear solve of a small circuit with no allocation: the working matrix
// lives in a file-scope __device__ array instead of memory allocated per call.
//
// Some callers may not allocate device memory while they run: an XLA custom
// call, whose buffers all come from XLA's own allocator that already holds
// most of the GPU, or a host that reserves all device memory up front for its
// own pool.  This entry point lets them solve small systems with only the
// buffers they pass in.
//
// J x = rhs is scattered from the circuit's CSR values into a dense
// column-major matrix in that array and solved by LU with partial pivoting in
// one CTA.  The set-up (looking up the array's device address with
// cudaGetSymbolAddress) runs once per device, on the first call made with that
// device current; the address is cached for the life of the process, so it
// does not survive a cudaDeviceReset.  Nothing in the array needs to start at
// zero: every call writes all n x n entries before reading them.  Calls that
// overlap in time on one device (other streams or host threads) share the
// array and race.
#include <mutex>

#include "vgb_core.h"

namespace vgb {

namespace {

constexpr int DENSE_THREADS = 256;

__device__ __align__(256) double g_dense_scratch[VGB_DENSE_STATIC_MAX * VGB_DENSE_STATIC_MAX];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
double* g_scratch_ptr[MAX_DEVICES] = {};

double* scratch_for_current_device() {
    int dev = 0;
    VGB_CUDA(cudaGetDevice(&dev));
    VGB_REQUIRE(dev >= 0 && dev < MAX_DEVICES, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_dense_scratch);
        if (e != cudaSuccess || !p)
            throw Error(VGB_ERR_CUDA, std::string("cudaGetSymbolAddress(dense scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    return g_scratch_ptr[dev];
}

__global__ void __launch_bounds__(DENSE_THREADS) dense_static_solve_kernel(int n, const int* __restrict__ indptr,
                                                                         const int* __restrict__ indices,
                                                                         const double* __restrict__ vals,
                                                                         const double* __restrict__ rhs, double* x,
                                                                         double* M, int* err, int* info) {
    __shared__ double b[VGB_DENSE_STATIC_MAX];
    __shared__ double r_val[DENSE_THREADS];
    __shared__ int r_idx[DENSE_THREADS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = DENSE_THREADS / 32;
    int first_bad = 0;  // LAPACK getrf convention: 1 + column of the first zero or non-finite pivot
    for (int t = tid; t < n * n; t += DENSE_THREADS) M[t] = 0.0;
    for (int i = tid; i < n; i += DENSE_THREADS) b[i] = rhs[i];
    __syncthreads();
    for (int r = warp; r < n; r += nw)
        for (int e = indptr[r] + lane; e < indptr[r + 1]; e += 32) M[r + indices[e] * n] = vals[e];
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        // pivot row: largest |M(i, k)|, i >= k (ties: smallest i)
        double best = -1.0;
        int bi = k;
        for (int i = k + tid; i < n; i += DENSE_THREADS) {
            const double v = fabs(M[i + k * n]);
            if (v > best) { best = v; bi = i; }
        }
        r_val[tid] = best;
        r_idx[tid] = bi;
        __syncthreads();
        for (int o = DENSE_THREADS / 2; o; o >>= 1) {
            if (tid < o) {
                const double v2 = r_val[tid + o];
                const int i2 = r_idx[tid + o];
                if (v2 > r_val[tid] || (v2 == r_val[tid] && i2 < r_idx[tid])) { r_val[tid] = v2; r_idx[tid] = i2; }
            }
            __syncthreads();
        }
        const int p = r_idx[0];
        if (p != k) {
            for (int j = tid; j < n; j += DENSE_THREADS) {
                const double t = M[k + j * n];
                M[k + j * n] = M[p + j * n];
                M[p + j * n] = t;
            }
            if (tid == 0) {
                const double t = b[k];
                b[k] = b[p];
                b[p] = t;
            }
        }
        __syncthreads();
        double piv = M[k + k * n];
        if (piv == 0.0 || !isfinite(piv)) {
            piv = 1e-30;
            __syncthreads();
            if (tid == 0) {
                M[k + k * n] = piv;
                if (err) atomicOr(err, DEV_ERR_PIVOT);
                if (!first_bad) first_bad = k + 1;
            }
        }
        for (int i = k + 1 + tid; i < n; i += DENSE_THREADS) M[i + k * n] /= piv;
        __syncthreads();
        for (int j = k + 1 + warp; j < n; j += nw) {
            const double u = M[k + j * n];
            for (int i = k + 1 + lane; i < n; i += 32) M[i + j * n] -= M[i + k * n] * u;
        }
        __syncthreads();
    }
    // L y = P b (unit lower), then U x = y
    for (int k = 0; k < n; ++k) {
        const double yk = b[k];
        for (int i = k + 1 + tid; i < n; i += DENSE_THREADS) b[i] -= M[i + k * n] * yk;
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
        if (tid == 0) b[k] /= M[k + k * n];
        __syncthreads();
        const double xk = b[k];
        for (int i = tid; i < k; i += DENSE_THREADS) b[i] -= M[i + k * n] * xk;
        __syncthreads();
    }
    for (int i = tid; i < n; i += DENSE_THREADS) x[i] = b[i];
    if (info && tid == 0) *info = first_bad;
}

}  // namespace

// The same dense LU with partial pivoting on a caller-owned matrix buffer
// (the per-circuit dense solver of small circuits).
void launch_dense_solve(int n, const int* indptr, const int* indices, const double* vals, const double* rhs,
                        double* x, double* M, int* err, cudaStream_t s) {
    if (n > 0) dense_static_solve_kernel<<<1, DENSE_THREADS, 0, s>>>(n, indptr, indices, vals, rhs, x, M, err, nullptr);
}

}  // namespace vgb

using namespace vgb;

extern "C" int vgb_linear_solve_dense_static(void* h, const double* csr_vals, const double* rhs, double* x,
                                             int* info, vgb_stream_t stream) {
    Circuit* c = static_cast<Circuit*>(h);
    if (!c) return VGB_ERR_INVALID;
    try {
        if (!c->finalized) throw Error(VGB_ERR_STATE, "circuit is not finalized");
        VGB_REQUIRE(csr_vals && rhs && x, "csr_vals, rhs and x are required");
        if (c->n_aug > VGB_DENSE_STATIC_MAX)
            throw Error(VGB_ERR_INVALID, "vgb_linear_solve_dense_static: n_aug = " + std::to_string(c->n_aug) +
                                             " exceeds the static scratch limit of " +
                                             std::to_string(VGB_DENSE_STATIC_MAX) + " unknowns");
        cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
        if (c->n_aug == 0) {
            if (info) VGB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
            return VGB_OK;
        }
        double* M = scratch_for_current_device();
        dense_static_solve_kernel<<<1, DENSE_THREADS, 0, s>>>(c->n_aug, c->d_indptr.p, c->d_indices.p, csr_vals, rhs,
                                                              x, M, nullptr, info);
        VGB_CUDA(cudaGetLastError());
        c->launches += 1;
        return VGB_OK;
    } catch (const Error& e) {
        c->last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        c->last_error = e.what();
        return VGB_ERR_INVALID;
    }
}
