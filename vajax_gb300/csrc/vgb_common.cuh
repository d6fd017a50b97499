// Shared helpers of the vajax_gb300 CUDA runtime.
#pragma once

#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <stdexcept>

#include "vajax_gb300.h"  // status codes VGB_OK, VGB_ERR_*

namespace vgb {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define VGB_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess)                                                           \
            throw ::vgb::Error(VGB_ERR_CUDA, std::string(#call) + ": " +          \
                                                     cudaGetErrorString(_e));            \
    } while (0)

#define VGB_REQUIRE(cond, msg)                                                           \
    do {                                                                                 \
        if (!(cond)) throw ::vgb::Error(VGB_ERR_INVALID, (msg));                   \
    } while (0)

// Safe math with the reference code generator's semantics.
__host__ __device__ __forceinline__ double vgb_sdiv(double a, double b) {
    return b == 0.0 ? 0.0 : a / b;
}
__host__ __device__ __forceinline__ double vgb_fmin(double a, double b) {
    return (a != a || b != b) ? (a + b) : (a < b ? a : b);
}
__host__ __device__ __forceinline__ double vgb_fmax(double a, double b) {
    return (a != a || b != b) ? (a + b) : (a > b ? a : b);
}
__host__ __device__ __forceinline__ double vgb_fmod_floor(double a, double b) {
    double r = fmod(a, b);
    if (r != 0.0 && ((r < 0.0) != (b < 0.0))) r += b;
    return r;
}
__host__ __device__ __forceinline__ double nan0(double x) { return x != x ? 0.0 : x; }

inline int ceil_div(long long a, int b) { return (int)((a + b - 1) / b); }

// Error flag bits written by device code (never trap).
enum DevErr : int {
    DEV_ERR_TIMEOUT = 1,
    DEV_ERR_PIVOT = 2,
    DEV_ERR_BOUNDS = 4,
};

} // namespace vgb
