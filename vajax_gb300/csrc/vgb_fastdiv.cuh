// Reciprocal and division in FP64 with fewer FP64 instructions than the IEEE
// division (about 6 and 9 FP64-instruction equivalents against 10 on GB300):
// the PTX rcp.approx.ftz.f64 seed refined by two Newton-Raphson steps
// y <- y + y (1 - b y); the quotient q = a y with one residual correction
// q + (a - b q) y (Markstein's form).  Division within 1 ulp, reciprocal
// within 1 ulp.  Arguments outside the safe exponent range (and zero,
// subnormals, infinities, NaN) take the IEEE operation.  Used by the
// generated device models and on the pivot chain of the factorisation.
#pragma once

#include <cuda_runtime.h>

namespace vgb {

__device__ __forceinline__ double vgb_rcp_nr(double b) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
    double e = fma(-b, y, 1.0);
    y = fma(y, e, y);
    e = fma(-b, y, 1.0);
    return fma(y, e, y);
}

// 1 / b, for |b| in [2^-500, 2^500) by vgb_rcp_nr, else IEEE.
__device__ __forceinline__ double vgb_rcp(double b) {
    const int eb = (__double2hiint(b) >> 20) & 0x7ff;
    if (eb < 1023 - 500 || eb >= 1023 + 500) return 1.0 / b;
    return vgb_rcp_nr(b);
}
__device__ __forceinline__ float vgb_rcp(float b) { return 1.0f / b; }

// a / b for finite a, b with |b| in [2^-500, 2^500) and |a| < 2^500 (the
// quotient stays a normal number); everything else is the IEEE division.
__device__ __forceinline__ double vgb_div(double a, double b) {
    const int eb = (__double2hiint(b) >> 20) & 0x7ff;
    const int ea = (__double2hiint(a) >> 20) & 0x7ff;
    if (eb < 1023 - 500 || eb >= 1023 + 500 || ea >= 1023 + 500) return a / b;
    const double y = vgb_rcp_nr(b);
    const double q = a * y;
    const double r = fma(-b, q, a);
    return fma(r, y, q);
}

} // namespace vgb
