// FP64 elementary functions for the generated device models.
//
// GB300 retires one FP64 warp-instruction per ~19 cycles per SM (64 cycles
// per SM sub-partition), whatever the number of active lanes, so the cost of
// a device evaluation at full occupancy is its count of FP64 instructions.
// Measured on the part (8 independent chains per warp), in FP64-instruction
// equivalents: the library's division, exp, log and pow take 10.2, 16.9,
// 31.8 and 90.8; the versions below take 8.7, 13.5, 17.8 and 32.0.  They
// keep full double accuracy (division within 1 ulp, exp and log within 2 ulp,
// pow within a few ulp of |y ln x|), far inside the 1e-10 relative tolerance
// of the model outputs.  Arguments outside the ranges handled here
// (overflow, underflow, subnormals, zero, infinities, NaN) go to the library
// functions, so every special case keeps IEEE semantics.
//
// Methods (each written here from the published description):
// * exp: table-driven reduction of P. T. P. Tang, "Table-driven
//   implementation of the exponential function in IEEE floating-point
//   arithmetic", ACM TOMS 15(2), 1989: x = (64 m + j) ln2/64 + r with
//   |r| <= ln2/128, exp(x) = 2^m 2^(j/64) exp(r); exp(r) - 1 by its Taylor
//   series to r^6 (truncation below 2^-60).
// * log: table-driven reduction of P. T. P. Tang, "Table-driven
//   implementation of the logarithm function in IEEE floating-point
//   arithmetic", ACM TOMS 16(4), 1990: x = 2^m (F + f) with F = 1 + j/128
//   nearest to the mantissa, ln x = m ln2 + ln F + ln(1 + f/F); ln(1 + u) by
//   its Taylor series to u^8 for |u| <= 2^-8 (truncation below 2^-66).
// * division: Newton-Raphson reciprocal y <- y + y (1 - b y) from the PTX
//   rcp.approx.ftz.f64 seed (two steps), then the quotient q = a y with one
//   residual correction q + (a - b q) y (Markstein's form).
// * pow(x, y) = exp(y ln x) for x > 0.
//
// The tables (2^(j/64), ln F, 1/F and the split constants) are generated at
// build time from 50-digit decimal arithmetic and rounded once to double
// (vajax_gb300/build.py, math_tables()).
#pragma once

#include <cuda_runtime.h>

#include "vgb_fastdiv.cuh"
#include "vgb_math_tables.cuh"

namespace vgb {

// The models' safe division (reference semantics: a / 0 = 0) on vgb_div.
__device__ __forceinline__ double vgb_msdiv(double a, double b) {
    const int eb = (__double2hiint(b) >> 20) & 0x7ff;
    const int ea = (__double2hiint(a) >> 20) & 0x7ff;
    if (eb < 1023 - 500 || eb >= 1023 + 500 || ea >= 1023 + 500) return b == 0.0 ? 0.0 : a / b;
    const double y = vgb_rcp_nr(b);
    const double q = a * y;
    const double r = fma(-b, q, a);
    return fma(r, y, q);
}

__device__ __forceinline__ double vgb_exp(double x) {
    const int hx = __double2hiint(x) & 0x7fffffff;
    if (hx >= 0x40861800) return exp(x);  // |x| >= 707, inf, NaN: overflow / subnormal results
    // k = nearest integer to x 64/ln2, read from the low word after adding 1.5 * 2^52
    const double shifter = 6755399441055744.0;
    const double t = fma(x, VGB_INV_LN2_64, shifter);
    const int k = __double2loint(t);
    const double kd = t - shifter;
    double r = fma(-kd, VGB_LN2_64_HI, x);  // kd * HI is exact (HI has 36 significant bits)
    r = fma(-kd, VGB_LN2_64_LO, r);
    double p = fma(r, 1.0 / 720.0, 1.0 / 120.0);
    p = fma(p, r, 1.0 / 24.0);
    p = fma(p, r, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r * r, r);  // exp(r) - 1
    const double T = __ldg(&VGB_EXP2_TAB[k & 63]);
    const double y = fma(T, p, T);
    const int m = k >> 6;  // floor(k / 64)
    return __hiloint2double(__double2hiint(y) + (m << 20), __double2loint(y));
}

__device__ __forceinline__ double vgb_log(double x) {
    const int hx = __double2hiint(x);
    if (hx < 0x00100000 || hx >= 0x7ff00000) return log(x);  // <= 0, subnormal, inf, NaN
    const int m = (hx >> 20) - 1023;
    const double f1 = __hiloint2double((hx & 0x000fffff) | 0x3ff00000, __double2loint(x));  // mantissa in [1, 2)
    const int j = ((hx & 0x000fffff) + (1 << 12)) >> 13;  // F = 1 + j/128 nearest to f1, j in 0..128
    const double F = __hiloint2double(0x3ff00000 + (j << 13), 0);  // 1 + j/128 (2.0 for j = 128)
    const double u = (f1 - F) * __ldg(&VGB_LOG_INVF[j]);  // f1 - F is exact
    double p = fma(u, -1.0 / 8.0, 1.0 / 7.0);
    p = fma(p, u, -1.0 / 6.0);
    p = fma(p, u, 1.0 / 5.0);
    p = fma(p, u, -1.0 / 4.0);
    p = fma(p, u, 1.0 / 3.0);
    p = fma(p, u, -0.5);
    p = fma(p, u * u, u);  // ln(1 + u)
    const double md = (double)m;
    const double hi = fma(md, VGB_LN2_HI, __ldg(&VGB_LOG_LNF_HI[j]));  // md * LN2_HI is exact
    const double lo = fma(md, VGB_LN2_LO, __ldg(&VGB_LOG_LNF_LO[j])) + p;  // exactly p for m = -1, j = 128
    return hi + lo;
}

__device__ __forceinline__ double vgb_pow(double x, double y) {
    const int hx = __double2hiint(x);
    const int ey = (__double2hiint(y) >> 20) & 0x7ff;
    if (hx < 0x00100000 || hx >= 0x7ff00000 || ey == 0x7ff) return pow(x, y);  // x <= 0, subnormal, inf, NaN
    const double z = y * vgb_log(x);
    if (!(fabs(z) < 707.0)) return pow(x, y);
    return vgb_exp(z);
}

} // namespace vgb
