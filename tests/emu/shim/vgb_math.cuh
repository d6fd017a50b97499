// Host stand-in for csrc/vgb_math.cuh (test infrastructure): the models' math
// functions as the C library's, with the models' safe-division semantics.
#pragma once
#include <cmath>

namespace vgb {
constexpr double VGB_INV_LN10 = 0.43429448190325182765;
inline double vgb_exp(double x) { return std::exp(x); }
inline double vgb_log(double x) { return std::log(x); }
inline double vgb_pow(double x, double y) { return std::pow(x, y); }
inline double vgb_msdiv(double a, double b) { return b == 0.0 ? 0.0 : a / b; }
}  // namespace vgb
