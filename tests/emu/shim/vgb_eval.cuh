// Host stand-in for csrc/vgb_eval.cuh, for compiling the generated model
// structs with a host compiler (test infrastructure, tests/emu/coop_emu.cpp):
// CUDA qualifiers become nothing, the named barrier of a cooperative group
// becomes a std::barrier shared by the host threads that play its warps.
#pragma once
#include <barrier>
#include <cmath>
#include <cstring>

#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __restrict__ __restrict

namespace vgb {
inline std::barrier<>* coop_emu_barrier = nullptr;
inline void vgb_coop_bar(int, int) { coop_emu_barrier->arrive_and_wait(); }
typedef double* vgb_xs_t;
inline double vgb_xs_ld(vgb_xs_t xs, int off) { return xs[off]; }
inline void vgb_xs_st(vgb_xs_t xs, int off, double v) { xs[off] = v; }
inline bool vgb_xs_ldb(vgb_xs_t xs, int off) { return xs[off] != 0.0; }
inline void vgb_xs_stb(vgb_xs_t xs, int off, bool b) { xs[off] = b ? 1.0 : 0.0; }
inline long long __double_as_longlong(double x) { long long r; std::memcpy(&r, &x, 8); return r; }
inline double __longlong_as_double(long long x) { double r; std::memcpy(&r, &x, 8); return r; }
// the models' NaN-propagating min / max and floored remainder (csrc/vgb_common.cuh)
inline double vgb_fmin(double a, double b) { return (a != a || b != b) ? (a + b) : (a < b ? a : b); }
inline double vgb_fmax(double a, double b) { return (a != a || b != b) ? (a + b) : (a > b ? a : b); }
inline double vgb_fmod_floor(double a, double b) {
    double r = std::fmod(a, b);
    if (r != 0.0 && ((r < 0.0) != (b < 0.0))) r += b;
    return r;
}
}  // namespace vgb
