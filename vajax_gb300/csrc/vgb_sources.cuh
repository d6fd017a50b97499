// Source waveforms evaluated on the device (vajax/analysis/sources.py:31-105),
// shared by the step loop of one circuit and by the batched engine.
#pragma once

#include "vgb_circuit.h"

namespace vgb {

__device__ inline double eval_source(int kind, const double* p, int cnt, double t) {
    if (kind == SRC_DC) return p[0];
    if (kind == SRC_PULSE) {
        // val0, val1, rise, fall, width, period, delay
        const double v0 = p[0], v1 = p[1], r = p[2], f = p[3], w = p[4], per = p[5], d = p[6];
        const double tp = vgb_fmod_floor(t - d, per);
        if (t < d) return v0;
        if (tp < r) return v0 + (v1 - v0) * tp / r;
        if (tp < r + w) return v1;
        if (tp < r + w + f) return v1 - (v1 - v0) * (tp - r - w) / f;
        return v0;
    }
    if (kind == SRC_PWL) {
        // [period, t0, v0, t1, v1, ...] (times already stretched, values scaled)
        const double period = p[0];
        const int np = (cnt - 1) / 2;
        const double* tv = p + 1;
        double tt = t;
        if (period > 0) tt = vgb_fmod_floor(t, period);
        if (tt <= tv[0]) return tv[1];
        if (tt >= tv[2 * (np - 1)]) return tv[2 * (np - 1) + 1];
        int lo = 0, hi = np - 1;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (tv[2 * mid] <= tt) lo = mid; else hi = mid;
        }
        const double t0 = tv[2 * lo], t1 = tv[2 * hi], v0 = tv[2 * lo + 1], v1 = tv[2 * hi + 1];
        const double dt = t1 - t0;
        return dt == 0.0 ? v1 : v0 + (tt - t0) * (v1 - v0) / dt;
    }
    if (kind == SRC_SINE) {
        return p[0] + p[1] * sin(2.0 * 3.141592653589793 * p[2] * t + p[3]);
    }
    return 0.0;
}

} // namespace vgb
