// Device float64 helpers that reproduce the reference's arithmetic (each operation rounded once, no
// contraction): the rounding of bbarolo/galmod.py:_lround and the channel of a velocity (_velgrid).
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

#define C_MS 2.99792458e08

// bbarolo/galmod.py:38-46
static __device__ __forceinline__ long long lround_ref(double x) {
    if (!(fabs(x) < 1e18)) return -(1LL << 62);
    if (x >= 0) return (long long)__dadd_rn(x, 0.5);
    return -(long long)__dadd_rn(-x, 0.5);
}

// bbarolo/galmod.py:49-62
static __device__ __forceinline__ double velgrid_exact(double v, const GridDev &g, int nl) {
    double w;
    if (g.axtyp == 4) w = v;
    else {
        double f0 = g.lfreq0[nl];
        if (g.velsys == 1) w = __dmul_rn(f0, __dsub_rn(1.0, __ddiv_rn(v, C_MS)));
        else if (g.velsys == 2) w = __dmul_rn(f0, __ddiv_rn(C_MS, __dadd_rn(C_MS, v)));
        else w = __dmul_rn(f0, __dsqrt_rn(__ddiv_rn(__dsub_rn(C_MS, v), __dadd_rn(C_MS, v))));
        if (g.axtyp == 2) w = __ddiv_rn(C_MS, w);
    }
    return __dsub_rn(__dadd_rn(__ddiv_rn(__dsub_rn(w, g.crval3), g.cdelt3), g.crpix3), 1.0);
}
