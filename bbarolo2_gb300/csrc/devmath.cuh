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

// Roundings and conversions between float32 and integers with float32 additions and integer operations only
// (the conversion instructions run on a slow shared pipe on this GPU): floor of |v| < 2^22, round-to-nearest-
// even of any float32 (as rintf) to a 64-bit integer, and a 64-bit integer to the float32 nearest to each 32-bit
// half.
#define BB_MAGIC15 12582912.0f         // 1.5 * 2^23: adding it rounds |v| < 2^22 to an integer in the low bits
static __device__ __forceinline__ int floor_small(float v, float &fl) {
    float r = __fsub_rn(__fadd_rn(v, BB_MAGIC15), BB_MAGIC15);   // nearest integer, exact
    if (r > v) r = __fsub_rn(r, 1.0f);
    fl = r;
    return __float_as_int(__fadd_rn(r, BB_MAGIC15)) - 0x4B400000;
}

static __device__ __forceinline__ long long f32_to_ll(float x) {
    const float ax = fabsf(x);
    long long v;
    if (ax >= 8388608.0f) {                                      // integral: mantissa * 2^e, e >= 0
        const int b = __float_as_int(ax);
        v = (long long)((b & 0x7fffff) | 0x800000) << (((b >> 23) & 255) - 150);
    } else {                                                     // 2^23 + ax rounds ax to an integer
        v = __float_as_int(__fadd_rn(ax, 8388608.0f)) - 0x4B000000;
    }
    return x < 0.0f ? -v : v;
}

static __device__ __forceinline__ float ll_to_f32(long long v) {
    return (float)(int)(v >> 32) * 4294967296.0f + (float)(unsigned)(v & 0xffffffffLL);
}

// Float-float arithmetic (an unevaluated sum hi + lo of two float32, ~44 significant bits; error-free
// transformations with explicit FMAs, no reassociation): used to decide the rounding of a pixel when its float32
// value is too close to a boundary, before the exact float64 path.
struct ff {
    float hi, lo;
};

static __device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

static __device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

static __device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast_two_sum(s.hi, s.lo);
}

static __device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_fast_two_sum(p, e);
}

// The float-float value of a float64
static __device__ __forceinline__ ff ff_of(double v) {
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

// round-half-up of x = a + b R c - b R s' ... evaluated as floor(x + 1/2) in float-float: false when x + 1/2 is
// within 1e-6 of an integer (the float-float error is below 1e-10 for |x| < 1e6, so the float64 value of the
// reference rounds the same way whenever this returns true)
static __device__ __forceinline__ bool ff_round(ff x, int &out) {
    const ff f = ff_add(x, ff{0.5f, 0.0f});
    if (!(fabsf(f.hi) < 1.0e6f)) return false;
    float m = floorf(f.hi);
    float d = __fadd_rn(__fsub_rn(f.hi, m), f.lo);
    if (d < 0.0f) {
        m -= 1.0f;
        d += 1.0f;
    } else if (d >= 1.0f) {
        m += 1.0f;
        d -= 1.0f;
    }
    if (d < 1.0e-6f || d > 1.0f - 1.0e-6f) return false;
    out = (int)m;
    return true;
}
