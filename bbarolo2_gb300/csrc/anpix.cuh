// Pixels of the ANALYTIC samples (bbarolo/galmod.py:400-406 and :514-517) in float32 with a rounding bound, shared
// by the ring maps and the model's fast path.
//
// The pixel is computed in float32 as xpos + R caz P1 - R saz P2 + z P3 (and the same for y). Counting the
// roundings (R, caz, the coefficients, z0 and the height each rounded to float32, then 2 products per term and 3
// sums), the float32 value is within 8u (|xpos| + |t1| + |t2| + |t3|) + u (|x| + 1/2) of the exact one, u = 2^-24;
// the reference's float64 value is within 1e-12 of it. MAPS_EPS = 16u (twice that bound): when the float32 value
// lies within MAPS_EPS x (|xpos| + |t1| + |t2| + |t3| + 1) of a half-integer, the pixel is recomputed in
// float-float (pixel_ff) and, if that is too close as well, with the reference's float64 operations.
#pragma once

#include "devmath.cuh"
#include "internal.h"

#define MAPS_EPS 9.5367431640625e-07f

namespace {

__device__ __forceinline__ bool round_fast(float v, float eps, int &out) {
    if (!(fabsf(v) < 1.0e6f)) return false;
    const float f = __fadd_rn(v, 0.5f);
    float fl;
    const int i = floor_small(f, fl);
    const float d = __fsub_rn(f, fl);
    if (d < eps || d > 1.0f - eps) return false;
    out = i;
    return true;
}

__device__ __forceinline__ int clamp_pix(long long v) {
    return v < -(1LL << 30) ? -(1 << 30) : (v > (1LL << 30) ? (1 << 30) : (int)v);
}

// The pixel of a sample at height zq z0 in float-float (x = xpos + R caz P1 - R saz P2 + z P3, y likewise);
// false if either coordinate is within 1e-6 of a rounding boundary.
__device__ __noinline__ bool pixel_ff(const AnSub &S, int kr, double2 c, double zq, int &g0, int &g1) {
    const ff R = {S.Rf[kr], S.Rl[kr]};
    const ff A = ff_mul(R, ff_of(c.x)), B = ff_mul(R, ff_of(c.y));
    const ff z = ff_mul(ff_of(zq), ff{S.z0f, S.z0l});
    const ff T2 = ff_mul(B, ff{S.P2, S.P2l});
    const ff x = ff_add(ff_add(ff_add(ff{S.xposf, S.xposl}, ff_mul(A, ff{S.P1, S.P1l})), ff{-T2.hi, -T2.lo}),
                        ff_mul(z, ff{S.P3, S.P3l}));
    const ff y = ff_add(ff_add(ff_add(ff{S.yposf, S.yposl}, ff_mul(A, ff{S.Q1, S.Q1l})), ff_mul(B, ff{S.Q2, S.Q2l})),
                        ff_mul(z, ff{S.Q3, S.Q3l}));
    return ff_round(x, g0) && ff_round(y, g1);
}

// The float32 part of a sample's pixels: x = bxf + zq zP3, y = byf + zq zQ3 (zq the grid's height in units of z0,
// zP3 = z0 P3 rounded once: the same count of roundings as above), and the half-widths hw = 1/2 - MAPS_EPS x (the
// magnitude sum with the grid's largest height) within which the nearest integer is the reference's pixel.
struct PixF {
    float bxf, byf, zP3, zQ3, hwx, hwy;
    bool fast;                      // all the sample's coordinates are below 2^20 (the rounding below is exact)
};

__device__ __forceinline__ PixF pix_setup(const AnSub &S, int kr, float2 cf, const float *zqf, int nzz) {
    const float Rf = S.Rf[kr];
    const float a1 = Rf * cf.x, a2 = Rf * cf.y;
    const float t1 = a1 * S.P1, t2 = a2 * S.P2, u1 = a1 * S.Q1, u2 = a2 * S.Q2;
    PixF p;
    p.bxf = S.xposf + (t1 - t2);
    p.byf = S.yposf + (u1 + u2);
    p.zP3 = S.z0f * S.P3;
    p.zQ3 = S.z0f * S.Q3;
    const float zmax = nzz > 1 ? fmaxf(fabsf(zqf[0]), fabsf(zqf[nzz - 1])) : 0.f;   // (the grid is symmetric)
    const float tx = zmax * fabsf(p.zP3), ty = zmax * fabsf(p.zQ3);
    const float xa = fabsf(S.xposf) + fabsf(t1) + fabsf(t2) + 1.0f + tx;
    const float ya = fabsf(S.yposf) + fabsf(u1) + fabsf(u2) + 1.0f + ty;
    p.hwx = 0.5f - xa * (MAPS_EPS * 1.0001f);
    p.hwy = 0.5f - ya * (MAPS_EPS * 1.0001f);
    p.fast = xa < 1.0e6f && ya < 1.0e6f;
    return p;
}

// The reference's pixel of a height (zqf its float32 value, *zqp the float64 one, both in units of z0): the
// nearest integer of the float32 coordinate (1.5 2^23 added and subtracted) when it is within hw of it, else
// float-float, else the reference's float64 operations; cp: the sample's cos/sin in float64.
__device__ __forceinline__ void sample_pixel(const AnSub &S, const PixF &p, int kr, const double2 *cp, int nzz,
                                             float zqf, const double *zqp, double cdelt0, double cdelt1, int &g0,
                                             int &g1) {
    const float zq = nzz > 1 ? zqf : 0.f;
    const float vx = fmaf(zq, p.zP3, p.bxf), vy = fmaf(zq, p.zQ3, p.byf);
    const float sx = __fadd_rn(vx, BB_MAGIC15), sy = __fadd_rn(vy, BB_MAGIC15);
    const float dx = __fsub_rn(vx, __fsub_rn(sx, BB_MAGIC15)), dy = __fsub_rn(vy, __fsub_rn(sy, BB_MAGIC15));
    if (p.fast && fabsf(dx) <= p.hwx && fabsf(dy) <= p.hwy) {
        g0 = __float_as_int(sx) - 0x4B400000;
        g1 = __float_as_int(sy) - 0x4B400000;
        return;
    }
    const double2 c = *cp;
    const double zd = nzz > 1 ? *zqp : 0.0;
    if (!pixel_ff(S, kr, c, zd, g0, g1)) {
        // bbarolo/galmod.py:514-517 in the reference's float64 operations
        const double R = S.R[kr];
        const double x = __dmul_rn(R, c.x);
        const double yb = __dmul_rn(__dmul_rn(R, c.y), S.cinc);
        const double z = nzz > 1 ? __dmul_rn(zd, S.z0) : 0.0;
        const double y = __dsub_rn(yb, __dmul_rn(z, S.sinc));
        g0 = clamp_pix(lround_ref(
            __dadd_rn(S.xpos, __ddiv_rn(__dsub_rn(__dmul_rn(x, S.spa), __dmul_rn(y, S.cpa)), cdelt0))));
        g1 = clamp_pix(lround_ref(
            __dadd_rn(S.ypos, __ddiv_rn(__dadd_rn(__dmul_rn(x, S.cpa), __dmul_rn(y, S.spa)), cdelt1))));
    }
}

}  // namespace
