// The Monte-Carlo GALMOD deposit on the device (the reference's _galmod_mc, bbarolo/galmod.py:92-171).
//
// The clouds of a sub-ring are drawn from one xoroshiro128+ stream; their draws do not depend on the ring
// parameters, so the host parses the stream once per (seed, layer, cloud counts) into a layout: per cloud
// its radius R, cos/sin of its azimuth and its layer deviate, per sub-cloud the first word of its normal
// deviate (the values of the rare normals that took the slow path of the ziggurat in a side list).
//
// Per evaluation the kernels place the clouds:
//   k_mc_bin      pixel of every cloud in the member's box, and the count of clouds per pixel;
//   k_scan_*      the offsets of the per-pixel lists (64 lists per tile of at most 64 pixels);
//   k_mc_scatter  the entry of every cloud (its pixel, sorted normals, channel centre and rounding bound, fixed-point
//                 flux) into its pixel's list (a counting sort);
//   deposit       one CTA per (member, tile): every sub-cloud of the tile's clouds is added, in 64-bit fixed
//                 point, to a shared-memory tile (pixels x channels), written once to HBM at the end:
//                 k_mc_deposit_px  the common case (a linear channel map, one line, at most 128 samples per
//                                  cloud, tiles of 32 or 64 pixels): pixel-owned lane groups;
//                 k_mc_deposit_lean  the same criteria on smaller tiles (more than 224 channels): a warp per
//                                  cloud;
//                 k_mc_deposit     everything else (several lines, non-linear axes, float64 output).
// Fixed-point sums are exact and independent of the order of the deposits: the model is deterministic.
//
// Indices are bit-exact with the reference: each pixel and channel is first computed in float32 with a
// bound on its rounding error; when the value lies within that bound of a rounding boundary (a half
// integer) it is recomputed with the reference's float64 operations, in its order, with no contraction
// (__dmul_rn/__dadd_rn/__ddiv_rn/__dsqrt_rn), so lround() gives the reference's integer.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "devmath.cuh"
#include "kernels.h"

#define ERR_LAYOUT 1

namespace {

// floor(v + 0.5) if it equals the reference's rounding of the exact value (|error of v| < eps)
__device__ __forceinline__ bool round_fast(float v, float eps, int &out) {
    if (!(fabsf(v) < 1.0e6f)) return false;
    float f = v + 0.5f;
    float fl = floorf(f);
    float d = f - fl;
    if (d < eps || d > 1.0f - eps) return false;
    out = (int)fl;
    return true;
}

// 2^-18: 64 float32 units of roundoff per unit of magnitude (the fast paths have fewer than 12 roundings)
#define EPS_REL 3.814697265625e-06f

// the exact pixel of a cloud (bbarolo/galmod.py:133-137)
__device__ __forceinline__ void pixel_exact(const SubMC &S, const GridDev &g, const double *cd, long long &g0,
                                            long long &g1) {
    double R = cd[0], caz = cd[1], saz = cd[2], fd = cd[3];
    double z = __dmul_rn(fd, S.z0);
    double x = __dmul_rn(R, caz);
    double y = __dsub_rn(__dmul_rn(__dmul_rn(R, saz), S.cinc), __dmul_rn(z, S.sinc));
    g0 = lround_ref(__dadd_rn(S.xpos, __ddiv_rn(__dsub_rn(__dmul_rn(x, S.spa), __dmul_rn(y, S.cpa)), g.cdelt0)));
    g1 = lround_ref(__dadd_rn(S.ypos, __ddiv_rn(__dadd_rn(__dmul_rn(x, S.cpa), __dmul_rn(y, S.spa)), g.cdelt1)));
}

// the exact line-of-sight velocity of a cloud (bbarolo/galmod.py:147-152)
__device__ __forceinline__ double vlos_exact(const SubMC &S, const double *cd) {
    double caz = cd[1], saz = cd[2];
    double z = __dmul_rn(cd[3], S.z0);
    double az_ = fabs(z);
    double vr = S.vrot;
    if (az_ > S.zcyl) {
        double v = __dsub_rn(S.vrot, __dmul_rn(S.dvdz, __dsub_rn(az_, S.zcyl)));
        vr = S.vrot >= 0.0 ? ((0.0 > v) ? 0.0 : v) : ((0.0 < v) ? 0.0 : v);
    }
    double vs = __dadd_rn(S.vsys, __dmul_rn(__dadd_rn(__dmul_rn(vr, caz), __dmul_rn(S.vrad, saz)), S.sinc));
    return __dadd_rn(vs, __dmul_rn(S.vvert, S.cinc));
}

// the pixel of a cloud: float32 with a rounding bound, float64 near a boundary; false if outside the box
__device__ __forceinline__ bool cloud_pixel(const SubMC &S, const GridDev &g, const MemberDev &M, float4 cf,
                                            const double *cd, int &ix, int &iy) {
    float z = cf.w * S.z0f;
    float a1 = cf.x * cf.y, a2 = cf.x * cf.z;
    float t1 = a1 * S.P1, t2 = a2 * S.P2, t3 = z * S.P3;
    float u1 = a1 * S.Q1, u2 = a2 * S.Q2, u3 = z * S.Q3;
    float gx = S.xposf + (t1 - t2) + t3;
    float gy = S.yposf + (u1 + u2) + u3;
    float ex = (fabsf(S.xposf) + fabsf(t1) + fabsf(t2) + fabsf(t3) + 1.0f) * EPS_REL;
    float ey = (fabsf(S.yposf) + fabsf(u1) + fabsf(u2) + fabsf(u3) + 1.0f) * EPS_REL;
    int a, b;
    if (round_fast(gx, ex, a) && round_fast(gy, ey, b)) {
        ix = a;
        iy = b;
    } else {
        long long g0, g1;
        pixel_exact(S, g, cd, g0, g1);
        if (g0 < M.blo0 || g0 >= M.bhi0 || g1 < M.blo1 || g1 >= M.bhi1) return false;
        ix = (int)g0;
        iy = (int)g1;
    }
    return ix >= M.blo0 && ix < M.bhi0 && iy >= M.blo1 && iy < M.bhi1;
}

// the list of pixel lp of a tile (see NOWN): the lists of warp w's pixels (lp = w mod 8) are contiguous
__device__ __forceinline__ int list_slot(int lp) { return (lp & 7) * 8 + (lp >> 3); }

// this warp's clouds in a tile: the concatenated lists of its pixels (begin, count)
__device__ __forceinline__ void warp_lists(const int *__restrict__ offset, const int *__restrict__ count, int lbase,
                                           int warp, int &beg, int &n) {
    beg = offset[lbase + 8 * warp];
    n = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) n += count[lbase + 8 * warp + j];
}

// The (member, cloud) of thread idx of the bin and scatter kernels: segment i (threads cstart[i] ..
// cstart[i + 1]) is cseg[i] = (member whose tiles take the clouds, member whose constants place them, first
// cloud, sign of the deposits): a member's own clouds, or, for a member that differs from member 0 in a few
// sub-rings, the clouds of those sub-rings with its constants (+) and with member 0's (-).
struct CloudSeg {
    int k, src, c, sign;
};
__device__ __forceinline__ CloudSeg cloud_of(const long long *__restrict__ cstart, const int4 *__restrict__ cseg,
                                             int nseg, long long idx) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cstart[mid] <= idx) lo = mid;
        else hi = mid - 1;
    }
    const int4 sg = cseg[lo];
    return CloudSeg{sg.x, sg.y, sg.z + (int)(idx - cstart[lo]), sg.w};
}

__global__ void k_mc_bin(GridDev g, LayoutDev L, const SubMC *__restrict__ sub, int nsub,
                         const MemberDev *__restrict__ mem, const long long *__restrict__ cstart,
                         const int4 *__restrict__ cseg, int nseg, long long ntot, int tx, int ty,
                         int *__restrict__ pix, int *__restrict__ tile_count, int *err) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ntot) return;
    const CloudSeg cl = cloud_of(cstart, cseg, nseg, idx);
    const int k = cl.k, c = cl.c;
    int ir = L.sub[c];
    const SubMC &S = sub[(size_t)cl.src * nsub + ir];
    const MemberDev &M = mem[k];
    if (!S.active || c - L.cloud_base[ir] >= S.nc) {
        atomicOr(err, ERR_LAYOUT);
        pix[idx] = -1;
        return;
    }
    float4 cf = L.cf[c];
    double wside = cf.y >= 0.0f ? S.wrec : S.wapp;   // (the sign of the float32 cosine is the sign of caz)
    int ix, iy;
    if (wside == 0.0 || !cloud_pixel(S, g, M, cf, L.cd + 4 * (size_t)c, ix, iy)) {
        pix[idx] = -1;
        return;
    }
    int px = ix - M.blo0, py = iy - M.blo1;
    pix[idx] = py * M.bx + px;
    const int lp = (py % ty) * tx + (px % tx);
    atomicAdd(&tile_count[(M.tile_off + (py / ty) * M.ntx + px / tx) * NOWN + list_slot(lp)], 1);
}

// The deposit entry of a (member, cloud) in its tile's list: computed here, one thread per entry.
struct __align__(16) Entry {
    int c;          // cloud
    int pb;         // first of the cloud's sorted normals (padded layout)
    int meta;       // nv | pixel in the tile << 16 | half << 24 | (placed with member 0's constants) << 25
    float tc;       // channel of the cloud's velocity (line 0, float32 with the bound epsc)
    long long fix;  // fixed-point flux of one sample (line 0)
    float eps;      // rounding bound of the float32 channel of every sample of the cloud (line 0)
    float sg;       // channels per unit normal deviate
};

// channel centre of a cloud and its rounding bound (float32), for line nl (see the fast path of k_mc_deposit)
__device__ __forceinline__ void cloud_centre(const SubMC &S, float4 cf, int nl, float &tc, float &epsc) {
    const float zf = cf.w * S.z0f;
    const float azf = fabsf(zf);
    float vr = S.vrotf;
    if (azf > S.zcylf) {
        float v = S.vrotf - S.dvdzf * (azf - S.zcylf);
        vr = S.vrotf >= 0.0f ? fmaxf(v, 0.0f) : fminf(v, 0.0f);
    }
    const float base = vr * cf.y + S.vradf * cf.z;
    const float mbase = fabsf(vr * cf.y) + fabsf(S.vradf * cf.z) + fabsf(S.dvdzf) * (azf + fabsf(S.zcylf));
    tc = S.c0[nl] + base * S.sia[nl];
    epsc = (fabsf(S.c0[nl]) + mbase * fabsf(S.sia[nl]) + 1.0f) * EPS_REL;
}

__global__ void k_mc_scatter(LayoutDev L, const SubMC *__restrict__ sub, int nsub, const MemberDev *__restrict__ mem,
                             const long long *__restrict__ cstart, const int4 *__restrict__ cseg, int nseg,
                             long long ntot, int tx, int ty, const int *__restrict__ pix, int *__restrict__ cursor,
                             Entry *__restrict__ bucket, int defer_fix) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ntot) return;
    int p = pix[idx];
    if (p < 0) return;
    const CloudSeg cl = cloud_of(cstart, cseg, nseg, idx);
    const int k = cl.k, c = cl.c;
    const MemberDev &M = mem[k];
    int py = p / M.bx, px = p - py * M.bx;
    const int lp = (py % ty) * tx + (px % tx);
    int slot = atomicAdd(&cursor[(M.tile_off + (py / ty) * M.ntx + px / tx) * NOWN + list_slot(lp)], 1);
    const float4 cf = L.cf[c];
    const int half = cf.y >= 0.0f ? 0 : 1;
    const int ir = L.sub[c];
    const int nv = L.nvs[ir];
    const SubMC &S = sub[(size_t)cl.src * nsub + ir];
    Entry e;
    e.c = c;
    e.pb = (int)(L.pbase[ir] + (long long)(c - L.cloud_base[ir]) * ((nv + 3) & ~3));
    e.meta = (nv & 0xffff) | (lp << 16) | (half << 24) | (cl.src != k ? 1 << 25 : 0);
    float epsc;
    cloud_centre(S, cf, 0, e.tc, epsc);
    // defer_fix: the fixed-point flux is not known yet (the flux normalisation computes it while the clouds are
    // binned): the entry holds its sub-ring constants' index and sign, for k_entry_fix
    if (defer_fix) e.fix = (long long)((size_t)cl.src * nsub + ir) * 2 + (cl.sign < 0 ? 1 : 0);
    else e.fix = cl.sign < 0 ? -S.fix[half][0] : S.fix[half][0];
    e.sg = S.sg[0];
    // the cloud's largest |normal| is at an end of its sorted run
    const float nmax = fmaxf(fabsf(__ldg(&L.nf[e.pb])), fabsf(__ldg(&L.nf[e.pb + nv - 1])));
    e.eps = fmaf(nmax, fabsf(e.sg) * EPS_REL, epsc);
    bucket[slot] = e;
}

// The fixed-point flux of the entries that k_mc_scatter left as (sub-ring constants' index, sign): one thread
// per entry of the lists (their number: the last list's offset plus its count).
__global__ void k_entry_fix(const SubMC *__restrict__ sub, const int *__restrict__ offset,
                            const int *__restrict__ count, int nlist, Entry *__restrict__ bucket) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)offset[nlist - 1] + count[nlist - 1];
    if (i >= total) return;
    Entry &e = bucket[i];
    const long long v = e.fix;
    const long long f = sub[(size_t)(v >> 1)].fix[(e.meta >> 24) & 1][0];
    e.fix = (v & 1) ? -f : f;
}

// the exact channel of a sub-cloud (bbarolo/galmod.py:153-170), not clipped to the cube
__device__ __noinline__ long long channel_exact_raw(const SubMC &S, const GridDev &g, const double *cd, double nx,
                                                    int nl) {
    const double vs = vlos_exact(S, cd);
    if (g.axtyp == 4 && g.nlines == 1) {
        double gz = __dadd_rn(__dmul_rn(vs, g.ia), g.ib);
        double sg = __dmul_rn(S.vdisptmp, g.ia);
        return lround_ref(__dadd_rn(gz, __dmul_rn(nx, sg)));
    }
    double v = __dadd_rn(vs, __dmul_rn(nx, S.vdisptmp));
    return lround_ref(velgrid_exact(v, g, nl));
}

// the exact channel in the cube, or -1 outside it
__device__ __forceinline__ int channel_exact(const SubMC &S, const GridDev &g, const double *cd, double nx, int nl) {
    const long long is = channel_exact_raw(S, g, cd, nx, nl);
    return (is < 0 || is >= g.nz) ? -1 : (int)is;
}

#define XQ 64         // capacity of a warp's queue of sub-clouds deferred to the exact path

// The exact normal deviate of sub-cloud iv of a cloud: from its first word, or from the list of slow ones
// (its ordinal among the cloud's slow normals counted from the words before it: a rare path).
__device__ __noinline__ double normal_exact(const LayoutDev &L, const ZigDev *zig, long long sb, int iv, int slow_base,
                                            int *err) {
    const int h = L.hz[sb + iv];
    const int iz = h & 127;
    const unsigned ah = h < 0 ? 0u - (unsigned)h : (unsigned)h;
    if (ah < zig->kn[iz]) return __dmul_rn((double)h, zig->wn[iz]);
    int o = slow_base;
    for (int j = 0; j < iv; j++) {
        const int hj = L.hz[sb + j];
        const unsigned aj = hj < 0 ? 0u - (unsigned)hj : (unsigned)hj;
        o += !(aj < zig->kn[hj & 127]);
    }
    if (o >= L.nslow) {
        atomicOr(err, ERR_LAYOUT);
        return 0.0;
    }
    return L.slow_val[o];
}

// Adds v to row[ch] for the lanes with a pending deposit, one lane at a time: the warp owns its pixels, so the
// plain read-modify-write is race-free once same-channel lanes are serialised (a rare path).
__device__ __forceinline__ void warp_serial_add(unsigned long long *row, bool pending, int ch, long long v, int lane) {
    unsigned mask = __ballot_sync(0xffffffffu, pending);
    while (mask) {
        const int src = __ffs(mask) - 1;
        const int c = __shfl_sync(0xffffffffu, ch, src);
        const long long w = __shfl_sync(0xffffffffu, v, src);
        if (lane == 0) row[c] += (unsigned long long)w;
        __syncwarp();
        mask &= mask - 1;
    }
}

__device__ __forceinline__ long long stream_base(const LayoutDev &L, int c, int ir, int nv) {
    return L.sub_base[ir] + (long long)(c - L.cloud_base[ir]) * nv;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

#define WB 256        // sorted normals of a cloud staged per warp (clouds with more samples: per-sample path)
#define DEPTH 3       // clouds in flight per warp (cp.async pipeline)
#define EMAX 8        // sorted samples per lane (WB / 32)

// The channels of one cloud's samples counted one by one (float32 with the exact fallback) into the warp's bins
// [ws, ws + 32 m) and added to the pixel's row; samples beyond the bins are added individually. Used when the
// binary search does not apply: non-linear spectral axes, more than WB samples, a centre out of range.
__device__ __noinline__ void deposit_per_sample(const GridDev &g, const LayoutDev &L, const ZigDev *zig,
                                                const SubMC &S, int c, long long pb, long long sb, int nv, float tc,
                                                float sg, float epsc, float epsn, long long fix, int nl, bool fast,
                                                unsigned long long *row, int *myh, int *myq, int lane, int *err) {
    const unsigned ltmask = (1u << lane) - 1u;
    const int nz = g.nz;
    const float span = 10.0f * fabsf(sg) + 2.0f;
    const int m = span <= 32.0f ? 1 : (span <= 64.0f ? 2 : 4);
    const int ws = fabsf(tc) < 1.0e6f ? (int)floorf(tc + 0.5f) - 16 * m : 0;
    int nq = 0;
    for (int j0 = 0; j0 < nv; j0 += 32) {
        const int i = j0 + lane;
        const bool act = i < nv;
        const float nf = act ? __ldg(&L.nf[pb + i]) : 0.0f;
        const float tt = fmaf(nf, sg, tc);
        const float eps = fmaf(fabsf(nf), epsn, epsc);
        const float f = tt + 0.5f;
        const float fl = floorf(f);
        const float dd = f - fl;
        const bool ok = fast && fabsf(tt) < 1.0e6f && dd >= eps && dd <= 1.0f - eps;
        const bool ex = act && !ok;
        if (__any_sync(0xffffffffu, ex)) {
            const unsigned eb = __ballot_sync(0xffffffffu, ex);
            if (ex) myq[nq + __popc(eb & ltmask)] = i;
            nq += __popc(eb);
        }
        const int isub = (int)fl;
        const bool dep = act && ok && isub >= 0 && isub < nz;
        const int d = isub - ws;
        const bool inw = dep && d >= 0 && d < 32 * m;
        if (inw) atomicAdd(&myh[d], 1);
        if (__any_sync(0xffffffffu, dep && !inw)) warp_serial_add(row, dep && !inw, isub, fix, lane);
        if (nq > XQ - 32 || (j0 + 32 >= nv && nq > 0)) {             // (warp-uniform)
            __syncwarp();
            for (int q0 = 0; q0 < nq; q0 += 32) {
                const int q = q0 + lane;
                int is = -1;
                if (q < nq) {
                    const double nx = normal_exact(L, zig, sb, L.ord[pb + myq[q]], __ldg(&L.slow_base[c]), err);
                    is = channel_exact(S, g, L.cd + 4 * (size_t)c, nx, nl);
                }
                warp_serial_add(row, is >= 0, is, fix, lane);
            }
            __syncwarp();
            nq = 0;
        }
    }
    __syncwarp();
    for (int q = 0; q < m; q++) {
        const int bb = lane + 32 * q;
        const int cnt = myh[bb];
        if (cnt) {
            row[ws + bb] += (unsigned long long)(fix * (long long)cnt);
            myh[bb] = 0;
        }
    }
    __syncwarp();
}

// The run-length deposit of one cloud whose E samples per lane are staged (sorted) in w: lane l takes samples
// l E .. l E + E - 1, computes their channels (float32 within one rounding bound for the cloud; the exact
// float64 channel near a half-integer), and every run of equal channels is added once to the pixel row:
// count = index of the next run's first sample - index of its first sample (channels are non-decreasing).
template <int E>
__device__ __forceinline__ void deposit_runs(const GridDev &g, const LayoutDev &L, const ZigDev *zig,
                                             const SubMC *__restrict__ subk, const float *w, int c, long long pb,
                                             int nv, float tc, float sg, float eps, long long fix,
                                             unsigned long long *row, int lane, int *err) {
    const int nz = g.nz;
    const int i0 = lane * E;
    int ch[E];
    unsigned need = 0;
#pragma unroll
    for (int j = 0; j < E; j++) {
        ch[j] = 0x7fffffff;                                   // (past the last sample: the terminator)
        const bool in = i0 + j < nv;
        const float f = fmaf(in ? w[i0 + j] : 0.0f, sg, tc) + 0.5f;
        const float fl = floorf(f);
        const float dd = f - fl;
        if (in) {
            if (dd >= eps && dd <= 1.0f - eps) ch[j] = (int)fl;
            else need |= 1u << j;
        }
    }
    if (__any_sync(0xffffffffu, need != 0)) {                 // rare: exact channels
        const int ir = __ldg(&L.sub[c]);
        const SubMC &S = subk[ir];
        const long long sb = stream_base(L, c, ir, nv);
        const int sbase = __ldg(&L.slow_base[c]);
#pragma unroll
        for (int j = 0; j < E; j++)
            if (need & (1u << j)) {
                const double nx = normal_exact(L, zig, sb, L.ord[pb + i0 + j], sbase, err);
                const long long is = channel_exact_raw(S, g, L.cd + 4 * (size_t)c, nx, 0);
                ch[j] = is < -0x3fffffffLL ? -0x3fffffff : (is > 0x3fffffffLL ? 0x3fffffff : (int)is);
            }
    }
    // run starts: a sample whose channel differs from the previous sample's (lane 0's first always starts)
    const int prev0 = __shfl_up_sync(0xffffffffu, ch[E - 1], 1);
    unsigned starts = 0;
#pragma unroll
    for (int j = 0; j < E; j++) {
        const int pv = j == 0 ? (lane == 0 ? (int)0x80000000 : prev0) : ch[j - 1];
        if (ch[j] != pv && i0 + j < nv) starts |= 1u << j;
    }
    // the first start after this lane's samples (or the end)
    const unsigned B = __ballot_sync(0xffffffffu, starts != 0);
    const unsigned after = lane < 31 ? (B & (0xffffffffu << (lane + 1))) : 0u;
    const int l2 = after ? __ffs(after) - 1 : lane;
    const unsigned s2 = __shfl_sync(0xffffffffu, starts, l2);
    const int nextl = after ? l2 * E + __ffs(s2) - 1 : nv;
    while (starts) {
        const int j = __ffs(starts) - 1;
        starts &= starts - 1;
        const int nxt = starts ? i0 + __ffs(starts) - 1 : nextl;
        int chj = ch[0];
#pragma unroll
        for (int q = 1; q < E; q++)
            if (q == j) chj = ch[q];
        const int cnt = nxt - (i0 + j);
        if (chj >= 0 && chj < nz) row[chj] += (unsigned long long)(fix * (long long)cnt);
    }
}

__global__ void __launch_bounds__(256) k_mc_deposit(GridDev g, LayoutDev L, const SubMC *__restrict__ sub, int nsub,
                                                    const MemberDev *__restrict__ mem, int tx, int ty,
                                                    const int *__restrict__ offset, const int *__restrict__ count,
                                                    const Entry *__restrict__ bucket, const ZigDev *__restrict__ zig,
                                                    const float *__restrict__ cd2if, const double *__restrict__ cd2i,
                                                    float *__restrict__ model, long long mstride,
                                                    double *__restrict__ model64, int *err) {
    extern __shared__ unsigned long long tile[];   // TP x nz sums, then the warps' staging slots, then nz scales
    __shared__ int bins[8][128 + XQ];
    __shared__ Entry ents[8][DEPTH];
    const int k = blockIdx.x;
    const MemberDev &M = mem[k];
    const int t = blockIdx.y;
    if (t >= M.ntx * M.nty) return;
    const int nz = g.nz;
    const int TP = tx * ty;
    const int tyi = t / M.ntx, txi = t - tyi * M.ntx;
    const int x0 = txi * tx, y0 = tyi * ty;
    float *mout = model + (size_t)k * mstride;
    // a tile without clouds (outside the disk): zeros, without the shared-memory tile
    {
        int any = 0;
        if (threadIdx.x < NOWN) any = count[(M.tile_off + t) * NOWN + threadIdx.x] != 0;
        if (!__syncthreads_or(any)) {
            const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
            for (int lp = wid; lp < TP; lp += 8) {
                const int py = y0 + lp / tx, px = x0 + lp % tx;
                if (py >= M.by || px >= M.bx) continue;
                float *o = mout + ((size_t)py * M.bx + px) * nz;
                for (int z = ln; z < nz; z += 32) o[z] = 0.0f;
                if (model64) {
                    double *o64 = model64 + (size_t)k * mstride + ((size_t)py * M.bx + px) * nz;
                    for (int z = ln; z < nz; z += 32) o64[z] = 0.0;
                }
            }
            return;
        }
    }
    // (the staging slots start at a 16-byte boundary: cp.async copies 16-byte chunks)
    float *stg = (float *)(((uintptr_t)(tile + (size_t)TP * nz) + 15) & ~(uintptr_t)15);
    float *chs = stg + 8 * DEPTH * WB;
    {
        ulonglong2 *t2 = (ulonglong2 *)tile;
        for (int i = threadIdx.x; i < TP * nz / 2; i += blockDim.x) t2[i] = make_ulonglong2(0ULL, 0ULL);
        if (((TP * nz) & 1) && threadIdx.x == 0) tile[TP * nz - 1] = 0ULL;
        for (int i = threadIdx.x; i < 8 * (128 + XQ); i += blockDim.x) (&bins[0][0])[i] = 0;
        for (int z = threadIdx.x; z < nz; z += blockDim.x) chs[z] = ldexpf(cd2if[z], -M.fix_exp);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int beg, n;                                                  // this warp's list: the clouds of its pixels
    warp_lists(offset, count, (M.tile_off + t) * NOWN, warp, beg, n);
    const bool fast_ok = g.fast_ok;
    const SubMC *__restrict__ subk = sub + (size_t)k * nsub;
    float *slots = stg + warp * DEPTH * WB;
    int *myh = bins[warp];
    int *myq = myh + 128;
    // the (pb, meta) of the list's entries, 32 per register chunk: chunk of the current entry and the next one
    int pa = lane < n ? __ldg(&bucket[beg + lane].pb) : 0, ma = lane < n ? __ldg(&bucket[beg + lane].meta) : 0;
    int pn = 32 + lane < n ? __ldg(&bucket[beg + 32 + lane].pb) : 0;
    int mn = 32 + lane < n ? __ldg(&bucket[beg + 32 + lane].meta) : 0;
    // prefetch of entry j and its normals into slot j % DEPTH (one commit group per entry); i: the entry in use
    auto issue = [&](int j, int i) {
        if (j < n) {
            const bool same = (j >> 5) == (i >> 5);
            const int pbj = __shfl_sync(0xffffffffu, same ? pa : pn, j & 31);
            const int mj = __shfl_sync(0xffffffffu, same ? ma : mn, j & 31);
            const Entry *src = bucket + beg + j;
            Entry *dst = &ents[warp][j % DEPTH];
            if (lane < 2) cp_async16((char *)dst + 16 * lane, (const char *)src + 16 * lane);
            const int nv = mj & 0xffff;
            if (nv <= WB) {
                const float *nsrc = L.nf + (unsigned)pbj;
                float *ndst = slots + (j % DEPTH) * WB;
                for (int q = lane; q < (nv + 3) >> 2; q += 32) cp_async16(ndst + 4 * q, nsrc + 4 * q);
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int d = 0; d < DEPTH - 1; d++) issue(d, 0);
    for (int i = 0; i < n; i++) {
        issue(i + DEPTH - 1, i);
        cp_async_wait<DEPTH - 1>();
        __syncwarp();
        const Entry en = ents[warp][i % DEPTH];
        const float *w = slots + (i % DEPTH) * WB;
        const int c = en.c;
        const int nv = en.meta & 0xffff, lp = (en.meta >> 16) & 255, half = (en.meta >> 24) & 1;
        unsigned long long *row = tile + (size_t)lp * nz;
        const float tc = en.tc, sg = en.sg;
        const long long fix = en.fix;
        const float span = 10.0f * fabsf(sg) + 2.0f;
        const int m = span <= 32.0f ? 1 : (span <= 64.0f ? 2 : 4);
        const bool fast = fast_ok && nv <= WB && fabsf(tc) < 1.0e5f;
        const int ws = fast ? (int)floorf(tc + 0.5f) - 16 * m : 0;
        if (fast) {
            const float eps = en.eps;
            const int E = (nv + 31) >> 5;
            if (E <= 1) deposit_runs<1>(g, L, zig, subk, w, c, (unsigned)en.pb, nv, tc, sg, eps, fix, row, lane, err);
            else if (E <= 2) deposit_runs<2>(g, L, zig, subk, w, c, (unsigned)en.pb, nv, tc, sg, eps, fix, row, lane, err);
            else if (E <= 4) deposit_runs<4>(g, L, zig, subk, w, c, (unsigned)en.pb, nv, tc, sg, eps, fix, row, lane, err);
            else deposit_runs<8>(g, L, zig, subk, w, c, (unsigned)en.pb, nv, tc, sg, eps, fix, row, lane, err);
        }
        if (!fast || g.nlines > 1) {
            // the general path: every line with the per-sample kernel (lines after the first, non-linear axes,
            // many samples, a centre out of range)
            const int ir = __ldg(&L.sub[c]);
            const SubMC &S = sub[(size_t)k * nsub + ir];
            const float4 cf = __ldg(&L.cf[c]);
            for (int nl = fast ? 1 : 0; nl < g.nlines; nl++) {
                float tcl, epscl;
                cloud_centre(S, cf, nl, tcl, epscl);
                deposit_per_sample(g, L, zig, S, c, (unsigned)en.pb, stream_base(L, c, ir, nv), nv, tcl, S.sg[nl],
                                   epscl, fabsf(S.sg[nl]) * EPS_REL, S.fix[half][nl], nl, fast_ok, row, myh, myq, lane,
                                   err);
            }
        }
        __syncwarp();
        if (((i + 1) & 31) == 0) {                            // next chunk of entries
            pa = pn;
            ma = mn;
            const int j = i + 1 + 32 + lane;
            pn = j < n ? __ldg(&bucket[beg + j].pb) : 0;
            mn = j < n ? __ldg(&bucket[beg + j].meta) : 0;
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    // write-out: a warp per pixel, lanes along the channels (the sums times cd2i 2^-e, as float32)
    for (int lp = warp; lp < TP; lp += 8) {
        const int py = y0 + lp / tx, px = x0 + lp % tx;
        if (py >= M.by || px >= M.bx) continue;
        const unsigned long long *src = tile + (size_t)lp * nz;
        float *o = mout + ((size_t)py * M.bx + px) * nz;
        for (int z = lane; z < nz; z += 32) {
            // (int64 -> float32 through two exact 32-bit halves: one rounding in the final add)
            const long long v = (long long)src[z];
            const float hi = (float)(int)(v >> 32) * 4294967296.0f;
            const float lo = (float)(unsigned)(v & 0xffffffffLL);
            o[z] = (hi + lo) * chs[z];
        }
        if (model64) {
            double *o64 = model64 + (size_t)k * mstride + ((size_t)py * M.bx + px) * nz;
            for (int z = lane; z < nz; z += 32) o64[z] = ldexp((double)(long long)src[z] * cd2i[z], -M.fix_exp);
        }
    }
}

// The common case in a lean kernel: a linear channel map, one line, at most 128 samples per cloud (4 per
// lane). Same entries, lists, staging and run-length deposit as k_mc_deposit; the rare clouds outside the
// fast criteria go through the per-sample path.
#ifndef LEAN_MINB
#define LEAN_MINB 3       // resident CTAs per SM of the lean deposit (registers: 65536 / (256 x LEAN_MINB))
#endif
__global__ void __launch_bounds__(256, LEAN_MINB) k_mc_deposit_lean(GridDev g, LayoutDev L, const SubMC *__restrict__ sub,
                                                           int nsub, const MemberDev *__restrict__ mem, int tx, int ty,
                                                           const int *__restrict__ offset,
                                                           const int *__restrict__ count,
                                                           const Entry *__restrict__ bucket,
                                                           const ZigDev *__restrict__ zig,
                                                           const float *__restrict__ cd2if, float *__restrict__ model,
                                                           long long mstride, int *err) {
    extern __shared__ unsigned long long tile[];
    __shared__ int bins[8][128 + XQ];
    __shared__ Entry ents[8][DEPTH];
    constexpr int E = 4;
    const int k = blockIdx.x;
    const int t = blockIdx.y;
    const int ntx = mem[k].ntx;
    if (t >= ntx * mem[k].nty) return;
    const int nz = g.nz;
    const int TP = tx * ty;
    const int tyi = t / ntx, txi = t - tyi * ntx;
    const int x0 = txi * tx, y0 = tyi * ty;
    const int bx = mem[k].bx, by = mem[k].by;
    const int lbase = (mem[k].tile_off + t) * NOWN;
    float *mout = model + (size_t)k * mstride;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    {
        int any = 0;
        if (threadIdx.x < NOWN) any = count[lbase + threadIdx.x] != 0;
        if (!__syncthreads_or(any)) {
            for (int lp = warp; lp < TP; lp += 8) {
                const int py = y0 + lp / tx, px = x0 + lp % tx;
                if (py >= by || px >= bx) continue;
                float *o = mout + ((size_t)py * bx + px) * nz;
                for (int z = lane; z < nz; z += 32) o[z] = 0.0f;
            }
            return;
        }
    }
    float *stg = (float *)(((uintptr_t)(tile + (size_t)TP * nz) + 15) & ~(uintptr_t)15);
    float *chs = stg + 8 * DEPTH * WB;
    {
        ulonglong2 *t2 = (ulonglong2 *)tile;
        for (int i = threadIdx.x; i < TP * nz / 2; i += blockDim.x) t2[i] = make_ulonglong2(0ULL, 0ULL);
        if (((TP * nz) & 1) && threadIdx.x == 0) tile[TP * nz - 1] = 0ULL;
        for (int i = threadIdx.x; i < 8 * (128 + XQ); i += blockDim.x) (&bins[0][0])[i] = 0;
        const int fe = mem[k].fix_exp;
        for (int z = threadIdx.x; z < nz; z += blockDim.x) chs[z] = ldexpf(cd2if[z], -fe);
    }
    __syncthreads();
    int beg, n;
    warp_lists(offset, count, lbase, warp, beg, n);
    float *slots = stg + warp * DEPTH * WB;
    int pa = lane < n ? __ldg(&bucket[beg + lane].pb) : 0, ma = lane < n ? __ldg(&bucket[beg + lane].meta) : 0;
    int pn = 32 + lane < n ? __ldg(&bucket[beg + 32 + lane].pb) : 0;
    int mn = 32 + lane < n ? __ldg(&bucket[beg + 32 + lane].meta) : 0;
    auto issue = [&](int j, int i) {
        if (j < n) {
            const bool same = (j >> 5) == (i >> 5);
            const int pbj = __shfl_sync(0xffffffffu, same ? pa : pn, j & 31);
            const int mj = __shfl_sync(0xffffffffu, same ? ma : mn, j & 31);
            if (lane < 2)
                cp_async16((char *)&ents[warp][j % DEPTH] + 16 * lane, (const char *)(bucket + beg + j) + 16 * lane);
            if (lane < ((mj & 0xffff) + 3) >> 2)
                cp_async16(slots + (j % DEPTH) * WB + 4 * lane, L.nf + (unsigned)pbj + 4 * lane);
        }
        cp_async_commit();
    };
    issue(0, 0);
    issue(1, 0);
    for (int i = 0; i < n; i++) {
        issue(i + 2, i);
        cp_async_wait<DEPTH - 1>();
        __syncwarp();
        const Entry en = ents[warp][i % DEPTH];
        const float *w = slots + (i % DEPTH) * WB;
        const int nv = en.meta & 0xffff;
        unsigned long long *row = tile + (size_t)((en.meta >> 16) & 255) * nz;
        const float tc = en.tc, sg = en.sg;
        const long long fix = en.fix;
        if (nv <= 32 * E && fabsf(tc) < 1.0e5f) {
            const float4 nn = *(const float4 *)(w + 4 * lane);     // (zeros past nv: masked below)
            const float hw = 0.5f - en.eps;
            const int i0 = lane * E;
            const float nv4[4] = {nn.x, nn.y, nn.z, nn.w};
            int ch[E];
            unsigned need = 0;
#pragma unroll
            for (int j = 0; j < E; j++) {
                const float f = fmaf(nv4[j], sg, tc) + 0.5f;
                const float fl = floorf(f);
                const bool okj = fabsf(f - fl - 0.5f) <= hw;
                ch[j] = i0 + j < nv ? (int)fl : 0x7fffffff;
                if (i0 + j < nv && !okj) need |= 1u << j;
            }
            if (need) {                                         // rare: exact channels
                const int ir = __ldg(&L.sub[en.c]);
                const SubMC &S = sub[(size_t)k * nsub + ir];
                const long long sb = stream_base(L, en.c, ir, nv);
                const int sbase = __ldg(&L.slow_base[en.c]);
#pragma unroll
                for (int j = 0; j < E; j++)
                    if (need & (1u << j)) {
                        const double nx = normal_exact(L, zig, sb, L.ord[(unsigned)en.pb + i0 + j], sbase, err);
                        const long long is = channel_exact_raw(S, g, L.cd + 4 * (size_t)en.c, nx, 0);
                        ch[j] = is < -0x3fffffffLL ? -0x3fffffff : (is > 0x3fffffffLL ? 0x3fffffff : (int)is);
                    }
            }
            const int prev0 = __shfl_up_sync(0xffffffffu, ch[E - 1], 1);
            unsigned starts = 0;
#pragma unroll
            for (int j = 0; j < E; j++) {
                const int pv = j == 0 ? (lane == 0 ? (int)0x80000000 : prev0) : ch[j - 1];
                if (ch[j] != pv && i0 + j < nv) starts |= 1u << j;
            }
            const unsigned B = __ballot_sync(0xffffffffu, starts != 0);
            const unsigned after = lane < 31 ? (B & (0xffffffffu << (lane + 1))) : 0u;
            const int l2 = after ? __ffs(after) - 1 : lane;
            const unsigned s2 = __shfl_sync(0xffffffffu, starts, l2);
            const int nextl = after ? l2 * E + __ffs(s2) - 1 : nv;
            while (starts) {
                const int j = __ffs(starts) - 1;
                starts &= starts - 1;
                const int nxt = starts ? i0 + __ffs(starts) - 1 : nextl;
                const int chj = j == 0 ? ch[0] : (j == 1 ? ch[1] : (j == 2 ? ch[2] : ch[3]));
                if (chj >= 0 && chj < nz) row[chj] += (unsigned long long)(fix * (long long)(nxt - i0 - j));
            }
        } else {
            const int ir = __ldg(&L.sub[en.c]);
            const SubMC &S = sub[(size_t)k * nsub + ir];
            deposit_per_sample(g, L, zig, S, en.c, (unsigned)en.pb, stream_base(L, en.c, ir, nv), nv, tc, sg, en.eps,
                               fabsf(sg) * EPS_REL, fix, 0, true, row, bins[warp], bins[warp] + 128, lane, err);
        }
        __syncwarp();
        if (((i + 1) & 31) == 0) {
            pa = pn;
            ma = mn;
            const int j = i + 1 + 32 + lane;
            pn = j < n ? __ldg(&bucket[beg + j].pb) : 0;
            mn = j < n ? __ldg(&bucket[beg + j].meta) : 0;
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    for (int lp = warp; lp < TP; lp += 8) {
        const int py = y0 + lp / tx, px = x0 + lp % tx;
        if (py >= by || px >= bx) continue;
        const unsigned long long *src = tile + (size_t)lp * nz;
        float *o = mout + ((size_t)py * bx + px) * nz;
        for (int z = lane; z < nz; z += 32) {
            const long long v = (long long)src[z];
            const float hi = (float)(int)(v >> 32) * 4294967296.0f;
            const float lo = (float)(unsigned)(v & 0xffffffffLL);
            o[z] = (hi + lo) * chs[z];
        }
    }
}

// A cloud of the pixel-owned deposit (nv = 0: none).
struct PxCloud {
    int c, pb, nv, src0;        // src0: placed with member 0's constants (a difference from member 0's model)
    float tc, sg, eps;
    long long fix;
};

__device__ __forceinline__ void px_entry(const Entry *__restrict__ bucket, int beg, int n, int j, PxCloud &p) {
    if (j < n) {
        const Entry en = bucket[beg + j];
        p.c = en.c;
        p.pb = en.pb;
        p.nv = en.meta & 0xffff;
        p.src0 = (en.meta >> 25) & 1;
        p.tc = en.tc;
        p.sg = en.sg;
        p.eps = en.eps;
        p.fix = en.fix;
    } else {
        p.c = 0; p.pb = 0; p.nv = 0; p.src0 = 0; p.tc = 0.0f; p.sg = 0.0f; p.eps = 0.0f; p.fix = 0;
    }
}

// this lane's (up to) SPL sorted samples of the cloud, 16-byte loads (the runs are padded to 4 samples with NaN;
// the samples past the cloud are NaN as well)
template <int SPL>
__device__ __forceinline__ void px_samples(const LayoutDev &L, const PxCloud &p, int i0, float4 (&w)[SPL / 4]) {
    const float4 *src = (const float4 *)(L.nf + (unsigned)p.pb + i0);
#pragma unroll
    for (int s = 0; s < SPL / 4; s++)
        w[s] = i0 + 4 * s < p.nv ? __ldg(src + s) : make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                                                             __int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
}

// The exact channel of sample i of a cloud (its float32 channel was too close to a half-integer).
__device__ __noinline__ int px_exact(const GridDev &g, const LayoutDev &L, const ZigDev *zig,
                                     const SubMC *__restrict__ subk, int c, int pb, int nv, int i, int *err) {
    const int ir = __ldg(&L.sub[c]);
    const double nx = normal_exact(L, zig, stream_base(L, c, ir, nv), L.ord[(unsigned)pb + i], __ldg(&L.slow_base[c]),
                                   err);
    const long long is = channel_exact_raw(subk[ir], g, L.cd + 4 * (size_t)c, nx, 0);
    return is < -0x3fffffffLL ? -0x3fffffff : (is > 0x3fffffffLL ? 0x3fffffff : (int)is);
}

// Run-length counting of one channel: a run that ends is added to the row, except the lane's first run, kept
// in (fch, fcnt) (see k_mc_deposit_px).
struct PxRuns {
    int cur, cnt, fch, fcnt;
    __device__ __forceinline__ void take(int ch, long long fix, int nz, unsigned long long *row) {
        if (ch != cur) {
            if (cur != (int)0x80000000) {
                if (fch == (int)0x80000000) {
                    fch = cur;
                    fcnt = cnt;
                } else if ((unsigned)cur < (unsigned)nz) {
                    row[cur] += (unsigned long long)(fix * (long long)cnt);
                }
            }
            cur = ch;
            cnt = 0;
        }
        cnt++;
    }
};

// A sample whose exact channel is deferred: added by the warp, with the other deferred samples, between clouds.
struct __align__(16) PxDefer {
    int c, pb, nv, i;       // cloud, its sorted normals, their count, the sample
    long long fix;          // fixed-point flux of the sample
    int row;                // its row in the tile (offset in sums)
    int src0;               // the cloud is placed with member 0's constants
};
#define PX_QCAP 64          // deferred samples per warp (at most 32 join per cloud step)

// The deferred samples of the warp: their exact channels (a lane each) added to the rows with shared-memory
// atomics (two samples may share a channel); the queue is emptied.
__device__ __forceinline__ void px_flush(const GridDev &g, const LayoutDev &L, const ZigDev *zig,
                                         const SubMC *__restrict__ subk, const SubMC *__restrict__ sub0, PxDefer *qe,
                                         int *qn, unsigned long long *tile, int lane, int *err) {
    __syncwarp();
    const int nq = *qn;
    for (int b = 0; b < nq; b += 32) {
        const int e = b + lane;
        if (e < nq) {
            const PxDefer x = qe[e];
            const int ch = px_exact(g, L, zig, x.src0 ? sub0 : subk, x.c, x.pb, x.nv, x.i, err);
            if ((unsigned)ch < (unsigned)g.nz) atomicAdd(tile + x.row + ch, (unsigned long long)x.fix);
        }
    }
    __syncwarp();
    if (lane == 0) *qn = 0;
    __syncwarp();
}

// The channels of this lane's SPL samples counted into the pixel's row (see k_mc_deposit_px). The float32
// channels are binned relative to c0 = (channel of the lane's first sample) - 1 into a register histogram of 11
// five-bit counts, one table increment per sample (a bin holds at most 31 samples unless all 32 of a 32-sample
// lane share one channel, counted apart); a sample too close to a half-integer is left out and deferred to the
// warp's queue. A lane with more than one such sample, a channel beyond the 11 bins (counted in the top bits) or
// a centre out of range counts its samples one by one, with the exact channels where needed.
// The lowest non-empty bin (the lane's first run, which the previous lane may share) is added after the group's
// lanes have merged equal ones; the other bins at once.
template <int SPL>
__device__ __forceinline__ void px_count(const GridDev &g, const LayoutDev &L, const ZigDev *zig,
                                         const SubMC *__restrict__ subk, const SubMC *__restrict__ sub0,
                                         const PxCloud &p, const float4 (&w)[SPL / 4],
                                         int i0, int q, unsigned long long *tile, int rowoff, PxDefer *qe, int *qn,
                                         const unsigned long long *inc, int *err) {
    constexpr int LPP = 128 / SPL;
    const int nz = g.nz;
    unsigned long long *row = tile + rowoff;
    const int m = min(SPL, p.nv - i0);                      // this lane's samples (<= 0: none)
    const bool fastc = fabsf(p.tc) < 1.0e5f;
    const float hw = 0.5f - p.eps;
    const float tc = p.tc, sg = p.sg;
    const long long fix = p.fix;
    // f = sample x sg + (tc + 1/2): the half folded into the centre (one rounding in place of another, within the
    // same bound); samples past the cloud are NaN, which fail the test below and add the empty increment
    const float tc5 = tc + 0.5f;
    const float fl0 = floorf(fmaf(w[0].x, sg, tc5)) - 1.0f;
    const float fl0m = fl0 - 12582912.0f;                  // (exact: an integer below 2^24 in magnitude)
    const float hwf = fastc ? hw : -1.0f;                  // (a centre out of range: no sample passes)
    // straight-line code: each sample adds inc[min(channel - c0, 30)] (bins 0..10 five bits each, a channel
    // beyond them one unit of bits 55..63; index 31: a sample left out)
    unsigned long long H = 0;
    unsigned need = 0;
    int dlast = 0;
#pragma unroll
    for (int s = 0; s < SPL / 4; s++) {
        const float vv[4] = {w[s].x, w[s].y, w[s].z, w[s].w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int i = 4 * s + e;
            const float f = fmaf(vv[e], sg, tc5);
            const float fl = floorf(f);
            const bool ok = fabsf(f - fl - 0.5f) <= hwf;
            const int d = __float_as_int(fl - fl0m) - 0x4B400000;      // (exact: small integers)
            need |= ok ? 0u : 1u << i;
            H += inc[ok ? min((unsigned)d, 30u) : 31u];
            if (SPL == 32) dlast = ok ? d : dlast;
        }
    }
    need &= m >= 32 ? 0xffffffffu : (m > 0 ? (1u << m) - 1u : 0u);
    int fch = (int)0x80000000, fcnt = 0;
    if (__popc(need) <= 1 && (H >> 55) == 0) {
        if (need) {
            const int slot = atomicAdd(qn, 1);
            qe[slot] = PxDefer{p.c, p.pb, p.nv, i0 + __ffs(need) - 1, fix, rowoff, p.src0};
        }
        if (H) {
            const int c0 = (int)fl0;
            const int ntake = m - (need ? 1 : 0);
            const int blo = (__ffsll((long long)H) - 1) / 5;
            // all 32 samples in one channel: 32 overflows its five bits into a single carry bit of H
            const bool one = SPL == 32 && ntake == 32 && H == 1ull << (5 * dlast + 5);
            fch = c0 + (one ? dlast : blo);
            fcnt = one ? 32 : (int)((H >> (5 * blo)) & 31);
#pragma unroll
            for (int b = 0; b < 11; b++) {
                const int cnt = (int)((H >> (5 * b)) & 31);
                const int ch = c0 + b;
                const bool put = !one & (cnt != 0) & (b != blo) & ((unsigned)ch < (unsigned)nz);
                if (put) row[ch] += (unsigned long long)(fix * (long long)cnt);
            }
        }
    } else {
        PxRuns r{(int)0x80000000, 0, (int)0x80000000, 0};
        for (int i = 0; i < m; i++) {
            const float f = fmaf(__ldg(&L.nf[(unsigned)p.pb + i0 + i]), sg, tc) + 0.5f;
            const float fl = floorf(f);
            int c = (int)fl;
            if (!(fastc && fabsf(f - fl - 0.5f) <= hw))
                c = px_exact(g, L, zig, p.src0 ? sub0 : subk, p.c, p.pb, p.nv, i0 + i, err);
            r.take(c, fix, nz, row);
        }
        // the open run: the lane's first run if it is the only one, else its last (a channel no other lane adds)
        if (r.cur != (int)0x80000000) {
            if (r.fch == (int)0x80000000) {
                r.fch = r.cur;
                r.fcnt = r.cnt;
            } else if ((unsigned)r.cur < (unsigned)nz) {
                row[r.cur] += (unsigned long long)(fix * (long long)r.cnt);
            }
        }
        fch = r.fch;
        fcnt = r.fcnt;
    }
    // the lowest runs of the group's lanes: their channels are non-decreasing along the lanes, so equal ones are
    // consecutive; a segmented scan sums them and the last lane of each segment adds the sum (one add per channel)
    __syncwarp();
    int v = fcnt;
#pragma unroll
    for (int d = 1; d < LPP; d <<= 1) {
        const int c2 = __shfl_up_sync(0xffffffffu, fch, d), v2 = __shfl_up_sync(0xffffffffu, v, d);
        if (q >= d && c2 == fch) v += v2;
    }
    const int cn = __shfl_down_sync(0xffffffffu, fch, 1);
    if ((q == LPP - 1 || cn != fch) && (unsigned)fch < (unsigned)nz) row[fch] += (unsigned long long)(fix * (long long)v);
    __syncwarp();
}

// The common case (a linear channel map, one line, at most 128 samples per cloud) with the tile's pixels owned
// by groups of LPP = 128 / SPL lanes: warp w owns the pixels lp = w + 8 grp of the tile (TP = 8 x 32 / LPP
// pixels), and a group takes the clouds of its pixel one after another, so a warp advances 32 / LPP clouds at a
// time. Lane q of a group counts the samples SPL q .. SPL q + SPL - 1 of the cloud in their sorted order (float32
// channels within the rounding bound of the cloud); the samples of the next cloud are loaded during the count.
// The channels are monotone along the sorted samples, so the lanes of a group can only meet on the channel of a
// run that crosses from one lane's samples into the next lane's: every lane's channels but its lowest are added
// at once (distinct channels), and the lowest ones after a segmented scan over the group's lanes.
// A sample within the bound of a half-integer (about one in a thousand) waits in the warp's queue; when the
// queue fills, its exact float64 channels are computed a lane each and added with shared-memory atomics.
// Rows: stride nz + 2 G sums (G pixels per warp) and a skew of 2 grp sums, so that equal channels of the warp's
// pixels fall in different banks.
#ifndef PX_MINB
#define PX_MINB 3         // resident CTAs per SM
#endif
// The channels of member 0's clouds, for the members that differ from it only in the flux of most sub-rings
// (k_mc_deposit_px, delta = 2), summed per (pixel, sub-ring, half): every cloud of such a group has the same
// fixed-point flux in a member, so the member adds count x its flux per channel. A warp per list of member 0
// (a pixel; its lists come first in the bucket, entries bucket[offset[l] .. + count[l]) for l < nlist0) takes its
// clouds in turn: their samples' exact channels as the deposit computes them (float32 within the cloud's
// rounding bound, else the reference's float64 operations), merged into an open record of the same sub-ring and
// half whose window of RP_W channels holds the cloud (the channels do not decrease along a cloud's sorted
// samples), else into a new one (RP_K open at most: when full they are written out). A record: rec = (first
// channel c0, sub-ring | half << 16 | extent << 17: its channels c0 .. c0 + extent - 1), cnt = RP_W 16-bit counts
// in the order of the lanes that add them (lpp lanes a group: channel c0 + d at (d % lpp) (RP_W / lpp) + d / lpp,
// so that each lane's counts are contiguous); at most 65535 samples a record. The records of a list take the
// places of its entries, nrec[l] of them.
#define RP_K 8
__global__ void __launch_bounds__(256) k_replay_records(GridDev g, LayoutDev L, const SubMC *__restrict__ sub0,
                                                        const ZigDev *__restrict__ zig,
                                                        const Entry *__restrict__ bucket,
                                                        const int *__restrict__ offset, const int *__restrict__ count,
                                                        int nlist0, int lpp, int2 *__restrict__ rec,
                                                        uint32_t *__restrict__ cnt, int *__restrict__ nrec,
                                                        unsigned long long *__restrict__ tmask, int nchw, int *err) {
    __shared__ uint32_t h[8][RP_K][RP_W];
    __shared__ int okey[8][RP_K], oc0[8][RP_K], otot[8][RP_K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long l = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (l >= nlist0) return;
    const int beg = __ldg(&offset[l]), n = __ldg(&count[l]);
    int used = 0, nr = 0;
    const int per = RP_W / lpp;                            // counts a lane
    auto flush = [&]() {
        for (int r = 0; r < used; r++) {
            // two 16-bit counts a word, position p = (d % lpp) per + d / lpp for channel c0 + d
            uint32_t v = 0;
#pragma unroll
            for (int b = 0; b < 2; b++) {
                const int p = 2 * lane + b, d = (p % per) * lpp + p / per;
                v |= h[warp][r][d] << (16 * b);
            }
            cnt[(size_t)(beg + nr) * (RP_W / 2) + lane] = v;
            // the extent: the last channel with a count, plus one
            const unsigned any = __ballot_sync(0xffffffffu, (h[warp][r][lane] | h[warp][r][lane + 32]) != 0);
            const unsigned hi = __ballot_sync(0xffffffffu, h[warp][r][lane + 32] != 0);
            const int ext = hi ? 64 - __clz(hi) : 32 - __clz(any);
            if (lane == 0) {
                rec[beg + nr] = make_int2(oc0[warp][r], okey[warp][r] | (ext << 17));
                // (the sub-rings with clouds in the tile)
                const int ir = okey[warp][r] & 0xffff;
                atomicOr(&tmask[(size_t)(l / NOWN) * nchw + (ir >> 6)], 1ull << (ir & 63));
            }
            nr++;
        }
        used = 0;
        __syncwarp();
    };
    for (int e = 0; e < n; e++) {
        const int c = __ldg(&bucket[beg + e].c), half = (__ldg(&bucket[beg + e].meta) >> 24) & 1;
        const int ir = __ldg(&L.sub[c]);
        const SubMC &S = sub0[ir];
        const int nv = __ldg(&L.nvs[ir]);
        const int pb = (int)(L.pbase[ir] + (long long)(c - L.cloud_base[ir]) * ((nv + 3) & ~3));
        float tc, epsc;
        cloud_centre(S, L.cf[c], 0, tc, epsc);
        const float sg = S.sg[0];
        const float nmax = fmaxf(fabsf(__ldg(&L.nf[pb])), fabsf(__ldg(&L.nf[pb + nv - 1])));
        const float eps = fmaf(nmax, fabsf(sg) * EPS_REL, epsc);
        const bool fastc = fabsf(tc) < 1.0e5f;
        const float hw = 0.5f - eps, tc5 = tc + 0.5f;
        int ch[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = lane + 32 * u;
            ch[u] = 0x7fffffff;
            if (i < nv) {
                const float f = fmaf(__ldg(&L.nf[pb + i]), sg, tc5);
                const float fl = floorf(f);
                ch[u] = (fastc && fabsf(f - fl - 0.5f) <= hw) ? (int)fl : px_exact(g, L, zig, sub0, c, pb, nv, i, err);
            }
        }
        const int cmin = __shfl_sync(0xffffffffu, ch[0], 0);
        const int last = nv - 1;
        const int cmax = __shfl_sync(0xffffffffu, ch[last >> 5], last & 31);
        const int key = ir | (half << 16);
        // an open record of the key whose window holds the cloud (lane r tests record r)
        bool fit = false;
        if (lane < used)
            fit = okey[warp][lane] == key && cmin >= oc0[warp][lane] && cmax < oc0[warp][lane] + RP_W &&
                  otot[warp][lane] + nv <= 65535;
        const unsigned m = __ballot_sync(0xffffffffu, fit);
        int r;
        if (m) {
            r = __ffs(m) - 1;
        } else {
            if (used == RP_K) flush();
            r = used++;
            for (int x = lane; x < RP_W; x += 32) h[warp][r][x] = 0;
            if (lane == 0) { okey[warp][r] = key; oc0[warp][r] = cmin; otot[warp][r] = 0; }
            __syncwarp();
        }
        const int base = oc0[warp][r];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (lane + 32 * u < nv) {
                const int d = ch[u] - base;
                if ((unsigned)d < (unsigned)RP_W) atomicAdd(&h[warp][r][d], 1u);
                else atomicOr(err, ERR_SHARE);
            }
        }
        if (lane == 0) otot[warp][r] += nv;
        __syncwarp();
    }
    flush();
    if (lane == 0) nrec[l] = nr;
}

template <int SPL>
__global__ void __launch_bounds__(256, PX_MINB) k_mc_deposit_px(GridDev g, LayoutDev L, const SubMC *__restrict__ sub,
                                                              int nsub, const MemberDev *__restrict__ mem, int tx,
                                                              int ty, const int *__restrict__ offset,
                                                              const int *__restrict__ count,
                                                              const Entry *__restrict__ bucket,
                                                              const ZigDev *__restrict__ zig,
                                                              const float *__restrict__ cd2if,
                                                              float *__restrict__ model, long long mstride,
                                                              const int *__restrict__ klist, int delta,
                                                              unsigned long long *__restrict__ base64,
                                                              int *__restrict__ tsrc, Replay rp, int *err) {
    constexpr int LPP = 128 / SPL;
    extern __shared__ unsigned long long tile[];           // TP rows of fixed-point sums, queues, nz scales
    __shared__ unsigned long long inc[32];                 // the histogram increments of px_count
    const int k = klist ? klist[blockIdx.x] : blockIdx.x;
    const int t = blockIdx.y;
    // delta: the member's lists hold the difference from member 0's model (same box and exponent), whose sums
    // are in base64, and a tile without entries is left unwritten (tsrc points the convolution to member 0's
    // model there); else member 0 (with base64) leaves its sums there
    unsigned long long *wbase = !delta && k == 0 ? base64 : nullptr;
    if (delta == 1 && threadIdx.x == 0 && blockIdx.y == 0 && mem[k].fix_exp != mem[0].fix_exp)
        atomicOr(err, ERR_SHARE);
    const int ntx = mem[k].ntx;
    if (t >= ntx * mem[k].nty) return;
    if (threadIdx.x < 32) inc[threadIdx.x] = threadIdx.x < 11 ? 1ull << (5 * threadIdx.x) : (threadIdx.x < 31 ? 1ull << 55 : 0ull);
    constexpr int G = 32 / LPP;                             // pixels per warp
    const int nz = g.nz, RS = nz + 2 * G;
    const int TP = tx * ty;
    const int tyi = t / ntx, txi = t - tyi * ntx;
    const int x0 = txi * tx, y0 = tyi * ty;
    const int bx = mem[k].bx, by = mem[k].by;
    const int lbase = (mem[k].tile_off + t) * NOWN;
    const int lbase0 = (mem[0].tile_off + t) * NOWN;       // (replay: member 0's lists of the same tile)
    const bool replay = delta == 2;
    float *mout = model + (size_t)k * mstride;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    {
        int any = 0;
        if (threadIdx.x < NOWN) any = count[lbase + threadIdx.x] != 0 || (replay && count[lbase0 + threadIdx.x] != 0);
        // a difference with member 0's records: also the tiles where member 0 has clouds of the changed sub-rings
        if (delta == 1 && rp.rec && threadIdx.x < rp.nchw)
            any |= (rp.tmask[(size_t)t * rp.nchw + threadIdx.x] & rp.chg[(size_t)k * rp.nchw + threadIdx.x]) != 0;
        if (!__syncthreads_or(any)) {
            if (tsrc && threadIdx.x == 0) tsrc[mem[k].tile_off + t] = delta == 1 ? 0 : k;
            if (delta == 1) return;
            for (int lp = warp; lp < TP; lp += 8) {
                const int py = y0 + lp / tx, px = x0 + lp % tx;
                if (py >= by || px >= bx) continue;
                const size_t v0 = ((size_t)py * bx + px) * nz;
                float *o = mout + v0;
                for (int z = lane; z < nz; z += 32) o[z] = 0.0f;
                if (wbase)
                    for (int z = lane; z < nz; z += 32) wbase[v0 + z] = 0ULL;
            }
            return;
        }
    }
    if (tsrc && threadIdx.x == 0) tsrc[mem[k].tile_off + t] = k;
    PxDefer *qall = (PxDefer *)(tile + (size_t)TP * RS);   // (16-byte aligned: TP RS is even)
    int *qns = (int *)(qall + 8 * PX_QCAP);
    float *chs = (float *)(qns + 8);
    {
        const int nt = TP * RS;
        if (threadIdx.x < 8) qns[threadIdx.x] = 0;
        ulonglong2 *t2 = (ulonglong2 *)tile;
        for (int i = threadIdx.x; i < nt / 2; i += blockDim.x) t2[i] = make_ulonglong2(0ULL, 0ULL);
        const int fe = mem[k].fix_exp;
        for (int z = threadIdx.x; z < nz; z += blockDim.x) chs[z] = ldexpf(cd2if[z], -fe);
    }
    __syncthreads();
    const int grp = lane / LPP, q = lane % LPP;
    const int lp = warp + 8 * grp;
    const bool own = lp < TP;
    const int beg = own ? offset[lbase + 8 * warp + grp] : 0;
    const int n = own ? count[lbase + 8 * warp + grp] : 0;
    const int rowoff = (own ? lp : 0) * RS + 2 * grp;
    PxDefer *qe = qall + warp * PX_QCAP;
    int *qn = qns + warp;
    const SubMC *__restrict__ subk = sub + (size_t)k * nsub;
    if (replay || (delta == 1 && rp.rec)) {
        // member 0's clouds of the pixel from its channel counts summed per (sub-ring, half) (k_replay_records):
        // a replay adds those of the sub-rings where the member is member 0 but for the flux, times the member's
        // fixed-point flux; a difference takes out those of the changed sub-rings, times member 0's (the member's
        // own clouds of those sub-rings are in its lists). Lane q of the group takes the channels c0 + q + LPP i of
        // a record's extent (its counts are contiguous in the record); the next record is loaded during the adds
        constexpr int CPL = RP_W / LPP, WPL = CPL / 2;      // channels, 32-bit words (two counts) per lane
        const unsigned long long *chg = rp.chg + (size_t)k * rp.nchw;
        unsigned long long *row = tile + rowoff;
        const int beg0 = own ? offset[lbase0 + 8 * warp + grp] : 0;
        const int n0 = own ? rp.nrec[lbase0 + 8 * warp + grp] : 0;
        const int nj0 = __reduce_max_sync(0xffffffffu, n0);
        auto load = [&](int jj, int2 &r, uint32_t (&w)[WPL]) {
            if (jj < n0) {
                r = __ldg(&rp.rec[beg0 + jj]);
                const uint4 *cw = (const uint4 *)(rp.cnt + (size_t)(beg0 + jj) * (RP_W / 2) + WPL * q);
#pragma unroll
                for (int x = 0; x < WPL / 4; x++) {
                    const uint4 v = __ldg(&cw[x]);
                    w[4 * x] = v.x; w[4 * x + 1] = v.y; w[4 * x + 2] = v.z; w[4 * x + 3] = v.w;
                }
            } else {
                r = make_int2(0, -1);
            }
        };
        int2 ra;
        uint32_t wa[WPL];
        load(0, ra, wa);
        for (int jj = 0; jj < nj0; jj++) {
            int2 rb;
            uint32_t wb[WPL];
            load(jj + 1, rb, wb);
            if (ra.y >= 0) {
                const int ir = ra.y & 0xffff;
                const bool changed = (__ldg(&chg[ir >> 6]) >> (ir & 63)) & 1ull;
                if (replay != changed) {
                    const long long fix = replay ? subk[ir].fix[(ra.y >> 16) & 1][0] : -sub[ir].fix[(ra.y >> 16) & 1][0];
                    const int ext = (ra.y >> 17) & 127;
                    const int ni = (ext - q + LPP - 1) / LPP;  // this lane's channels in the extent
#pragma unroll
                    for (int x = 0; x < CPL; x++) {
                        if (x >= ni) break;
                        const int cnt = (wa[x >> 1] >> (16 * (x & 1))) & 0xffff, ch = ra.x + q + LPP * x;
                        if (cnt && (unsigned)ch < (unsigned)nz) row[ch] += (unsigned long long)(fix * (long long)cnt);
                    }
                }
            }
            ra = rb;
#pragma unroll
            for (int w = 0; w < WPL; w++) wa[w] = wb[w];
        }
        __syncwarp();
    }
    const int nj = __reduce_max_sync(0xffffffffu, n);
    const int i0 = SPL * q;                                 // this lane's samples: i0 .. min(i0 + SPL, nv) - 1
    // software pipeline: the samples of the next cloud and the entry after it are loaded during a count
    PxCloud ca, cb;
    float4 wa[SPL / 4], wb[SPL / 4];
    px_entry(bucket, beg, n, 0, ca);
    px_samples<SPL>(L, ca, i0, wa);
    px_entry(bucket, beg, n, 1, cb);
    for (int j = 0; j < nj; j++) {
        px_samples<SPL>(L, cb, i0, wb);
        PxCloud cn;
        px_entry(bucket, beg, n, j + 2, cn);
        px_count<SPL>(g, L, zig, subk, sub, ca, wa, i0, q, tile, rowoff, qe, qn, inc, err);
        __syncwarp();
        if (*qn > PX_QCAP - 32) px_flush(g, L, zig, subk, sub, qe, qn, tile, lane, err);
        ca = cb;
        cb = cn;
#pragma unroll
        for (int s = 0; s < SPL / 4; s++) wa[s] = wb[s];
    }
    __syncwarp();
    if (*qn) px_flush(g, L, zig, subk, sub, qe, qn, tile, lane, err);
    __syncthreads();
    for (int p = warp; p < TP; p += 8) {
        const int py = y0 + p / tx, px = x0 + p % tx;
        if (py >= by || px >= bx) continue;
        const unsigned long long *src = tile + (size_t)p * RS + 2 * (p >> 3);
        const size_t v0 = ((size_t)py * bx + px) * nz;
        float *o = mout + v0;
        if (delta == 1) {
            for (int z = lane; z < nz; z += 32) o[z] = ll_to_f32((long long)(src[z] + base64[v0 + z])) * chs[z];
        } else {
            for (int z = lane; z < nz; z += 32) o[z] = ll_to_f32((long long)src[z]) * chs[z];
            if (wbase)
                for (int z = lane; z < nz; z += 32) wbase[v0 + z] = src[z];
        }
    }
}

// The constants of the sub-rings that a member shares with member 0 (reused = 1; the host left them unwritten):
// member 0's, with the fixed-point deposits of the member's own exponent (the host's llrint(valrel w Q)).
__global__ void k_fill_submc(SubMC *__restrict__ sub, int nsub, int nb, const signed char *__restrict__ reused,
                             const MemberDev *__restrict__ mem, int nlines) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nb * nsub) return;
    if (!reused[i]) return;
    const int k = (int)(i / nsub), ir = (int)(i - (long long)k * nsub);
    SubMC S = sub[ir];
    if (S.active) {
        const double Q = ldexp(1.0, mem[k].fix_exp);
        for (int nl = 0; nl < nlines && nl < BBGPU_MAXL; nl++) {
            S.fix[0][nl] = __double2ll_rn(__dmul_rn(__dmul_rn(S.valrel[nl], S.wrec), Q));
            S.fix[1][nl] = __double2ll_rn(__dmul_rn(__dmul_rn(S.valrel[nl], S.wapp), Q));
        }
    }
    sub[i] = S;
}

// A plain copy of member 0's entry into the entries marked reused (structures of 8-byte words).
__global__ void k_fill_copy(unsigned long long *__restrict__ base, int words, int nsub, int nb,
                            const signed char *__restrict__ reused) {
    const long long i = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (i >= (long long)nb * nsub || !reused[i]) return;
    const int ir = (int)(i % nsub);
    for (int w = threadIdx.x & 31; w < words; w += 32) base[(size_t)i * words + w] = base[(size_t)ir * words + w];
}

// exclusive scan of n counts in three passes: block sums, scan of the sums, block scans
__global__ void k_scan_a(const int *__restrict__ count, int n, int *__restrict__ bsum) {
    __shared__ int r[32];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    int v = i < n ? count[i] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = r[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) bsum[blockIdx.x] = v;
    }
}

__global__ void k_scan_b(int *__restrict__ bsum, int nb) {
    // one CTA of 1024 threads over nb block sums (chunks per thread), in place, exclusive
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int chunk = (nb + 1023) / 1024;
    const int b = t * chunk, e = min(nb, b + chunk);
    int s = 0;
    for (int i = b; i < e; i++) s += bsum[i];
    part[t] = s;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        int v = t >= d ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int i = b; i < e; i++) {
        const int c = bsum[i];
        bsum[i] = run;
        run += c;
    }
}

__global__ void k_scan_c(const int *__restrict__ count, int n, const int *__restrict__ bsum, int *__restrict__ offset,
                         int *__restrict__ cursor) {
    __shared__ int r[32];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int v = i < n ? count[i] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) r[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = r[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        r[lane] = w;
    }
    __syncthreads();
    const int ex = x - v + (wid > 0 ? r[wid - 1] : 0) + bsum[blockIdx.x];
    if (i < n) {
        offset[i] = ex;
        cursor[i] = ex;
    }
}

}  // namespace

void launch_replay_records(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub0,
                           const ZigDev *zig, const void *bucket, const int *offset, const int *count, int nlist0,
                           int tp, int *rec, uint32_t *cnt, int *nrec, unsigned long long *tmask, int nchw,
                           int *err) {
    if (nlist0 <= 0) return;
    cudaMemsetAsync(tmask, 0, sizeof(unsigned long long) * (size_t)(nlist0 / NOWN) * nchw, s);
    const long long nt = 32LL * nlist0;
    const int lpp = tp == 64 ? 4 : 8;                      // lanes a pixel of k_mc_deposit_px (128 / SPL)
    k_replay_records<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(g, L, sub0, zig, (const Entry *)bucket, offset, count,
                                                                 nlist0, lpp, (int2 *)rec, cnt, nrec, tmask, nchw,
                                                                 err);
}

void launch_mc_bin(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub, int nsub,
                   const MemberDev *mem, const long long *cstart, const int *cseg, int nseg, long long ntot, int tx,
                   int ty, int *pix, int *tile_count, int *err) {
    if (ntot == 0 || nseg == 0) return;
    k_mc_bin<<<(unsigned)((ntot + 255) / 256), 256, 0, s>>>(g, L, sub, nsub, mem, cstart, (const int4 *)cseg, nseg,
                                                            ntot, tx, ty, pix, tile_count, err);
}

void launch_scan_tiles(cudaStream_t s, const int *count, int *offset, int *cursor, int n, int *scratch) {
    const int nb = (n + 1023) / 1024;
    if (nb == 0) return;
    k_scan_a<<<nb, 1024, 0, s>>>(count, n, scratch);
    k_scan_b<<<1, 1024, 0, s>>>(scratch, nb);
    k_scan_c<<<nb, 1024, 0, s>>>(count, n, scratch, offset, cursor);
}

void launch_mc_scatter(cudaStream_t s, const LayoutDev &L, const SubMC *sub, int nsub, const MemberDev *mem,
                       const long long *cstart, const int *cseg, int nseg, long long ntot, int tx, int ty,
                       const int *pix, int *cursor, void *bucket, int defer_fix) {
    if (ntot == 0 || nseg == 0) return;
    k_mc_scatter<<<(unsigned)((ntot + 255) / 256), 256, 0, s>>>(L, sub, nsub, mem, cstart, (const int4 *)cseg, nseg,
                                                                ntot, tx, ty, pix, cursor, (Entry *)bucket,
                                                                defer_fix);
}

void launch_entry_fix(cudaStream_t s, const SubMC *sub, const int *offset, const int *count, int nlist,
                      long long ntot, void *bucket) {
    if (ntot == 0 || nlist == 0) return;
    k_entry_fix<<<(unsigned)((ntot + 255) / 256), 256, 0, s>>>(sub, offset, count, nlist, (Entry *)bucket);
}

bool mc_deposit_shares(int lean, bool model64, int tx, int ty) {
    return lean && !model64 && (tx * ty == 64 || tx * ty == 32);
}

// dynamic shared memory of the pixel-owned deposit (TP pixels a tile), the kernel configured for it once
static size_t px_smem(const GridDev &g, int TP) {
    const size_t smem_px = (size_t)TP * (g.nz + TP / 4) * sizeof(unsigned long long) +
                           (size_t)8 * PX_QCAP * sizeof(PxDefer) + 8 * sizeof(int) + (size_t)g.nz * sizeof(float);
    static size_t cfg32 = 0, cfg16 = 0;
    size_t &cfg = TP == 64 ? cfg32 : cfg16;
    if (smem_px > 48 * 1024 && smem_px > cfg) {
        if (TP == 64)
            cudaFuncSetAttribute(k_mc_deposit_px<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_px);
        else
            cudaFuncSetAttribute(k_mc_deposit_px<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_px);
        cfg = smem_px;
    }
    return smem_px;
}

void launch_mc_deposit(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub, int nsub,
                       const MemberDev *mem, const MemberDev *mem_host, int nb, int tx, int ty,
                       const int *offset, const int *count, const void *bucket, const ZigDev *zig,
                       const float *cd2if, const double *cd2i, float *model, long long mstride, double *model64,
                       int *err, int lean, const int *klist, int nk, int delta, long long *base64, int *tsrc,
                       Replay rp) {
    int maxt = 0;
    for (int k = 0; k < nb; k++) maxt = max(maxt, mem_host[k].ntx * mem_host[k].nty);
    if (maxt == 0 || nb == 0 || (klist && nk == 0)) return;
    size_t smem = (size_t)tx * ty * g.nz * sizeof(unsigned long long) + 16 + (size_t)8 * DEPTH * WB * sizeof(float) +
                  (size_t)g.nz * sizeof(float);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_mc_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    dim3 grid(klist ? nk : nb, maxt);
    if (lean && !model64) {
        static size_t cfg_lean = 0;
        if (smem > 48 * 1024 && smem > cfg_lean) {
            cudaFuncSetAttribute(k_mc_deposit_lean, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cfg_lean = smem;
        }
        const int TP = tx * ty;
        if (TP == 64 || TP == 32) {
            // pixel-owned deposit: 8 (TP 64) or 4 (TP 32) pixels per warp
            const size_t smem_px = px_smem(g, TP);
            unsigned long long *b64 = (unsigned long long *)base64;
            if (TP == 64)
                k_mc_deposit_px<32><<<grid, 256, smem_px, s>>>(g, L, sub, nsub, mem, tx, ty, offset, count,
                                                               (const Entry *)bucket, zig, cd2if, model, mstride,
                                                               klist, delta, b64, tsrc, rp, err);
            else
                k_mc_deposit_px<16><<<grid, 256, smem_px, s>>>(g, L, sub, nsub, mem, tx, ty, offset, count,
                                                               (const Entry *)bucket, zig, cd2if, model, mstride,
                                                               klist, delta, b64, tsrc, rp, err);
            return;
        }
        k_mc_deposit_lean<<<grid, 256, smem, s>>>(g, L, sub, nsub, mem, tx, ty, offset, count, (const Entry *)bucket,
                                                 zig, cd2if, model, mstride, err);
        return;
    }
    k_mc_deposit<<<grid, 256, smem, s>>>(g, L, sub, nsub, mem, tx, ty, offset, count, (const Entry *)bucket, zig, cd2if,
                                        cd2i, model, mstride, model64, err);
}

void launch_fill_submc(cudaStream_t s, SubMC *sub, int nsub, int nb, const signed char *reused, const MemberDev *mem,
                       int nlines) {
    const long long n = (long long)nb * nsub;
    if (n == 0) return;
    k_fill_submc<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(sub, nsub, nb, reused, mem, nlines);
}

void launch_fill_copy(cudaStream_t s, void *base, size_t elt_bytes, int nsub, int nb, const signed char *reused) {
    const long long n = (long long)nb * nsub;
    if (n == 0) return;
    k_fill_copy<<<(unsigned)((n + 7) / 8), 256, 0, s>>>((unsigned long long *)base, (int)(elt_bytes / 8), nsub, nb,
                                                       reused);
}
