// The Monte-Carlo GALMOD deposit on the device (the reference's _galmod_mc, bbarolo/galmod.py:92-171).
//
// The clouds of a sub-ring are drawn from one xoroshiro128+ stream; their draws do not depend on the ring
// parameters, so the host parses the stream once per (seed, layer, cloud counts) into a layout: per cloud
// its radius R, cos/sin of its azimuth and its layer deviate, per sub-cloud the first word of its normal
// deviate (the values of the rare normals that took the slow path of the ziggurat in a side list).
//
// Per evaluation two kernels place the clouds:
//   k_mc_bin      pixel of every cloud in the member's box, and the count of clouds per pixel tile;
//   k_mc_scatter  the clouds of each tile gathered into a bucket (counting sort by tile);
//   k_mc_deposit  one CTA per (member, tile): every sub-cloud of the tile's clouds is added, in 64-bit fixed
//                 point, to a shared-memory tile (pixels x channels), written once to HBM at the end.
// Fixed-point sums are exact and independent of the order of the deposits: the model is deterministic.
//
// Indices are bit-exact with the reference: each pixel and channel is first computed in float32 with a
// bound on its rounding error; when the value lies within that bound of a rounding boundary (a half
// integer) it is recomputed with the reference's float64 operations, in its order, with no contraction
// (__dmul_rn/__dadd_rn/__ddiv_rn/__dsqrt_rn), so lround() gives the reference's integer.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

#define C_MS 2.99792458e08
#define ERR_LAYOUT 1

namespace {

// bbarolo/galmod.py:38-46
__device__ __forceinline__ long long lround_ref(double x) {
    if (!(fabs(x) < 1e18)) return -(1LL << 62);
    if (x >= 0) return (long long)__dadd_rn(x, 0.5);
    return -(long long)__dadd_rn(-x, 0.5);
}

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

// bbarolo/galmod.py:49-62
__device__ __forceinline__ double velgrid_exact(double v, const GridDev &g, int nl) {
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

__global__ void k_mc_bin(GridDev g, LayoutDev L, const SubMC *__restrict__ sub, int nsub,
                         const MemberDev *__restrict__ mem, int nb, int tx, int ty, int *__restrict__ pix,
                         int *__restrict__ tile_count, int *err) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nb * L.ncloud) return;
    int k = (int)(idx / L.ncloud);
    int c = (int)(idx - (long long)k * L.ncloud);
    int ir = L.sub[c];
    const SubMC &S = sub[(size_t)k * nsub + ir];
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
    atomicAdd(&tile_count[M.tile_off + (py / ty) * M.ntx + px / tx], 1);
}

__global__ void k_scan_tiles(const int *__restrict__ count, int *__restrict__ offset, int *__restrict__ cursor,
                             int n) {
    // one CTA of 1024 threads: each scans a contiguous chunk, then the chunk totals are scanned
    __shared__ int part[1024];
    int t = threadIdx.x;
    int chunk = (n + 1023) / 1024;
    int b = t * chunk, e = min(n, b + chunk);
    int s = 0;
    for (int i = b; i < e; i++) s += count[i];
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
        offset[i] = run;
        cursor[i] = run;
        run += count[i];
    }
}

__global__ void k_mc_scatter(LayoutDev L, const MemberDev *__restrict__ mem, int nb, int tx, int ty,
                             const int *__restrict__ pix, int *__restrict__ cursor, int *__restrict__ bucket) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nb * L.ncloud) return;
    int p = pix[idx];
    if (p < 0) return;
    int k = (int)(idx / L.ncloud);
    int c = (int)(idx - (long long)k * L.ncloud);
    const MemberDev &M = mem[k];
    int py = p / M.bx, px = p - py * M.bx;
    int slot = atomicAdd(&cursor[M.tile_off + (py / ty) * M.ntx + px / tx], 1);
    bucket[slot] = c;
}

__global__ void __launch_bounds__(256) k_mc_deposit(GridDev g, LayoutDev L, const SubMC *__restrict__ sub, int nsub,
                                                    const MemberDev *__restrict__ mem, int tx, int ty,
                                                    const int *__restrict__ pix, const int *__restrict__ offset,
                                                    const int *__restrict__ count, const int *__restrict__ bucket,
                                                    const ZigDev *__restrict__ zig, const float *__restrict__ cd2if,
                                                    const double *__restrict__ cd2i, float *__restrict__ model,
                                                    long long mstride, double *__restrict__ model64, int *err) {
    extern __shared__ unsigned long long tile[];
    __shared__ unsigned s_kn[128];
    __shared__ float s_wnf[128];
    __shared__ double s_wn[128];
    const int k = blockIdx.x;
    const MemberDev &M = mem[k];
    const int t = blockIdx.y;
    if (t >= M.ntx * M.nty) return;
    const int nz = g.nz;
    const int TP = tx * ty;
    for (int i = threadIdx.x; i < TP * nz; i += blockDim.x) tile[i] = 0ULL;
    for (int i = threadIdx.x; i < 128; i += blockDim.x) {
        s_kn[i] = zig->kn[i];
        s_wnf[i] = zig->wnf[i];
        s_wn[i] = zig->wn[i];
    }
    __syncthreads();
    const int tyi = t / M.ntx, txi = t - tyi * M.ntx;
    const int x0 = txi * tx, y0 = tyi * ty;
    const int beg = offset[M.tile_off + t], n = count[M.tile_off + t];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned ltmask = (1u << lane) - 1u;
    const int nlines = g.nlines;
    for (int e = warp; e < n; e += nw) {
        const int c = bucket[beg + e];
        const int p = pix[(size_t)k * L.ncloud + c];
        const int py = p / M.bx, px = p - py * M.bx;
        const int lp = (py - y0) * tx + (px - x0);
        const int ir = L.sub[c];
        const SubMC &S = sub[(size_t)k * nsub + ir];
        const float4 cf = L.cf[c];
        const double *cd = L.cd + 4 * (size_t)c;
        const int half = cf.y >= 0.0f ? 0 : 1;
        // channel centre of the cloud (fast path): c0 + (vr caz + vrad saz) sin(i) ia, vr lagged above zcyl
        const float zf = cf.w * S.z0f;
        const float azf = fabsf(zf);
        float vr = S.vrotf;
        if (azf > S.zcylf) {
            float v = S.vrotf - S.dvdzf * (azf - S.zcylf);
            vr = S.vrotf >= 0.0f ? fmaxf(v, 0.0f) : fminf(v, 0.0f);
        }
        const float base = vr * cf.y + S.vradf * cf.z;
        const float mbase = fabsf(vr * cf.y) + fabsf(S.vradf * cf.z) + fabsf(S.dvdzf) * (azf + fabsf(S.zcylf));
        const long long sb = L.sub_base[ir] + (long long)(c - L.cloud_base[ir]) * S.nv;
        int slow_ord = L.slow_base[c];
        bool have_vs = false;
        double vs = 0.0;
        unsigned long long *row = tile + (size_t)lp * nz;
        for (int it = 0; it < S.nv; it += 32) {
            const int iv = it + lane;
            const bool act = iv < S.nv;
            const int h = act ? L.hz[sb + iv] : 0;
            const int iz = h & 127;
            const unsigned ah = h < 0 ? (unsigned)(-(long long)h) : (unsigned)h;
            const bool slow = act && !(ah < s_kn[iz]);
            const unsigned bal = __ballot_sync(0xffffffffu, slow);
            double nex = 0.0;
            float nf;
            if (slow) {
                const long long o = (long long)slow_ord + __popc(bal & ltmask);
                if (o < L.nslow) {
                    nex = L.slow_val[o];
                } else {
                    atomicOr(err, ERR_LAYOUT);
                    nex = 0.0;
                }
                nf = (float)nex;
            } else {
                nf = __int2float_rn(h) * s_wnf[iz];
            }
            slow_ord += __popc(bal);
            if (!act) continue;
            for (int nl = 0; nl < nlines; nl++) {
                int isub;
                bool ok = false;
                if (g.fast_ok) {
                    const float tc = S.c0[nl] + base * S.sia[nl];
                    const float ns = nf * S.sg[nl];
                    const float eps = (fabsf(S.c0[nl]) + mbase * fabsf(S.sia[nl]) + fabsf(ns) + 1.0f) * EPS_REL;
                    ok = round_fast(tc + ns, eps, isub);
                }
                if (!ok) {
                    if (!have_vs) {
                        vs = vlos_exact(S, cd);
                        have_vs = true;
                    }
                    const double nx = slow ? nex : __dmul_rn((double)h, s_wn[iz]);
                    long long is;
                    if (g.axtyp == 4 && nlines == 1) {
                        double gz = __dadd_rn(__dmul_rn(vs, g.ia), g.ib);
                        double sg = __dmul_rn(S.vdisptmp, g.ia);
                        is = lround_ref(__dadd_rn(gz, __dmul_rn(nx, sg)));
                    } else {
                        double v = __dadd_rn(vs, __dmul_rn(nx, S.vdisptmp));
                        is = lround_ref(velgrid_exact(v, g, nl));
                    }
                    isub = (is < 0 || is >= nz) ? -1 : (int)is;
                }
                if (isub >= 0 && isub < nz) atomicAdd(&row[isub], (unsigned long long)S.fix[half][nl]);
            }
        }
    }
    __syncthreads();
    float *mout = model + (size_t)k * mstride;
    for (int i = threadIdx.x; i < TP * nz; i += blockDim.x) {
        const int lp = i / nz, z = i - lp * nz;
        const int py = y0 + lp / tx, px = x0 + lp % tx;
        if (py >= M.by || px >= M.bx) continue;
        const long long v = (long long)tile[i];
        const size_t o = ((size_t)py * M.bx + px) * nz + z;
        mout[o] = ldexpf(__ll2float_rn(v) * cd2if[z], -M.fix_exp);
        if (model64) model64[(size_t)k * mstride + o] = ldexp((double)v * cd2i[z], -M.fix_exp);
    }
}

}  // namespace

void launch_mc_bin(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub, int nsub,
                   const MemberDev *mem, int nb, int tx, int ty, int *pix, int *tile_count, int *err) {
    long long n = (long long)nb * L.ncloud;
    if (n == 0) return;
    k_mc_bin<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, L, sub, nsub, mem, nb, tx, ty, pix, tile_count, err);
}

void launch_scan_tiles(cudaStream_t s, const int *count, int *offset, int *cursor, int n) {
    k_scan_tiles<<<1, 1024, 0, s>>>(count, offset, cursor, n);
}

void launch_mc_scatter(cudaStream_t s, const LayoutDev &L, const MemberDev *mem, int nb, int tx, int ty,
                       const int *pix, int *cursor, int *bucket) {
    long long n = (long long)nb * L.ncloud;
    if (n == 0) return;
    k_mc_scatter<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(L, mem, nb, tx, ty, pix, cursor, bucket);
}

void launch_mc_deposit(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub, int nsub,
                       const MemberDev *mem, const MemberDev *mem_host, int nb, int tx, int ty, const int *pix,
                       const int *offset, const int *count, const int *bucket, const ZigDev *zig,
                       const float *cd2if, const double *cd2i, float *model, long long mstride, double *model64,
                       int *err) {
    int maxt = 0;
    for (int k = 0; k < nb; k++) maxt = max(maxt, mem_host[k].ntx * mem_host[k].nty);
    if (maxt == 0 || nb == 0) return;
    size_t smem = (size_t)tx * ty * g.nz * sizeof(unsigned long long);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_mc_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    dim3 grid(nb, maxt);
    k_mc_deposit<<<grid, 256, smem, s>>>(g, L, sub, nsub, mem, tx, ty, pix, offset, count, bucket, zig, cd2if, cd2i,
                                        model, mstride, model64, err);
}
