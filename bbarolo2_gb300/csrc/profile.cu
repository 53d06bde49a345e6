// The flux normalisation of the batched likelihood on the device: the deconvolved density profile of
// Bayesian3DFIT (bbarolo/bayesian/density.py:39-88, bbarolo/profile.py:33-138) for every member of a batch.
//
//   k_an_maps_fast   the total-intensity map of each ring with unit density (the ANALYTIC samples of
//                    _ring_maps_analytic, bbarolo/galmod.py:468-536), one thread per (member, azimuth sample),
//                    its heights in order: pixels in float32 with a rounding bound (float64 near a boundary, so
//                    every sample lands on the reference's pixel), run weights in float32, runs queued in shared
//                    memory and deposited by the whole warp, 64-bit fixed-point sums (deterministic); maps
//                    (member, pixel, ring) ring-fastest in the likelihood box;
//   k_maps_to_f32    x mean(cd2i) sum(relint) x scale factor, float32 (then the beam convolution of
//                    k_conv_resid with the rings as channels);
//   k_prof_gram      the normal equations of the weighted least squares: G = A^T A, h = A^T b over the pixels
//                    used (A = maps / rms), exact float64 products of the float32 maps, fixed-order sums;
//   k_prof_solve     one CTA per member: solve_profile's two non-negative least-squares solves with the
//                    smoothness prior, Lawson-Hanson on the normal equations (Cholesky of the passive set),
//                    warm-started from a passive set;
//   k_mc_dens        the densities of the model's sub-rings (ring weights) into the MC sub-ring constants
//                    (flux per sub-cloud, fixed-point deposits and exponent), checking the cloud layout;
//   k_an_dens        the same for an ANALYTIC model (flux per sample, line amplitudes, exponent).
//
// The maps need float32 accuracy only: the system is well conditioned (cond(A) ~ 1e2 on the 160x160x128
// workload) and float32 map errors move the densities by ~1e-8; the Gram matrix squares the condition number
// and is therefore accumulated in float64.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "anpix.cuh"
#include "devmath.cuh"
#include "kernels.h"

#define FULL 0xffffffffu
#define EPS_REL 3.814697265625e-06f
#define GRAM_TP 128         // pixels per CTA of k_prof_gram

namespace {

// ------------------------------------------------------------------------------------------- ring maps
// One thread per (member, azimuth sample); its heights in order, consecutive heights in one pixel merged into
// a run (the reference's order), each run deposited into the maps of its one or two rings. The pixels:
// sample_pixel (float32 with a rounding bound, exact fallbacks).
//
// The finished runs of a thread wait in a shared-memory queue (pixel, weight) and are deposited by the whole
// warp at once when a queue is full and at the end: the warp's loop over heights then carries no divergent
// deposit code, and each drain pass keeps all lanes busy. The sums are 64-bit fixed point, so the order of
// the deposits does not change the maps.
#define MAPS_TB 128         // threads per CTA
#define MAPS_QD 16          // queued runs per thread

#ifndef MAPS_MINB
#define MAPS_MINB 8         // resident CTAs per SM (64 registers)
#endif
__global__ void __launch_bounds__(MAPS_TB, MAPS_MINB) k_an_maps_fast(GridDev g, const AnSub *__restrict__ subs, int nsub,
                                                          const int *__restrict__ sbase, const int *__restrict__ ssub,
                                                          const double2 *__restrict__ cs,
                                                          const float2 *__restrict__ csf,
                                                          const long long *__restrict__ mstart,
                                                          const int4 *__restrict__ mseg, int nseg, long long ntot,
                                                          const double *__restrict__ zq,
                                                          const float *__restrict__ zqf,
                                                          const float *__restrict__ wqf, const int *__restrict__ widx,
                                                          const float *__restrict__ wvalf, ProfBox box,
                                                          const int *__restrict__ fix_exp,
                                                          unsigned long long *__restrict__ maps64) {
    __shared__ uint2 runq[MAPS_QD][MAPS_TB];
    const int tid = threadIdx.x;
    const long long gs = (long long)blockIdx.x * MAPS_TB + tid;
    // this thread's sample; nzz = 0: nothing to deposit (the thread still takes part in the warp's drains)
    int u = 0, kr = 0, nzz = 0, off = 0, i0 = -1, i1 = -1;
    long long s = 0;
    const AnSub *S = subs;
    PixF px{};
    float v0 = 0.f, v1 = 0.f;
    if (gs < ntot) {
        int lo = 0, hi = nseg - 1;                    // the thread's segment: the last one starting at or before gs
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (mstart[mid] <= gs) lo = mid;
            else hi = mid - 1;
        }
        const int4 sg = mseg[lo];
        u = sg.x;
        s = gs - mstart[lo] + (sg.z >= 0 ? sbase[sg.z] : 0);
        const int ir = ssub[s];
        const int k = sg.y;
        S = subs + (size_t)k * nsub + ir;
        const float2 cf = csf[s];
        const bool rec = cf.x >= 0.0f;                // (the sign of the float32 table is the float64 test's)
        if (S->active && !(S->wzero & (rec ? 1 : 2))) {
            kr = (int)(s - sbase[ir]) >= S->naz ? 1 : 0;
            const float wsidef = rec ? S->wrecf : S->wappf;
            px = pix_setup(*S, kr, cf, zqf + S->zq_off, S->nzz);
            nzz = S->nzz;
            off = S->zq_off;
            const int e = fix_exp[k];
            const float sgn = (float)sg.w;            // (-1: the base member's deposits taken out, exactly)
            i0 = widx[2 * ir];
            i1 = widx[2 * ir + 1];
            v0 = i0 >= 0 ? sgn * ldexpf(S->fluxscf * wvalf[2 * ir] * wsidef, e) : 0.f;
            v1 = i1 >= 0 ? sgn * ldexpf(S->fluxscf * wvalf[2 * ir + 1] * wsidef, e) : 0.f;
        }
    }
    unsigned long long *out = maps64 + (size_t)u * box.npix * box.nrp;
    int cnt = 0;
    auto push = [&](int g0, int g1, float ws) {
        const unsigned px = (unsigned)(g0 - box.blo0), py = (unsigned)(g1 - box.blo1);
        if (px < (unsigned)box.bx && py < (unsigned)box.by) {
            runq[cnt][tid] = make_uint2(py * (unsigned)box.bx + px, __float_as_uint(ws));
            cnt++;
        }
    };
    auto drain = [&]() {
        const int m = __reduce_max_sync(FULL, cnt);
        for (int j = 0; j < m; j++) {
            if (j < cnt) {
                const uint2 r = runq[j][tid];
                unsigned long long *o = out + (size_t)r.x * box.nrp;
                const float ws = __uint_as_float(r.y);
                if (i0 >= 0) {
                    const long long q = f32_to_ll(v0 * ws);
                    if (q) atomicAdd(o + i0, (unsigned long long)q);
                }
                if (i1 >= 0) {
                    const long long q = f32_to_ll(v1 * ws);
                    if (q) atomicAdd(o + i1, (unsigned long long)q);
                }
            }
        }
        cnt = 0;
    };
    const int nzmax = __reduce_max_sync(FULL, nzz);
    int rg0 = 0, rg1 = 0;
    float rws = 0.f;
    for (int kz = 0; kz < nzmax; kz++) {
        if (kz < nzz) {
            int g0, g1;
            sample_pixel(*S, px, kr, cs + s, nzz, nzz > 1 ? zqf[off + kz] : 0.f, zq + off + kz, g.cdelt0, g.cdelt1,
                         g0, g1);
            const float w = wqf[off + kz];
            if (kz > 0 && g0 == rg0 && g1 == rg1) {
                rws += w;
            } else {
                if (kz > 0) push(rg0, rg1, rws);
                rg0 = g0;
                rg1 = g1;
                rws = w;
            }
        }
        if (__any_sync(FULL, cnt == MAPS_QD)) drain();    // (at most one push per height: room for the next)
    }
    if (nzz > 0) push(rg0, rg1, rws);
    drain();
}

// maps (row u, pixel, ring) int64 units 2^-e -> float32 x scale; a row with a base row holds the difference from
// it (the sum, modulo 2^64, is the row's maps: exact whatever the order of the deposits)
// With a block table (ptab, initialised by k_ptab_init): a row with a base row marks the 8 x 8 pixel blocks
// where its difference is not zero (there its maps are its own; elsewhere they are the base row's, bit for bit).
__global__ void k_maps_to_f32(const long long *__restrict__ in, const int *__restrict__ fix_exp,
                              const int *__restrict__ uidx, const int *__restrict__ ubase, long long per_member,
                              float scale, float *__restrict__ out, int *__restrict__ ptab, int nblk, int nbx,
                              int nrp, int bx) {
    const int u = blockIdx.y;
    const float sc = ldexpf(scale, -fix_exp[uidx[u]]);
    const long long *src = in + (size_t)u * per_member;
    const long long *bas = ubase[u] >= 0 ? in + (size_t)ubase[u] * per_member : nullptr;
    float *dst = out + (size_t)u * per_member;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < per_member;
         i += (long long)gridDim.x * blockDim.x) {
        long long v = src[i];
        if (bas) {
            if (ptab && v != 0) {
                const int q = (int)i / nrp, py = q / bx, px = q - py * bx;      // (per_member < 2^31)
                ptab[(size_t)u * nblk + (py >> 3) * nbx + (px >> 3)] = u;
            }
            v = (long long)((unsigned long long)v + (unsigned long long)bas[i]);
        }
        dst[i] = ll_to_f32(v) * sc;
    }
}

// the block table: a row with a base row starts with the base row's maps everywhere, the others with their own
__global__ void k_ptab_init(int *__restrict__ ptab, const int *__restrict__ ubase, int nu, int nblk) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nu * nblk) return;
    const int u = (int)(i / nblk);
    ptab[i] = ubase[u] >= 0 ? ubase[u] : u;
}

// the solutions of the rows, to the members: x[k] = xu[prof_of[k]], status likewise
__global__ void k_prof_gather(const double *__restrict__ xu, const int *__restrict__ stu,
                              const int *__restrict__ prof_of, int n, double *__restrict__ x, int *__restrict__ st) {
    const int k = blockIdx.x, u = prof_of[k];
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[(size_t)k * n + i] = xu[(size_t)u * n + i];
    if (threadIdx.x == 0) st[k] = stu[u];
}

// ------------------------------------------------------------------------------------------- Gram matrix
// CTA (tile of GRAM_TP used pixels, member k). Entry e < n(n+1)/2: G[i][j] (i <= j, row-major packed upper),
// then h[i]. The tile is staged in shared memory with the range of rings not zero at each pixel, so that each entry
// sums its products over the band of rings that overlap there. Float32 maps: the maps as they are, the maps times
// the pixel weights and the weighted data in float-float (hi + lo, about 46 bits), each product of a float-float and
// a float32 map and its sum carried in float-float with error-free transformations (float32 units, no float64
// pipe), the tile's sum converted to float64 at the end; float64 maps: float64 FMAs; the entries outside the union of the tile's bands (the used pixels come in compact blocks, so
// the union is narrow) are zero without a loop. Partial sums per tile, summed over the tiles in order by
// k_prof_gram_reduce.
// pix == nullptr: the pixels 0 .. npix_used - 1; wpix == nullptr: unit weights.
// s = sh + sl += (xh + xl) b: the product by TwoProduct (the float32 product and its exact error) plus xl b, the
// sum by TwoSum (operations rounded one by one: no contraction)
__device__ __forceinline__ void ff_madd(float &sh, float &sl, float xh, float xl, float b) {
    const float p = __fmul_rn(xh, b);
    float e = __fmaf_rn(xh, b, -p);
    e = __fmaf_rn(xl, b, e);
    const float s = __fadd_rn(sh, p);
    const float z = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, z)), __fsub_rn(p, z));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

__device__ __forceinline__ void out_entry(double *part, int k, int t, int nent, int e, double v) {
    part[((size_t)k * gridDim.x + t) * nent + e] = v;
}

template <class T>
__global__ void __launch_bounds__(256) k_prof_gram(const T *__restrict__ K, ProfBox box, const int *__restrict__ pix,
                                                   const double *__restrict__ wpix, const double *__restrict__ wy,
                                                   int npix_used, const int *__restrict__ ent_i,
                                                   const int *__restrict__ ent_j, int nent,
                                                   double *__restrict__ part, KRows kr) {
    extern __shared__ double gsm[];
    const int n = box.nrp;
    constexpr bool FF = sizeof(T) == 4;
    double *Kd = gsm;                                       // GRAM_TP x n maps
    double *Kw = Kd + GRAM_TP * n;                          // GRAM_TP x n maps x pixel weight
    double *wys = Kw + GRAM_TP * n;                         // GRAM_TP weighted data
    float *Kf = (float *)gsm;                               // (FF: the maps; maps x weight, hi and lo; data, hi, lo)
    float *Kwh = Kf + GRAM_TP * n, *Kwl = Kwh + GRAM_TP * n;
    float *wyh = Kwl + GRAM_TP * n, *wyl = wyh + GRAM_TP;
    int *lo = FF ? (int *)(wyl + GRAM_TP) : (int *)(wys + GRAM_TP), *hi = lo + GRAM_TP;   // rings not zero: lo .. hi
    __shared__ int srow[GRAM_TP];                           // the row whose K holds each pixel
    const int k = blockIdx.y, t = blockIdx.x;
    const int p0 = t * GRAM_TP;
    const int np = min(GRAM_TP, npix_used - p0);
    if (kr.ktab) {
        // a row's convolution left the tiles it shares with row 0 unwritten: K of row 0 there (the same values);
        // a tile of such pixels only has row 0's sums, taken by the reduction
        int own = 0;
        for (int pp = threadIdx.x; pp < np; pp += blockDim.x) {
            const int q = pix ? pix[p0 + pp] : p0 + pp;
            const int py = q / box.bx, px = q - py * box.bx;
            const int r = kr.ktab[(size_t)k * kr.nct + (py >> kr.shy) * kr.ntx + (px >> kr.shx)];
            srow[pp] = r;
            if (r != 0 && kr.blk) {
                // the pixel's K is row 0's when no 8 x 8 block within the beam's reach (one block each way:
                // half-widths of at most 8 pixels) holds the row's own maps
                const int by0 = py >> 3, bx0 = px >> 3;
                bool eq = true;
                for (int dy = -1; dy <= 1 && eq; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int yy = by0 + dy, xx = bx0 + dx;
                        if (yy < 0 || xx < 0 || yy >= kr.nby || xx >= kr.nbx) continue;
                        if (kr.blk[(size_t)k * kr.nby * kr.nbx + yy * kr.nbx + xx] != 0) { eq = false; break; }
                    }
                own |= !eq;
            } else {
                own |= r != 0;
            }
        }
        own = __syncthreads_or(own);
        if (k != 0 && !own) {
            if (threadIdx.x == 0) kr.gflag[(size_t)k * gridDim.x + t] = 1;
            return;
        }
        if (threadIdx.x == 0) kr.gflag[(size_t)k * gridDim.x + t] = 0;
    } else {
        for (int pp = threadIdx.x; pp < np; pp += blockDim.x) srow[pp] = k;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < np * n; i += blockDim.x) {
        const int pp = i / n, r = i - pp * n;
        const long long q = pix ? pix[p0 + pp] : p0 + pp;
        const T kv = K[((size_t)srow[pp] * box.npix + q) * n + r];
        const double w = wpix ? wpix[p0 + pp] : 1.0;
        if constexpr (FF) {
            // kv x w in float-float: kv x wh exactly (TwoProduct), plus kv x wl rounded
            const float wh = (float)w, wl = (float)(w - (double)wh);
            const float ph = __fmul_rn(kv, wh);
            Kf[i] = kv;
            Kwh[i] = ph;
            Kwl[i] = __fadd_rn(__fmaf_rn(kv, wh, -ph), __fmul_rn(kv, wl));
        } else {
            Kd[i] = (double)kv;
            Kw[i] = (double)kv * w;
        }
    }
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        if constexpr (FF) {
            const double y = wy[p0 + i];
            const float yh = (float)y;
            wyh[i] = yh;
            wyl[i] = (float)(y - (double)yh);
        } else {
            wys[i] = wy[p0 + i];
        }
    }
    __syncthreads();
    __shared__ int band[2];                                 // the tile's rings: band[0] .. band[1]
    if (threadIdx.x == 0) { band[0] = n; band[1] = -1; }
    __syncthreads();
    for (int pp = threadIdx.x; pp < np; pp += blockDim.x) {
        int a = n, b = -1;
        for (int r = 0; r < n; r++)
            if (FF ? Kf[pp * n + r] != 0.0f : Kd[pp * n + r] != 0.0) {
                a = min(a, r);
                b = r;
            }
        lo[pp] = a;
        hi[pp] = b;
        if (b >= a) {
            atomicMin(&band[0], a);
            atomicMax(&band[1], b);
        }
    }
    __syncthreads();
    const int blo = band[0], bhi = band[1];
    double *out = part + ((size_t)k * gridDim.x + t) * nent;
    for (int e = threadIdx.x; e < nent; e += blockDim.x) {
        const int i = ent_i[e], j = ent_j[e];
        double acc = 0.0;
        if constexpr (FF) {
            float sh = 0.0f, sl = 0.0f;
            if (j >= 0) {
                if (i >= blo && j <= bhi)
                    for (int pp = 0; pp < np; pp++)
                        if (lo[pp] <= i && j <= hi[pp])
                            ff_madd(sh, sl, Kwh[pp * n + i], Kwl[pp * n + i], Kf[pp * n + j]);
            } else {
                if (i >= blo && i <= bhi)
                    for (int pp = 0; pp < np; pp++)
                        if (lo[pp] <= i && i <= hi[pp]) ff_madd(sh, sl, wyh[pp], wyl[pp], Kf[pp * n + i]);
            }
            out_entry(part, k, t, nent, e, (double)sh + (double)sl);
            continue;
        }
        if (j >= 0) {
            if (i >= blo && j <= bhi)                       // (an entry outside the tile's rings sums to zero)
                for (int pp = 0; pp < np; pp++)
                    if (lo[pp] <= i && j <= hi[pp]) acc = fma(Kw[pp * n + i], Kd[pp * n + j], acc);
        } else {
            if (i >= blo && i <= bhi)
                for (int pp = 0; pp < np; pp++)
                    if (lo[pp] <= i && i <= hi[pp]) acc = fma(wys[pp], Kd[pp * n + i], acc);
        }
        out[e] = acc;
    }
}

__global__ void k_prof_gram_reduce(const double *__restrict__ part, int ntile, int nent, double *__restrict__ gh,
                                   const int *__restrict__ gflag) {
    const int k = blockIdx.y;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nent) return;
    double acc = 0.0;
    for (int t = 0; t < ntile; t++) {
        const bool z = gflag && gflag[(size_t)k * ntile + t];      // (row 0's sums: see k_prof_gram)
        acc += part[((size_t)(z ? 0 : k) * ntile + t) * nent + e];
    }
    gh[(size_t)k * nent + e] = acc;
}

// ------------------------------------------------------------------------------------------- NNLS
// Shared state of one member's solve (one CTA, PS_THREADS threads).
#define PS_THREADS 128

struct Solver {
    int n;
    double *H;      // n x n (the normal matrix of the current system)
    double *F;      // factor of the passive block, n x n
    double *g;      // right-hand side
    double *x, *z, *w;
    int *P, *idx;   // passive flags, passive indices
    int *blocked;
    int *sflag;     // shared scalars
    double *sval;
    double *rs;     // 1 / sqrt of the pivots of the factorisation
};

// Cholesky of H[P,P] into F and solve F F^T z_P = g_P; false if the block is not positive definite.
// 1 / d for d > 0 in float64 without a division: a float32 seed and two Newton steps (within an ulp or two of
// the quotient; float64 division is slow on this part)
__device__ __forceinline__ double rcp_newton(double d) {
    double y = (double)(1.0f / (float)d);
    y = y * (2.0 - d * y);
    y = y * (2.0 - d * y);
    return y;
}

__device__ bool chol_solve(Solver &S, int p) {
    const int tid = threadIdx.x;
    const int n = S.n;
    for (int e = tid; e < p * p; e += blockDim.x) {
        const int a = e / p, b = e - a * p;
        S.F[a * n + b] = S.H[S.idx[a] * n + S.idx[b]];
    }
    if (tid == 0) S.sflag[0] = 1;
    __syncthreads();
    // right-looking elimination on the unscaled columns (one barrier a column): the trailing block takes
    // F[r][c] F[q][c] / F[c][c]; the columns are scaled to the Cholesky factor at the end, L[r][c] = F[r][c] /
    // sqrt(F[c][c]), the diagonal sqrt(F[c][c]) (the same products as the scaled form, in another order)
    for (int c = 0; c < p; c++) {
        const double d = S.F[c * n + c];
        if (!(d > 0.0)) {
            if (tid == 0) S.sflag[0] = 0;
            if (tid == 0) S.F[c * n + c] = 1.0;
            __syncthreads();
            continue;
        }
        const double inv = (d > 1e-30 && d < 1e30) ? rcp_newton(d) : 1.0 / d;
        // the trailing block's lower triangle: rows on the warps, columns on the lanes
        const int nwarp = blockDim.x >> 5, wid = tid >> 5, ln = tid & 31;
        for (int r = c + 1 + wid; r < p; r += nwarp) {
            const double frc = S.F[r * n + c] * inv;
            for (int q = c + 1 + ln; q <= r; q += 32) S.F[r * n + q] -= frc * S.F[q * n + c];
        }
        __syncthreads();
    }
    for (int c = tid; c < p; c += blockDim.x) {
        const double d = S.F[c * n + c];
        S.rs[c] = d > 0.0 ? 1.0 / sqrt(d) : 1.0;
    }
    __syncthreads();
    for (int e = tid; e < p * p; e += blockDim.x) {
        const int r = e / p, c = e - r * p;
        if (r > c) S.F[r * n + c] *= S.rs[c];
    }
    __syncthreads();
    for (int c = tid; c < p; c += blockDim.x) {
        const double d = S.F[c * n + c];
        S.F[c * n + c] = d > 0.0 ? sqrt(d) : 1.0;
    }
    __syncthreads();
    const bool ok = S.sflag[0] != 0;
    // forward then back substitution (one warp; lanes over the dot products)
    if (tid < 32) {
        for (int r = 0; r < p; r++) {
            double acc = 0.0;
            for (int q = tid; q < r; q += 32) acc += S.F[r * n + q] * S.z[q];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
            if (tid == 0) S.z[r] = (S.g[S.idx[r]] - acc) * S.rs[r];   // (F[r][r] = 1 / rs[r])
            __syncwarp();
        }
        for (int r = p - 1; r >= 0; r--) {
            double acc = 0.0;
            for (int q = r + 1 + tid; q < p; q += 32) acc += S.F[q * n + r] * S.z[q];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
            if (tid == 0) S.z[r] = (S.z[r] - acc) * S.rs[r];
            __syncwarp();
        }
    }
    __syncthreads();
    return ok;
}

__device__ int gather_passive(Solver &S) {
    if (threadIdx.x == 0) {
        int p = 0;
        for (int j = 0; j < S.n; j++)
            if (S.P[j]) S.idx[p++] = j;
        S.sflag[1] = p;
    }
    __syncthreads();
    return S.sflag[1];
}

// min 1/2 x^T H x - g^T x subject to x >= 0 (Lawson-Hanson), starting from the passive set in S.P.
// Returns 0, or 1 if a passive block was not positive definite, 2 if the iteration limit was reached.
__device__ int nnls(Solver &S) {
    const int n = S.n, tid = threadIdx.x;
    int status = 0;
    for (int j = tid; j < n; j += blockDim.x) {
        S.x[j] = 0.0;
        S.blocked[j] = 0;
    }
    __syncthreads();
    // warm start: drop the non-positive components until the passive least squares is positive
    for (int it = 0; it <= n; it++) {
        const int p = gather_passive(S);
        if (p == 0) break;
        if (!chol_solve(S, p)) {
            status = 1;
            for (int j = tid; j < n; j += blockDim.x) S.P[j] = 0;
            __syncthreads();
            break;
        }
        if (tid == 0) {
            int bad = 0;
            for (int a = 0; a < p; a++)
                if (!(S.z[a] > 0.0)) {
                    S.P[S.idx[a]] = 0;
                    bad = 1;
                }
            if (!bad)
                for (int a = 0; a < p; a++) S.x[S.idx[a]] = S.z[a];
            S.sflag[2] = bad;
        }
        __syncthreads();
        if (!S.sflag[2]) break;
    }
    double gmax = 0.0;
    for (int j = 0; j < n; j++) gmax = fmax(gmax, fabs(S.g[j]));
    const double tol = 1e-12 * (gmax > 0 ? gmax : 1.0);
    for (int outer = 0; outer < 3 * n; outer++) {
        // w = g - H x
        for (int j = tid; j < n; j += blockDim.x) {
            double acc = S.g[j];
            for (int q = 0; q < n; q++) acc -= S.H[j * n + q] * S.x[q];
            S.w[j] = acc;
        }
        __syncthreads();
        if (tid == 0) {
            int t = -1;
            double best = tol;
            for (int j = 0; j < n; j++)
                if (!S.P[j] && !S.blocked[j] && S.w[j] > best) {
                    best = S.w[j];
                    t = j;
                }
            S.sflag[3] = t;
            if (t >= 0) S.P[t] = 1;
        }
        __syncthreads();
        const int t = S.sflag[3];
        if (t < 0) return status;
        for (int inner = 0; inner < 3 * n; inner++) {
            const int p = gather_passive(S);
            if (!chol_solve(S, p)) {
                status |= 1;
                if (tid == 0) {
                    S.P[t] = 0;
                    S.blocked[t] = 1;
                }
                __syncthreads();
                break;
            }
            if (tid == 0) {
                int allpos = 1, tpos = 1;
                for (int a = 0; a < p; a++)
                    if (!(S.z[a] > 0.0)) {
                        allpos = 0;
                        if (S.idx[a] == t) tpos = 0;
                    }
                if (allpos) {
                    for (int j = 0; j < n; j++) S.x[j] = 0.0;
                    for (int a = 0; a < p; a++) S.x[S.idx[a]] = S.z[a];
                    for (int j = 0; j < n; j++) S.blocked[j] = 0;
                    S.sflag[4] = 1;
                } else if (inner == 0 && !tpos) {
                    // the entering variable is not positive in the least squares: numerically at its bound
                    S.P[t] = 0;
                    S.blocked[t] = 1;
                    S.sflag[4] = 1;
                } else {
                    double alpha = 2.0;
                    for (int a = 0; a < p; a++)
                        if (!(S.z[a] > 0.0)) {
                            const int j = S.idx[a];
                            const double den = S.x[j] - S.z[a];
                            const double al = den > 0.0 ? S.x[j] / den : 0.0;
                            alpha = fmin(alpha, al);
                        }
                    for (int a = 0; a < p; a++) {
                        const int j = S.idx[a];
                        S.x[j] += alpha * (S.z[a] - S.x[j]);
                        if (!(S.x[j] > 0.0)) {
                            S.x[j] = 0.0;
                            S.P[j] = 0;
                        }
                    }
                    S.sflag[4] = 0;
                }
            }
            __syncthreads();
            if (S.sflag[4]) break;
        }
    }
    return status | 2;
}

// H = G + sum_i wi^2 L_i^T L_i (L_i: the 3 weights of second difference i at columns lc[i][0..2])
__device__ void build_H(Solver &S, const double *G, const int *lc, const double *lv, const double *wr, int nrow) {
    // H = G + sum over the prior rows i of w_i^2 lv_i lv_i^T (columns lc_i); each entry takes its terms in the
    // order of the rows (i, then a, then b), a thread an entry
    const int n = S.n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int j = e / n, q = e - j * n;
        double h = G[e];
        for (int i = 0; i < nrow; i++) {
            const int c0 = lc[3 * i], c1 = lc[3 * i + 1], c2 = lc[3 * i + 2];
            if ((c0 != j && c1 != j && c2 != j) || (c0 != q && c1 != q && c2 != q)) continue;
            const double w2 = wr[i] * wr[i];
            for (int a = 0; a < 3; a++) {
                if (lc[3 * i + a] != j) continue;
                for (int b = 0; b < 3; b++)
                    if (lc[3 * i + b] == q) h += w2 * lv[3 * i + a] * lv[3 * i + b];
            }
        }
        S.H[e] = h;
    }
    __syncthreads();
}

// One CTA per member: solve_profile (bbarolo/profile.py:91-138) on the normal equations gh (packed G, h).
__global__ void __launch_bounds__(PS_THREADS) k_prof_solve(const double *__restrict__ gh, ProfConst pc,
                                                           const int *__restrict__ lc, const double *__restrict__ lv,
                                                           const int *__restrict__ ord,
                                                           const unsigned char *__restrict__ near,
                                                           const int *__restrict__ p0, double *__restrict__ xout,
                                                           int *__restrict__ pout, int *__restrict__ status) {
    extern __shared__ double psm[];
    const int n = pc.n, k = blockIdx.x, tid = threadIdx.x;
    Solver S;
    S.n = n;
    double *G = psm;
    S.H = G + n * n;
    S.F = S.H + n * n;
    S.g = S.F + n * n;
    S.x = S.g + n;
    S.z = S.x + n;
    S.w = S.z + n;
    double *wr = S.w + n;                       // n weights of the prior rows
    double *x0 = wr + n;
    S.rs = x0 + n;
    S.sval = S.rs + n;
    S.P = (int *)(S.sval + 8);
    S.idx = S.P + n;
    S.blocked = S.idx + n;
    S.sflag = S.blocked + n;
    const int nent = n * (n + 1) / 2;
    const double *ghk = gh + (size_t)k * (nent + n);
    for (int e = tid; e < nent; e += blockDim.x) {
        // packed upper row-major: row i holds (i, i..n-1)
        int i = 0, rem = e;
        while (rem >= n - i) {
            rem -= n - i;
            i++;
        }
        const int j = i + rem;
        G[i * n + j] = ghk[e];
        G[j * n + i] = ghk[e];
    }
    for (int j = tid; j < n; j += blockDim.x) {
        S.g[j] = ghk[nent + j];
        S.P[j] = p0[j];
    }
    __syncthreads();
    int st = 0;
    const int nrow = n - 2;
    if (!(pc.smooth != 0.0) || n < 3) {
        build_H(S, G, lc, lv, wr, 0);
        st = nnls(S);
    } else {
        double traa = 0.0;
        for (int j = 0; j < n; j++) traa += G[j * n + j];
        const double srel = sqrt(0.1 * traa / fmax(pc.norm, 1e-300));
        for (int i = tid; i < nrow; i += blockDim.x) wr[i] = srel;
        __syncthreads();
        build_H(S, G, lc, lv, wr, nrow);
        st = nnls(S);
        for (int j = tid; j < n; j += blockDim.x) x0[j] = S.x[j];
        __syncthreads();
        // the reduced chi2 of the first solution, sum (b - A x0)^2 = b.b - 2 x0.h + x0^T G x0: the terms of each a
        // by a thread (S.w), then summed in the order of a by thread 0
        for (int a = tid; a < n; a += blockDim.x) {
            double r = 0.0;
            for (int b = 0; b < n; b++) r += G[a * n + b] * x0[b];
            S.w[a] = x0[a] * r;
        }
        __syncthreads();
        if (tid == 0) {
            double xm = 0.0;
            for (int j = 0; j < n - 1; j++) xm += x0[j];
            xm /= (double)(n - 1);
            S.sval[0] = xm;
            double xh = 0.0, xgx = 0.0;
            for (int a = 0; a < n; a++) {
                xh += x0[a] * S.g[a];
                xgx += S.w[a];
            }
            const double chi2 = (pc.bb - 2.0 * xh + xgx) / fmax((double)(pc.m - n), 1.0);
            const double corr = fmax(pc.corr, 1.0) * fmax(chi2, 1.0);
            S.sval[1] = sqrt(corr) * pc.d * pc.d / pc.smooth;
            S.sval[2] = sqrt(pc.floor_) * srel;
        }
        __syncthreads();
        if (S.sval[0] > 0) {
            const double xm = S.sval[0];
            for (int i = tid; i < nrow; i += blockDim.x) {
                const double xc = fmax(x0[ord[i + 1]], 0.1 * xm);
                double wi = S.sval[1] / xc;
                wi = fmax(wi, S.sval[2]);
                if (near[i]) wi = srel;
                wr[i] = wi;
            }
        }
        __syncthreads();
        if (S.sval[0] > 0) {
            for (int j = tid; j < n; j += blockDim.x) S.P[j] = x0[j] > 0.0;
            __syncthreads();
            build_H(S, G, lc, lv, wr, nrow);
            st |= nnls(S);
        }
    }
    for (int j = tid; j < n; j += blockDim.x) {
        xout[(size_t)k * n + j] = S.x[j];
        pout[(size_t)k * n + j] = S.x[j] > 0.0;
    }
    if (tid == 0) status[k] = st;
}

// ------------------------------------------------------------------------------------------- model densities
// One CTA per member: dens of the model's sub-rings from the ring densities x (the ring weights), then the
// dens-dependent fields of the MC sub-ring constants (bbarolo/galmod.py:107-122) and the fixed-point exponent.
// Flags ERR_PROFILE_LAYOUT in err when a density changes the cloud layout (a sub-ring switched off, or a
// cloud count above the 10-per-pixel floor).
__global__ void k_mc_dens(GridDev g, SubMC *__restrict__ sub, int nsub, MemberDev *__restrict__ mem,
                          const double *__restrict__ x, int nx, const int *__restrict__ widx,
                          const double *__restrict__ wval, const double *__restrict__ rap, int *err) {
    __shared__ double red[256];
    const int k = blockIdx.x, tid = threadIdx.x;
    const double *xk = x + (size_t)k * nx;
    double bound = 0.0;
    for (int ir = tid; ir < nsub; ir += blockDim.x) {
        SubMC &S = sub[(size_t)k * nsub + ir];
        double dens = 0.0;
        for (int m = 0; m < 2; m++) {
            const int r = widx[2 * ir + m];
            if (r >= 0) dens += wval[2 * ir + m] * xk[r];
        }
        const double ra = rap[ir];
        const bool act = dens != 0.0;
        int bad = act != (S.active != 0);
        if (act && S.active) {
            const double dp = g.cmode == 1 ? dens : (g.cmode == 2 ? __dmul_rn(dens, dens) : pow(dens, (double)g.cmode));
            const double cd = __dmul_rn(g.cdens, dp);
            long long nc = lround_ref(__dmul_rn(cd, ra));
            if ((double)lround_ref(__ddiv_rn((double)nc, ra)) < 10.) nc = lround_ref(__dmul_rn(10.0, ra));
            if (nc != S.nc) bad = 1;
            const double fl = (double)(float)__ddiv_rn(__dmul_rn(__dmul_rn(dens, ra), g.pixarea),
                                                       (double)((long long)S.nc * S.nv));
            const double wmax = fmax(fabs(S.wrec), fabs(S.wapp));
            for (int nl = 0; nl < g.nlines && nl < BBGPU_MAXL; nl++) {
                S.valrel[nl] = __dmul_rn(g.relint[nl], fl);
                bound += (double)S.nc * (double)S.nv * fabs(S.valrel[nl]) * wmax;
            }
        }
        if (bad) atomicOr(err, ERR_PROFILE_LAYOUT);
    }
    red[tid] = bound;
    __syncthreads();
    for (int d = blockDim.x / 2; d > 0; d >>= 1) {
        if (tid < d) red[tid] += red[tid + d];
        __syncthreads();
    }
    const double B = red[0];
    const int e = B > 0 ? (int)floor(62.0 - log2(B)) : 0;
    const double Q = ldexp(1.0, e);
    for (int ir = tid; ir < nsub; ir += blockDim.x) {
        SubMC &S = sub[(size_t)k * nsub + ir];
        if (!S.active) continue;
        for (int nl = 0; nl < g.nlines && nl < BBGPU_MAXL; nl++) {
            S.fix[0][nl] = llrint(S.valrel[nl] * S.wrec * Q);
            S.fix[1][nl] = llrint(S.valrel[nl] * S.wapp * Q);
        }
    }
    if (tid == 0) mem[k].fix_exp = e;
}

// The ANALYTIC counterpart of k_mc_dens (one CTA per member): fluxsc = dens x ring area / (2 naz)
// (bbarolo/galmod.py:367), the line amplitudes relint x fluxsc, and the member's fixed-point exponent from the
// bound of its deposits (as the host's). A sub-ring at zero density deposits nothing; one that the host set up
// as empty (no vertical grid) but whose density is not zero is an error.
__global__ void k_an_dens(GridDev g, AnSub *__restrict__ sub, int nsub, MemberDev *__restrict__ mem,
                          const double *__restrict__ x, int nx, const int *__restrict__ widx,
                          const double *__restrict__ wval, const double *__restrict__ rap, double per, int *err) {
    __shared__ double red[256];
    const int k = blockIdx.x, tid = threadIdx.x;
    const double *xk = x + (size_t)k * nx;
    double bound = 0.0;
    for (int ir = tid; ir < nsub; ir += blockDim.x) {
        AnSub &S = sub[(size_t)k * nsub + ir];
        double dens = 0.0;
        for (int m = 0; m < 2; m++) {
            const int r = widx[2 * ir + m];
            if (r >= 0) dens += wval[2 * ir + m] * xk[r];
        }
        if (!S.active) {
            if (dens != 0.0) atomicOr(err, ERR_PROFILE_LAYOUT);
            continue;
        }
        if (dens == 0.0) {
            S.active = 0;
            continue;
        }
        const double fl = __ddiv_rn(__dmul_rn(__dmul_rn(dens, rap[ir]), g.pixarea), (double)((long long)S.naz * 2));
        S.fluxsc = fl;
        S.fluxscf = (float)fl;
        for (int nl = 0; nl < g.nlines && nl < BBGPU_MAXL; nl++) S.a[nl] = __dmul_rn(g.relint[nl], fl);
        S.af = (float)S.a[0];
        bound += fabs(fl) * fmax(fabs(S.wrec), fabs(S.wapp)) * per * (double)((long long)S.naz * 2);
    }
    red[tid] = bound;
    __syncthreads();
    for (int d = blockDim.x / 2; d > 0; d >>= 1) {
        if (tid < d) red[tid] += red[tid + d];
        __syncthreads();
    }
    if (tid == 0) {
        const double B = red[0];
        int e = 0;
        if (B > 0.0) {
            int ex = 0;
            frexp(B * 1.01, &ex);                   // B x 1.01 < 2^ex
            e = min(62 - ex, 1000);
        }
        mem[k].fix_exp = e;
    }
}

}  // namespace

void launch_an_dens(cudaStream_t s, const GridDev &g, AnSub *sub, int nsub, MemberDev *mem, int nb, const double *x,
                    int nx, const int *widx, const double *wval, const double *rap, double per, int *err) {
    if (nb == 0) return;
    k_an_dens<<<nb, 256, 0, s>>>(g, sub, nsub, mem, x, nx, widx, wval, rap, per, err);
}

void launch_an_maps_fast(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase,
                         const int *ssub, const double *cs, const float *csf, const long long *mstart,
                         const int *mseg, int nseg, long long ntot, const double *zq, const float *zqf,
                         const float *wqf, const int *widx, const float *wvalf, const ProfBox &box,
                         const int *fix_exp, long long *maps64) {
    if (ntot == 0 || nseg == 0) return;
    k_an_maps_fast<<<(unsigned)((ntot + MAPS_TB - 1) / MAPS_TB), MAPS_TB, 0, s>>>(
        g, subs, nsub, sbase, ssub, (const double2 *)cs, (const float2 *)csf, mstart, (const int4 *)mseg, nseg, ntot,
        zq, zqf, wqf, widx, wvalf, box, fix_exp, (unsigned long long *)maps64);
}

void launch_maps_to_f32(cudaStream_t s, const long long *in, const int *fix_exp, const int *uidx, const int *ubase,
                        int nu, long long per_member, float scale, float *out, int *ptab, const ProfBox &box) {
    if (nu == 0 || per_member == 0) return;
    const int nbx = (box.bx + 7) / 8, nblk = nbx * ((box.by + 7) / 8);
    if (ptab) {
        const long long n = (long long)nu * nblk;
        k_ptab_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ptab, ubase, nu, nblk);
    }
    dim3 grid((unsigned)std::min<long long>((per_member + 255) / 256, 1024), nu);
    k_maps_to_f32<<<grid, 256, 0, s>>>(in, fix_exp, uidx, ubase, per_member, scale, out, ptab, nblk, nbx, box.nrp,
                                       box.bx);
}

void launch_prof_gather(cudaStream_t s, const double *xu, const int *stu, const int *prof_of, int nb, int n, double *x,
                        int *st) {
    if (nb == 0) return;
    k_prof_gather<<<nb, 64, 0, s>>>(xu, stu, prof_of, n, x, st);
}

int prof_gram_tiles(int npix_used) { return (npix_used + GRAM_TP - 1) / GRAM_TP; }

template <class T>
static void prof_gram(cudaStream_t s, const T *K, const ProfBox &box, const int *pix, const double *wpix,
                      const double *wy, int npix_used, const int *ent_i, const int *ent_j, int nent, int nb,
                      double *part, double *gh, KRows kr) {
    const int nt = prof_gram_tiles(npix_used);
    if (nb == 0 || nt == 0) return;
    const size_t smem = sizeof(T) == 4
                            ? (size_t)(3 * GRAM_TP * box.nrp + 2 * GRAM_TP) * sizeof(float) + 2 * GRAM_TP * sizeof(int)
                            : (size_t)(2 * GRAM_TP * box.nrp + GRAM_TP) * sizeof(double) + 2 * GRAM_TP * sizeof(int);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_prof_gram<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_prof_gram<T><<<dim3(nt, nb), 256, smem, s>>>(K, box, pix, wpix, wy, npix_used, ent_i, ent_j, nent, part, kr);
    k_prof_gram_reduce<<<dim3((nent + 127) / 128, nb), 128, 0, s>>>(part, nt, nent, gh, kr.ktab ? kr.gflag : nullptr);
}

void launch_prof_gram(cudaStream_t s, const float *K, const ProfBox &box, const int *pix, const double *wpix,
                      const double *wy, int npix_used, const int *ent_i, const int *ent_j, int nent, int nb,
                      double *part, double *gh, KRows kr) {
    prof_gram<float>(s, K, box, pix, wpix, wy, npix_used, ent_i, ent_j, nent, nb, part, gh, kr);
}

void launch_prof_gram64(cudaStream_t s, const double *A, const ProfBox &box, const double *b, int m, const int *ent_i,
                        const int *ent_j, int nent, double *part, double *gh) {
    prof_gram<double>(s, A, box, nullptr, nullptr, b, m, ent_i, ent_j, nent, 1, part, gh, KRows{});
}

size_t prof_solve_smem(int n) { return (size_t)(3 * n * n + 7 * n + 8) * sizeof(double) + (size_t)(4 * n + 8) * sizeof(int); }

void launch_prof_solve(cudaStream_t s, const double *gh, const ProfConst &pc, const int *lc, const double *lv,
                       const int *ord, const unsigned char *near, const int *p0, int nb, double *x, int *pout,
                       int *status) {
    if (nb == 0) return;
    const size_t smem = prof_solve_smem(pc.n);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_prof_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_prof_solve<<<nb, PS_THREADS, smem, s>>>(gh, pc, lc, lv, ord, near, p0, x, pout, status);
}

void launch_mc_dens(cudaStream_t s, const GridDev &g, SubMC *sub, int nsub, MemberDev *mem, int nb, const double *x,
                    int nx, const int *widx, const double *wval, const double *rap, int *err) {
    if (nb == 0) return;
    k_mc_dens<<<nb, 256, 0, s>>>(g, sub, nsub, mem, x, nx, widx, wval, rap, err);
}
