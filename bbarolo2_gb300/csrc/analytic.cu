// The ANALYTIC GALMOD deposit and the ring maps on the device (the reference's _galmod_analytic and
// _ring_maps_analytic, bbarolo/galmod.py:326-536).
//
// One warp per azimuthal sample (sub-ring, radial sample, azimuth). The warp computes the pixels of the
// sample's vertical samples (lanes over heights), merges consecutive heights that fall in the same pixel
// (lane 0, in order, as the reference), and deposits each merged run: for a model, the channel-integrated
// line profile (lanes over channels, computed once per sample and line from the tabulated normal CDF), for
// ring maps the run's weight. All arithmetic that decides an index or a value is the reference's float64,
// each operation rounded once in its order (no contraction), so pixels and channels are bit-exact. The sums
// are in 64-bit fixed point (units 2^-e, e per member from a bound on its total flux): integer atomics, exact
// and independent of the order of the deposits, so the model is deterministic; it differs from the
// reference's running float64 sum by rounding only.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "anpix.cuh"
#include "devmath.cuh"
#include "kernels.h"

#define PHI_N 6146
#define AN_WPB 8            // warps per CTA
#define FULL 0xffffffffu

namespace {

// bbarolo/galmod.py:183-191: the normal CDF at t from the table (512 entries per unit from -6)
__device__ __forceinline__ double phi_interp(double t, const double *__restrict__ tab) {
    const double x = __dmul_rn(__dadd_rn(t, 6.0), 512.0);
    if (x <= 0.0) return 0.0;
    if (!(x < (double)(PHI_N - 1))) return 1.0;
    const int k = (int)x;
    const double t0 = tab[k], t1 = tab[k + 1];
    return __dadd_rn(t0, __dmul_rn(__dsub_rn(x, (double)k), __dsub_rn(t1, t0)));
}

// bbarolo/galmod.py:400-406: the pixel of the vertical sample at height z (z = 0 for a thin layer)
__device__ __forceinline__ void an_pixel(const AnSub &S, double cdelt0, double cdelt1, double xs, double xc,
                                         double yb, double z, int &g0, int &g1) {
    const double y = __dsub_rn(yb, __dmul_rn(z, S.sinc));
    g0 = clamp_pix(lround_ref(__dadd_rn(S.xpos, __ddiv_rn(__dsub_rn(xs, __dmul_rn(y, S.cpa)), cdelt0))));
    g1 = clamp_pix(lround_ref(__dadd_rn(S.ypos, __ddiv_rn(__dadd_rn(xc, __dmul_rn(y, S.spa)), cdelt1))));
}

// bbarolo/galmod.py:194-214: the CDF at the channel edges k0 .. k0 + nk of the line at velocity v (lanes over
// edges) into pe; the profile of channel k0 + j is |pe[j + 1] - pe[j]| * cd2i[k0 + j].
__device__ __forceinline__ void an_profile(const GridDev &g, int nl, double v, const AnSub &S,
                                           const double *__restrict__ vedges, const double *__restrict__ ptab,
                                           double *pe, int &k0, int &nk) {
    const int lane = threadIdx.x & 31;
    const long long kc = lround_ref(velgrid_exact(v, g, nl));
    long long a0 = kc - S.K, a1 = kc + S.K + 1;
    if (a0 < 0) a0 = 0;
    if (a1 > g.nz) a1 = g.nz;
    if (a1 <= a0) {
        k0 = 0;
        nk = 0;
        return;
    }
    k0 = (int)a0;
    nk = (int)(a1 - a0);
    const double *ve = vedges + (size_t)nl * (g.nz + 1) + k0;
    for (int j = lane; j <= nk; j += 32) pe[j] = phi_interp(__dmul_rn(__dsub_rn(ve[j], v), S.inv), ptab);
    __syncwarp();
}

// The channels of a profile times aw, added in fixed point to the spectrum o (whole warp).
__device__ __forceinline__ void an_add(unsigned long long *o, const double *pe, const double *__restrict__ cd2i,
                                       int k0, int nk, double aw, double fscale) {
    const int lane = threadIdx.x & 31;
    for (int j = lane; j < nk; j += 32) {
        double f = __dsub_rn(pe[j + 1], pe[j]);
        f = f >= 0 ? f : -f;
        const double t = __dmul_rn(aw, __dmul_rn(f, cd2i[k0 + j]));
        const long long q = __double2ll_rn(__dmul_rn(t, fscale));
        if (q) atomicAdd(o + k0 + j, (unsigned long long)q);
    }
}

// The runs of consecutive vertical samples in one pixel (bbarolo/galmod.py:412-421 and :518-524), in order:
// emit(g0, g1, ws) is called by the whole warp for each run (warp-uniform arguments).
template <class F>
__device__ __forceinline__ void an_runs(const AnSub &S, const double *__restrict__ zq, const double *__restrict__ wq,
                                        double cdelt0, double cdelt1, double xs, double xc, double yb, int *sgx,
                                        int *sgy, int *rg0, int *rg1, double *rws, F emit) {
    const int lane = threadIdx.x & 31;
    const int nzz = S.nzz;
    int og0 = 0, og1 = 0;
    double ows = 0.0;
    bool open = false;
    for (int base = 0; base < nzz; base += 32) {
        const int cnt = min(32, nzz - base);
        if (lane < cnt) {
            const double z = nzz > 1 ? __dmul_rn(zq[base + lane], S.z0) : 0.0;
            an_pixel(S, cdelt0, cdelt1, xs, xc, yb, z, sgx[lane], sgy[lane]);
        }
        __syncwarp();
        int nr = 0;
        if (lane == 0) {
            for (int t = 0; t < cnt; t++) {
                const int a = sgx[t], b = sgy[t];
                const double w = wq[base + t];
                if (open && a == og0 && b == og1) {
                    ows = __dadd_rn(ows, w);
                } else {
                    if (open) {
                        rg0[nr] = og0;
                        rg1[nr] = og1;
                        rws[nr] = ows;
                        nr++;
                    }
                    og0 = a;
                    og1 = b;
                    ows = w;
                    open = true;
                }
            }
        }
        nr = __shfl_sync(FULL, nr, 0);
        __syncwarp();
        for (int r = 0; r < nr; r++) emit(rg0[r], rg1[r], rws[r]);
        __syncwarp();
    }
    if (lane == 0) {
        rg0[0] = og0;
        rg1[0] = og1;
        rws[0] = ows;
    }
    __syncwarp();
    emit(rg0[0], rg1[0], rws[0]);
    __syncwarp();
}

struct AnWarp {
    int sgx[32], sgy[32], rg0[33], rg1[33];
    double rws[33];
    int k0[BBGPU_MAXL], nk[BBGPU_MAXL];
};

// The (member, sample) of warp gs of a batch, by segments of warps: segment i (warps astart[i] .. astart[i + 1])
// is aseg[i] = (member whose model takes the deposits, member whose constants make them, sub-ring (-1: every
// sample of the table), sign of the deposits); s is the sample in the table.
struct AnSeg {
    int k, src, sign;
    long long s;
};
__device__ __forceinline__ bool an_seg(long long gs, const long long *__restrict__ astart,
                                       const int4 *__restrict__ aseg, int nseg, long long ntot,
                                       const int *__restrict__ sbase, AnSeg &o) {
    if (gs >= ntot) return false;
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (astart[mid] <= gs) lo = mid;
        else hi = mid - 1;
    }
    const int4 sg = aseg[lo];
    o.k = sg.x;
    o.src = sg.y;
    o.sign = sg.w;
    o.s = gs - astart[lo] + (sg.z >= 0 ? sbase[sg.z] : 0);
    return true;
}

// The sample s of member src: sub-ring S, cos/sin of its azimuth; false if nothing to deposit.
__device__ __forceinline__ bool an_sample(long long s, int src, int nsub, const AnSub *__restrict__ subs,
                                          const int *__restrict__ sbase, const int *__restrict__ ssub,
                                          const double2 *__restrict__ cs, const AnSub *&S, double &caz,
                                          double &saz, double &R) {
    const int ir = ssub[s];
    S = subs + (size_t)src * nsub + ir;
    if (!S->active) return false;
    const int local = (int)(s - sbase[ir]);
    const double2 c = cs[s];
    caz = c.x;
    saz = c.y;
    R = S->R[local >= S->naz ? 1 : 0];
    return true;
}

// Models: out64 (per member: box (by, bx, nz), stride mstride) += fixed-point deposits.
__global__ void __launch_bounds__(AN_WPB * 32) k_an_model(GridDev g, const AnSub *__restrict__ subs, int nsub,
                                                          const int *__restrict__ sbase, const int *__restrict__ ssub,
                                                          const double2 *__restrict__ cs,
                                                          const long long *__restrict__ astart,
                                                          const int4 *__restrict__ aseg, int nseg, long long ntot,
                                                          const double *__restrict__ zq, const double *__restrict__ wq,
                                                          const double *__restrict__ vedges,
                                                          const double *__restrict__ cd2i,
                                                          const double *__restrict__ ptab,
                                                          const MemberDev *__restrict__ mem,
                                                          unsigned long long *__restrict__ out64, long long mstride,
                                                          int skip_fast) {
    extern __shared__ double an_smem[];
    __shared__ AnWarp wsm[AN_WPB];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gs = (long long)blockIdx.x * AN_WPB + w;
    AnSeg sg;
    if (!an_seg(gs, astart, aseg, nseg, ntot, sbase, sg)) return;
    const int k = sg.k;
    const AnSub *Sp;
    double caz, saz, R;
    if (!an_sample(sg.s, sg.src, nsub, subs, sbase, ssub, cs, Sp, caz, saz, R)) return;
    const AnSub &S = *Sp;
    if (skip_fast && S.anfast) return;                 // (k_an_model_fast's samples)
    const double wside = caz >= 0.0 ? S.wrec : S.wapp;
    if (wside == 0.0) return;
    const MemberDev &M = mem[k];
    const int nz = g.nz, nl_n = g.nlines;
    double *pe = an_smem + (size_t)w * nl_n * (nz + 2);
    AnWarp &W = wsm[w];
    // (a negative unit: the deposits of member 0's constants taken out of a difference, rounded symmetrically)
    const double fscale = sg.sign < 0 ? -ldexp(1.0, M.fix_exp) : ldexp(1.0, M.fix_exp);
    unsigned long long *o64 = out64 + (size_t)k * mstride;
    const double x = __dmul_rn(R, caz);
    const double yb = __dmul_rn(__dmul_rn(R, saz), S.cinc);
    const double xs = __dmul_rn(x, S.spa), xc = __dmul_rn(x, S.cpa);
    // bbarolo/galmod.py:407
    const double vplane = __dadd_rn(__dadd_rn(S.vsys, __dmul_rn(__dadd_rn(__dmul_rn(S.vrot, caz), __dmul_rn(S.vrad, saz)),
                                                                S.sinc)),
                                    __dmul_rn(S.vvert, S.cinc));
    const double *zqs = zq + S.zq_off, *wqs = wq + S.zq_off;
    if (!S.zdep) {
        bool ready = false;
        auto emit = [&](int g0, int g1, double ws) {
            if (g0 < M.blo0 || g0 >= M.bhi0 || g1 < M.blo1 || g1 >= M.bhi1) return;
            if (!ready) {
                for (int nl = 0; nl < nl_n; nl++) {
                    int k0, nk;
                    an_profile(g, nl, vplane, S, vedges, ptab, pe + (size_t)nl * (nz + 2), k0, nk);
                    W.k0[nl] = k0;
                    W.nk[nl] = nk;
                }
                ready = true;
            }
            unsigned long long *o = o64 + ((size_t)(g1 - M.blo1) * M.bx + (size_t)(g0 - M.blo0)) * nz;
            for (int nl = 0; nl < nl_n; nl++) {
                if (W.nk[nl] == 0) continue;
                const double aw = __dmul_rn(__dmul_rn(S.a[nl], wside), ws);
                an_add(o, pe + (size_t)nl * (nz + 2), cd2i, W.k0[nl], W.nk[nl], aw, fscale);
            }
            __syncwarp();
        };
        an_runs(S, zqs, wqs, g.cdelt0, g.cdelt1, xs, xc, yb, W.sgx, W.sgy, W.rg0, W.rg1, W.rws, emit);
        return;
    }
    // bbarolo/galmod.py:430-463: the velocity depends on |z|; the samples at +z and -z share a profile
    const int nzz = S.nzz;
    for (int kz = 0; kz < (nzz + 1) / 2; kz++) {
        const int kz2 = nzz - 1 - kz;
        int ga = 0, gb = 0;
        if (lane < 2) {
            const double z = __dmul_rn(zqs[lane == 0 ? kz : kz2], S.z0);
            an_pixel(S, g.cdelt0, g.cdelt1, xs, xc, yb, z, ga, gb);
        }
        const int gx1 = __shfl_sync(FULL, ga, 0), gy1 = __shfl_sync(FULL, gb, 0);
        const int gx2 = __shfl_sync(FULL, ga, 1), gy2 = __shfl_sync(FULL, gb, 1);
        const bool in1 = !(gx1 < M.blo0 || gx1 >= M.bhi0 || gy1 < M.blo1 || gy1 >= M.bhi1);
        const bool in2 = kz2 != kz && !(gx2 < M.blo0 || gx2 >= M.bhi0 || gy2 < M.blo1 || gy2 >= M.bhi1);
        if (!(in1 || in2)) continue;
        const double az_ = fabs(__dmul_rn(zqs[kz], S.z0));
        double v = vplane;
        if (az_ > S.zcyl) {
            const double lv = __dsub_rn(S.vrot, __dmul_rn(S.dvdz, __dsub_rn(az_, S.zcyl)));
            const double vr = S.vrot >= 0.0 ? ((0.0 > lv) ? 0.0 : lv) : ((0.0 < lv) ? 0.0 : lv);
            v = __dadd_rn(__dadd_rn(S.vsys, __dmul_rn(__dadd_rn(__dmul_rn(vr, caz), __dmul_rn(S.vrad, saz)), S.sinc)),
                          __dmul_rn(S.vvert, S.cinc));
        }
        for (int nl = 0; nl < nl_n; nl++) {
            int k0, nk;
            an_profile(g, nl, v, S, vedges, ptab, pe, k0, nk);
            if (nk == 0) continue;
            const double a = __dmul_rn(S.a[nl], wside);
            if (in1 && in2 && gx1 == gx2 && gy1 == gy2) {
                unsigned long long *o = o64 + ((size_t)(gy1 - M.blo1) * M.bx + (size_t)(gx1 - M.blo0)) * nz;
                an_add(o, pe, cd2i, k0, nk, __dmul_rn(a, __dadd_rn(wqs[kz], wqs[kz2])), fscale);
            } else {
                if (in1) {
                    unsigned long long *o = o64 + ((size_t)(gy1 - M.blo1) * M.bx + (size_t)(gx1 - M.blo0)) * nz;
                    an_add(o, pe, cd2i, k0, nk, __dmul_rn(a, wqs[kz]), fscale);
                }
                if (in2) {
                    unsigned long long *o = o64 + ((size_t)(gy2 - M.blo1) * M.bx + (size_t)(gx2 - M.blo0)) * nz;
                    an_add(o, pe, cd2i, k0, nk, __dmul_rn(a, wqs[kz2]), fscale);
                }
            }
            __syncwarp();
        }
    }
}

// ------------------------------------------------------------------------------ the model's float32 path
// Sub-rings with one line on a linear channel map and a velocity independent of the height (anfast): one warp
// per (member, azimuth sample).
//   pixels  lanes over heights, float32 with a rounding bound and exact fallbacks (sample_pixel), the reference's
//           pixel of every height;
//   runs    consecutive heights in one pixel (a ballot of the run starts), their weights by a segmented scan
//           (float32), a run crossing a pass of 32 heights carried to the next pass;
//   line    computed at the first run in the box: the velocity and its channel in float-float (the reference's
//           float64 _velgrid within 1e-6 of a channel boundary), the centre channel kc exact, then the
//           channel-integrated profile over kc - K .. kc + K in float32: the edges relative to a reference
//           velocity in float-float (so that (edge - v) / sig keeps ~1e-7), the normal CDF from the reference's
//           table (float32 copy, linear interpolation as _phi);
//   deposit lanes over channels, 64-bit fixed-point atomics of profile x amplitude x run weight (float32
//           products, each rounded to the unit 2^-e: exact and order-independent sums).
#define ANF_WPB 8

__device__ __forceinline__ float phi_f32(float t, const float *__restrict__ tab) {
    const float x = (t + 6.0f) * 512.0f;
    if (!(x > 0.0f)) return 0.0f;
    if (x >= (float)(PHI_N - 1)) return 1.0f;
    const int k = (int)x;
    const float t0 = __ldg(tab + k), t1 = __ldg(tab + k + 1);
    return fmaf(x - (float)k, t1 - t0, t0);
}

// The line of a float32-path sample: bbarolo/galmod.py:407 and :410 (_velgrid, _lround) in float-float (about 44
// bits: the channel and the velocity relative to vref within ~1e-11 of the reference's float64 values); within 1e-6
// of a channel boundary the reference's float64 operations decide the centre channel. Returns the centre channel
// and the line-of-sight velocity v (float-float).
__device__ __forceinline__ long long fast_line_centre(const AnSub &S, const GridDev &g, float4 cq,
                                                      const double2 *__restrict__ cp, ff &v) {
    const ff caz{cq.x, cq.y}, saz{cq.z, cq.w};
    v = ff_add(ff_mul(ff{S.vroth, S.vrotl}, caz), ff_mul(ff{S.vradh, S.vradl}, saz));
    v = ff_add(ff_mul(v, ff{S.sinch, S.sincl}), ff_mul(ff{S.vverth, S.vvertl}, ff{S.cinch, S.cincl}));
    v = ff_add(ff{S.vsysh, S.vsysl}, v);
    const ff chd = ff_add(ff_mul(v, ff{g.ia0h, g.ia0l}), ff{g.ib0h, g.ib0l});
    int kci;
    if (ff_round(chd, kci)) return kci;
    const double2 c = *cp;
    const double vplane = __dadd_rn(__dadd_rn(S.vsys, __dmul_rn(__dadd_rn(__dmul_rn(S.vrot, c.x),
                                                                          __dmul_rn(S.vrad, c.y)), S.sinc)),
                                    __dmul_rn(S.vvert, S.cinc));
    return lround_ref(velgrid_exact(vplane, g, 0));
}

__global__ void __launch_bounds__(ANF_WPB * 32, 4) k_an_model_fast(GridDev g, const AnSub *__restrict__ subs, int nsub,
                                                                const int *__restrict__ sbase,
                                                                const int *__restrict__ ssub,
                                                                const double2 *__restrict__ cs,
                                                                const float2 *__restrict__ csf,
                                                                const float4 *__restrict__ csff,
                                                                const long long *__restrict__ astart,
                                                                const int4 *__restrict__ aseg, int nseg,
                                                                long long ntot, const double *__restrict__ zq,
                                                                const float *__restrict__ zqf,
                                                                const float *__restrict__ wqf,
                                                                const float2 *__restrict__ vef,
                                                                const float *__restrict__ cd2if,
                                                                const float *__restrict__ ptabf,
                                                                const MemberDev *__restrict__ mem,
                                                                unsigned long long *__restrict__ out64,
                                                                long long mstride, int skip_thin) {
    extern __shared__ float anf_smem[];                     // per warp: the CDF at the edges, the profile
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gs = (long long)blockIdx.x * ANF_WPB + w;
    AnSeg sg;
    if (!an_seg(gs, astart, aseg, nseg, ntot, sbase, sg)) return;
    const int k = sg.k;
    const long long s = sg.s;
    const int ir = ssub[s];
    const AnSub &S = subs[(size_t)sg.src * nsub + ir];
    if (!S.active || !S.anfast || (skip_thin && S.nzz == 1)) return;
    const float2 cf = csf[s];
    const bool rec = cf.x >= 0.0f;                          // (the sign of the float32 table is the float64 test's)
    if (S.wzero & (rec ? 1 : 2)) return;
    const int kr = (int)(s - sbase[ir]) >= S.naz ? 1 : 0;
    const PixF px = pix_setup(S, kr, cf, zqf + S.zq_off, S.nzz);
    const MemberDev &M = mem[k];
    const int nz = g.nz, nzz = S.nzz, off = S.zq_off;
    float *phe = anf_smem + (size_t)w * 2 * (nz + 2);
    float *prof = phe + nz + 2;
    unsigned long long *o64 = out64 + (size_t)k * mstride;
    int k0 = 0, nk = -1;                                    // the line's channels (nk < 0: not computed yet)
    auto line = [&]() {
        ff v;
        const long long kc = fast_line_centre(S, g, csff[s], cs + s, v);
        long long a0 = kc - S.K, a1 = kc + S.K + 1;
        if (a0 < 0) a0 = 0;
        if (a1 > nz) a1 = nz;
        if (a1 <= a0) {
            nk = 0;
            return;
        }
        k0 = (int)a0;
        nk = (int)(a1 - a0);
        const ff vr = ff_add(v, ff{-g.vrefh, -g.vrefl});
        const float vrh = vr.hi, vrl = vr.lo;
        const float amp = (float)sg.sign * ldexpf(S.af * (rec ? S.wrecf : S.wappf), M.fix_exp);
        for (int j = lane; j <= nk; j += 32) {
            const float2 e = __ldg(vef + k0 + j);
            const float t = (__fsub_rn(e.x, vrh) + __fsub_rn(e.y, vrl)) * S.invf;
            phe[j] = phi_f32(t, ptabf);
        }
        __syncwarp();
        for (int j = lane; j < nk; j += 32) prof[j] = fabsf(phe[j + 1] - phe[j]) * __ldg(cd2if + k0 + j) * amp;
        __syncwarp();
    };
    auto deposit = [&](int g0, int g1, float ws) {          // (warp-uniform arguments)
        if (g0 < M.blo0 || g0 >= M.bhi0 || g1 < M.blo1 || g1 >= M.bhi1) return;
        if (nk < 0) line();
        if (nk == 0) return;
        unsigned long long *o = o64 + ((size_t)(g1 - M.blo1) * M.bx + (size_t)(g0 - M.blo0)) * nz + k0;
        for (int j = lane; j < nk; j += 32) {
            const long long q = f32_to_ll(prof[j] * ws);
            if (q) atomicAdd(o + j, (unsigned long long)q);
        }
    };
    bool open = false;                                      // a run carried from the previous pass
    int cg0 = 0, cg1 = 0;
    float cws = 0.0f;
    for (int base = 0; base < nzz; base += 32) {
        const int cnt = min(32, nzz - base);
        const bool valid = lane < cnt;
        int g0 = 0x7fffffff, g1 = 0x7fffffff;
        float wv = 0.0f;
        if (valid) {
            sample_pixel(S, px, kr, cs + s, nzz, nzz > 1 ? zqf[off + base + lane] : 0.f, zq + off + base + lane,
                         g.cdelt0, g.cdelt1, g0, g1);
            wv = wqf[off + base + lane];
        }
        const int pg0 = __shfl_up_sync(FULL, g0, 1), pg1 = __shfl_up_sync(FULL, g1, 1);
        const bool start = valid && (lane == 0 ? (!open || g0 != cg0 || g1 != cg1) : (g0 != pg0 || g1 != pg1));
        const unsigned smask = __ballot_sync(FULL, start);
        if (open && (smask & 1u)) {                         // the carried run ended with the previous pass
            deposit(cg0, cg1, cws);
            open = false;
        }
        // segmented inclusive scan of the weights (a segment: from a run start to the lane before the next)
        const unsigned upto = smask & (0xffffffffu >> (31 - lane));
        const int head = upto ? 31 - __clz(upto) : 0;
        float v = wv;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float t = __shfl_up_sync(FULL, v, d);
            if (lane - d >= head) v += t;
        }
        if (!upto && open) v += cws;                        // (the lanes that continue the carried run)
        const bool nstart = lane < 31 && ((smask >> (lane + 1)) & 1u);
        const bool last = lane == cnt - 1;
        const bool final_pass = base + 32 >= nzz;
        const bool done = valid && ((!last && nstart) || (last && final_pass));
        unsigned dmask = __ballot_sync(FULL, done);
        while (dmask) {
            const int e = __ffs(dmask) - 1;
            dmask &= dmask - 1;
            deposit(__shfl_sync(FULL, g0, e), __shfl_sync(FULL, g1, e), __shfl_sync(FULL, v, e));
        }
        if (!final_pass) {
            cg0 = __shfl_sync(FULL, g0, cnt - 1);
            cg1 = __shfl_sync(FULL, g1, cnt - 1);
            cws = __shfl_sync(FULL, v, cnt - 1);
            open = true;
        }
    }
}

// The float32 path of the samples of thin sub-rings (one height, nzz = 1), 32 samples a warp: each lane sets up its
// own sample (segment, pixel, box test, line centre, amplitude), then the warp deposits the samples in the box one
// after another with its lanes over the channels. The same operations as k_an_model_fast on such a sample (one run
// of one height: its weight is the height's), so the deposits are the same integers; the warp-uniform set-up that
// k_an_model_fast repeats on 32 lanes for each sample is done once per lane here.
__global__ void __launch_bounds__(ANF_WPB * 32, 4) k_an_model_thin(GridDev g, const AnSub *__restrict__ subs, int nsub,
                                                                   const int *__restrict__ sbase,
                                                                   const int *__restrict__ ssub,
                                                                   const double2 *__restrict__ cs,
                                                                   const float2 *__restrict__ csf,
                                                                   const float4 *__restrict__ csff,
                                                                   const long long *__restrict__ astart,
                                                                   const int4 *__restrict__ aseg, int nseg,
                                                                   long long ntot, const double *__restrict__ zq,
                                                                   const float *__restrict__ zqf,
                                                                   const float *__restrict__ wqf,
                                                                   const float2 *__restrict__ vef,
                                                                   const float *__restrict__ cd2if,
                                                                   const float *__restrict__ ptabf,
                                                                   const MemberDev *__restrict__ mem,
                                                                   unsigned long long *__restrict__ out64,
                                                                   long long mstride) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gs = ((long long)blockIdx.x * ANF_WPB + w) * 32 + lane;
    const int nz = g.nz;
    bool ok = false;
    int k0 = 0, nk = 0;
    long long opix = 0;
    float vrh = 0.0f, vrl = 0.0f, invf = 0.0f, amp = 0.0f, ws = 0.0f;
    AnSeg sg;
    if (an_seg(gs, astart, aseg, nseg, ntot, sbase, sg)) {
        const long long s = sg.s;
        const int ir = ssub[s];
        const AnSub &S = subs[(size_t)sg.src * nsub + ir];
        const float2 cf = csf[s];
        const bool rec = cf.x >= 0.0f;
        if (S.active && S.anfast && S.nzz == 1 && !(S.wzero & (rec ? 1 : 2))) {
            const int kr = (int)(s - sbase[ir]) >= S.naz ? 1 : 0;
            const PixF px = pix_setup(S, kr, cf, zqf + S.zq_off, 1);
            int g0, g1;
            sample_pixel(S, px, kr, cs + s, 1, 0.f, zq + S.zq_off, g.cdelt0, g.cdelt1, g0, g1);
            const MemberDev &M = mem[sg.k];
            if (g0 >= M.blo0 && g0 < M.bhi0 && g1 >= M.blo1 && g1 < M.bhi1) {
                ff v;
                const long long kc = fast_line_centre(S, g, csff[s], cs + s, v);
                long long a0 = kc - S.K, a1 = kc + S.K + 1;
                if (a0 < 0) a0 = 0;
                if (a1 > nz) a1 = nz;
                if (a1 > a0) {
                    ok = true;
                    k0 = (int)a0;
                    nk = (int)(a1 - a0);
                    const ff vr = ff_add(v, ff{-g.vrefh, -g.vrefl});
                    vrh = vr.hi;
                    vrl = vr.lo;
                    invf = S.invf;
                    amp = (float)sg.sign * ldexpf(S.af * (rec ? S.wrecf : S.wappf), M.fix_exp);
                    ws = wqf[S.zq_off];
                    opix = (long long)sg.k * mstride + ((long long)(g1 - M.blo1) * M.bx + (g0 - M.blo0)) * nz + k0;
                }
            }
        }
    }
    unsigned todo = __ballot_sync(FULL, ok);
    while (todo) {
        const int e = __ffs(todo) - 1;
        todo &= todo - 1;
        const int ek0 = __shfl_sync(FULL, k0, e), enk = __shfl_sync(FULL, nk, e);
        const float evh = __shfl_sync(FULL, vrh, e), evl = __shfl_sync(FULL, vrl, e);
        const float einv = __shfl_sync(FULL, invf, e), eamp = __shfl_sync(FULL, amp, e);
        const float ews = __shfl_sync(FULL, ws, e);
        const long long eop = __shfl_sync(FULL, opix, e);
        for (int j = lane; j < enk; j += 32) {
            const float2 ea = __ldg(vef + ek0 + j), eb = __ldg(vef + ek0 + j + 1);
            const float ta = (__fsub_rn(ea.x, evh) + __fsub_rn(ea.y, evl)) * einv;
            const float tb = (__fsub_rn(eb.x, evh) + __fsub_rn(eb.y, evl)) * einv;
            const float p = fabsf(phi_f32(tb, ptabf) - phi_f32(ta, ptabf)) * __ldg(cd2if + ek0 + j) * eamp;
            const long long q = f32_to_ll(p * ews);
            if (q) atomicAdd(out64 + eop + j, (unsigned long long)q);
        }
    }
}

// Ring maps: maps64 (nr, by, bx) += fixed-point weights of the runs (bbarolo/galmod.py:518-529).
__global__ void __launch_bounds__(AN_WPB * 32) k_an_maps(GridDev g, const AnSub *__restrict__ subs, int nsub,
                                                         const int *__restrict__ sbase, const int *__restrict__ ssub,
                                                         const double2 *__restrict__ cs, long long nsamp,
                                                         const double *__restrict__ zq, const double *__restrict__ wq,
                                                         const long long *__restrict__ widx,
                                                         const double *__restrict__ wval, MemberDev M,
                                                         unsigned long long *__restrict__ maps64) {
    __shared__ AnWarp wsm[AN_WPB];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gs = (long long)blockIdx.x * AN_WPB + w;
    if (gs >= nsamp) return;
    const AnSub *Sp;
    double caz, saz, R;
    if (!an_sample(gs, 0, nsub, subs, sbase, ssub, cs, Sp, caz, saz, R)) return;
    const AnSub &S = *Sp;
    const double wside = caz >= 0.0 ? S.wrec : S.wapp;
    if (wside == 0.0) return;
    AnWarp &W = wsm[w];
    const double fscale = ldexp(1.0, M.fix_exp);
    const double x = __dmul_rn(R, caz);
    const double yb = __dmul_rn(__dmul_rn(R, saz), S.cinc);
    const double xs = __dmul_rn(x, S.spa), xc = __dmul_rn(x, S.cpa);
    const size_t plane = (size_t)M.by * M.bx;
    auto emit = [&](int g0, int g1, double ws) {
        if (g0 < M.blo0 || g0 >= M.bhi0 || g1 < M.blo1 || g1 >= M.bhi1) return;
        if (lane < 2) {
            const long long r = widx[2 * S.sub + lane];
            if (r >= 0) {
                const double t = __dmul_rn(__dmul_rn(__dmul_rn(S.fluxsc, ws), wval[2 * S.sub + lane]), wside);
                const long long q = __double2ll_rn(__dmul_rn(t, fscale));
                if (q)
                    atomicAdd(maps64 + (size_t)r * plane + (size_t)(g1 - M.blo1) * M.bx + (size_t)(g0 - M.blo0),
                              (unsigned long long)q);
            }
        }
    };
    an_runs(S, zq + S.zq_off, wq + S.zq_off, g.cdelt0, g.cdelt1, xs, xc, yb, W.sgx, W.sgy, W.rg0, W.rg1, W.rws,
            emit);
}

// fixed point (units 2^-e of member k) -> float32 model and, optionally, float64 copy
// (mbase[k] >= 0: member k holds the difference from that member's sums, added modulo 2^64: the same box and unit)
__global__ void k_fix_to_model(const long long *__restrict__ in, const MemberDev *__restrict__ mem, long long mstride,
                               int nz, float *__restrict__ model, double *__restrict__ model64,
                               const int *__restrict__ mbase) {
    const int k = blockIdx.y;
    const MemberDev &M = mem[k];
    const long long n = (long long)M.by * M.bx * nz;
    const double sc = ldexp(1.0, -M.fix_exp);
    const long long *bas = mbase && mbase[k] >= 0 ? in + (size_t)mbase[k] * mstride : nullptr;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long q = in[(size_t)k * mstride + i];
        if (bas) q = (long long)((unsigned long long)q + (unsigned long long)bas[i]);
        const double v = __dmul_rn((double)q, sc);
        model[(size_t)k * mstride + i] = (float)v;
        if (model64) model64[(size_t)k * mstride + i] = v;
    }
}

}  // namespace

size_t an_smem_bytes(int nz, int nlines) { return (size_t)AN_WPB * nlines * (nz + 2) * sizeof(double); }

void launch_an_model(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase, const int *ssub,
                     const double *cs, const long long *astart, const int *aseg, int nseg, long long ntot,
                     const double *zq, const double *wq, const double *vedges, const double *cd2i, const double *ptab,
                     const MemberDev *mem, long long *out64, long long mstride, int skip_fast) {
    const long long nw = ntot;
    if (nw == 0 || nseg == 0) return;
    const size_t smem = an_smem_bytes(g.nz, g.nlines);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_an_model, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_an_model<<<(unsigned)((nw + AN_WPB - 1) / AN_WPB), AN_WPB * 32, smem, s>>>(
        g, subs, nsub, sbase, ssub, (const double2 *)cs, astart, (const int4 *)aseg, nseg, ntot, zq, wq, vedges, cd2i,
        ptab, mem, (unsigned long long *)out64, mstride, skip_fast);
}

size_t an_fast_smem_bytes(int nz) { return (size_t)ANF_WPB * 2 * (nz + 2) * sizeof(float); }

void launch_an_model_fast(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase,
                          const int *ssub, const double *cs, const float *csf, const float *csff,
                          const long long *astart, const int *aseg, int nseg, long long ntot,
                          const double *zq, const float *zqf, const float *wqf, const float *vef, const float *cd2if,
                          const float *ptabf, const MemberDev *mem, long long *out64, long long mstride, int thin,
                          int thick) {
    const long long nw = ntot;
    if (nw == 0 || nseg == 0) return;
    if (thin)
        k_an_model_thin<<<(unsigned)((nw + 32 * ANF_WPB - 1) / (32 * ANF_WPB)), ANF_WPB * 32, 0, s>>>(
            g, subs, nsub, sbase, ssub, (const double2 *)cs, (const float2 *)csf, (const float4 *)csff, astart,
            (const int4 *)aseg, nseg, ntot, zq, zqf, wqf, (const float2 *)vef, cd2if, ptabf, mem,
            (unsigned long long *)out64, mstride);
    if (!thick) return;
    const size_t smem = an_fast_smem_bytes(g.nz);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_an_model_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_an_model_fast<<<(unsigned)((nw + ANF_WPB - 1) / ANF_WPB), ANF_WPB * 32, smem, s>>>(
        g, subs, nsub, sbase, ssub, (const double2 *)cs, (const float2 *)csf, (const float4 *)csff, astart,
        (const int4 *)aseg, nseg, ntot, zq, zqf, wqf,
        (const float2 *)vef, cd2if, ptabf, mem, (unsigned long long *)out64, mstride, thin);
}

void launch_an_maps(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase, const int *ssub,
                    const double *cs, long long nsamp, const double *zq, const double *wq, const long long *widx,
                    const double *wval, const MemberDev &M, long long *maps64) {
    if (nsamp == 0) return;
    k_an_maps<<<(unsigned)((nsamp + AN_WPB - 1) / AN_WPB), AN_WPB * 32, 0, s>>>(
        g, subs, nsub, sbase, ssub, (const double2 *)cs, nsamp, zq, wq, widx, wval, M, (unsigned long long *)maps64);
}

void launch_fix_to_model(cudaStream_t s, const long long *in, const MemberDev *mem, int nb, long long mstride, int nz,
                         float *model, double *model64, const int *mbase) {
    if (nb == 0) return;
    dim3 grid(256, nb);
    k_fix_to_model<<<grid, 256, 0, s>>>(in, mem, mstride, nz, model, model64, mbase);
}
