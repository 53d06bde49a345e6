// The column engine of the bi-conical wind models of WINDFIT on the device (the reference's WindModel,
// bbarolo/windmodel.py:212-602, and the normal equations of its columns that BayesianWind solves for the
// amplitudes of the cells, bbarolo/bayesian/wind.py:742-753).
//
// A wind model is linear in the amplitudes of a fixed grid of cells on the cones; column k (cell k) is a dense box of
// the cube. Per evaluation (one set of wind parameters):
//   k_wind_points    one thread per quadrature point: sky position, line-of-sight velocity and dispersion, the
//                    un-normalised weight r^2 sin(theta) (bbarolo/windmodel.py:225-288);
//   k_wind_cells     one warp per cell: its clipped volume, the weights normalised to it, the mean radius;
//   k_wind_rawbox    one warp per cell: the pixels and channels that its points reach (windmodel.py:291-319);
//   (host)           offsets of the raw boxes and of the beam-grown boxes: one read of ncell x 6 integers;
//   k_wind_deposit   one warp per point, lanes over channels: the channel-integrated line (the tabulated normal
//                    CDF) times the bilinear weights of the four nearest pixels, added to the raw box of the cell
//                    (float64 atomics; windmodel.py:322-366);
//   k_wind_conv_*    one thread per voxel of a box: the beam convolution of each raw box into its grown box, as
//                    two 1D passes for a separable beam, else with the 2D kernel, each sum in the reference's order
//                    (windmodel.py:369-423);
//   k_wind_lists     the voxel lists of the reference (windmodel.py:477-527): the entries (A != 0, |A| >= rel x
//                    the peak of the column, W != 0) counted per voxel, offsets by a scan, then written;
//   k_wind_lists_gram  one warp per voxel: b[k] += A_k Wd and G[k, l] += W A_k A_l over the pairs of its entries
//                    (windmodel.py:530-554), float64 atomics.
// Everything is float64, as the reference. The sums differ from the reference's sequential sums by rounding only
// (the deposits' order is not fixed, and the reductions are trees).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/bbgpu.h"
#include "internal.h"
#include "kernels.h"

#define WIND_PHI_N 6146
#define WIND_MAXL 4
#define WIND_MAXRAD 256
#define WIND_MAXCELL 16384
#define WIND_SMEM_VALS 26624          // the largest raw box deposited in shared memory (208 KB of 64-bit sums)
#define W_C_MS 2.99792458e08
#define FULLMASK 0xffffffffu

struct WindGridDev {
    int nx, ny, nz, nlines, axtyp, velsys;
    double cd0, cd1, sig_instr, chmin, crval3, cdelt3, crpix3;
    double lfreq0[WIND_MAXL], relint[WIND_MAXL];
};

struct WindLim {             // the raw limits: the cube box grown by the beam ([lo, hi) in x, y and channels)
    long long x0, x1, y0, y1, k0, k1;
};

struct WindParsDev {
    double x0, y0, vsys, sinc, cinc, spa, cpa, th_in, th_out, rmax;
    int nrad;
};

struct bbgpu_wind {
    int device = 0;
    cudaStream_t s = nullptr;
    WindGridDev g{};
    int hx = 0, hy = 0, separable = 1;
    double *d_vedges = nullptr, *d_ptab = nullptr;
    float2 *d_kern = nullptr, *d_kx = nullptr, *d_ky = nullptr;     // the beam taps as float-float (hi, lo)
    // cells and their quadrature
    int ncell = 0;
    long long npts = 0;
    double *d_cells = nullptr;
    int4 *d_qn = nullptr;
    long long *d_qoff = nullptr;
    int *d_pcell = nullptr;
    int tabmax = 0;                     // the largest per-cell sample table of k_wind_points_cell (doubles)
    // points of the last bbgpu_wind_points / bbgpu_wind_set_points
    double *d_gx = nullptr, *d_gy = nullptr, *d_vel = nullptr, *d_sig = nullptr, *d_w = nullptr, *d_rr = nullptr;
    double *d_vol = nullptr, *d_rbar = nullptr, *d_weight = nullptr, *d_rad = nullptr;
    bool have_points = false;
    // boxes of the last bbgpu_wind_boxes
    long long *d_rbox = nullptr, *d_box = nullptr, *d_roffs = nullptr, *d_offs = nullptr, *d_toffs = nullptr;
    std::vector<long long> h_rbox, h_box, h_offs, h_roffs, h_toffs;
    double *d_rbuf = nullptr, *d_buf = nullptr;
    float2 *d_rff = nullptr, *d_tmp = nullptr;      // raw boxes scaled to [0, 1) and the x pass, float-float
    int *d_bexp = nullptr;                          // the power of two of each raw box
    size_t cap_rbuf = 0, cap_buf = 0, cap_tmp = 0, cap_rff = 0;
    long long total = 0;
    bool have_boxes = false;
    // normal equations
    double *d_W = nullptr, *d_Wd = nullptr, *d_thr = nullptr, *d_G = nullptr, *d_b = nullptr, *d_out = nullptr;
    size_t cap_out = 0;
    int *d_cnt = nullptr, *d_start = nullptr, *d_cursor = nullptr, *d_scan = nullptr, *d_ecell = nullptr;
    double *d_eval = nullptr;
    size_t cap_cnt = 0, cap_start = 0, cap_cursor = 0, cap_scan = 0, cap_ecell = 0, cap_eval = 0;
    bool have_weights = false;
    int64_t launches = 0;
    std::string err;
};

namespace {

// bbarolo/galmod.py:183-191: the normal CDF at t from the table (512 entries per unit from -6)
__device__ __forceinline__ double wphi(double t, const double *__restrict__ tab) {
    const double x = __dmul_rn(__dadd_rn(t, 6.0), 512.0);
    if (x <= 0.0) return 0.0;
    const long long k = (long long)x;
    if (k >= WIND_PHI_N - 1) return 1.0;
    const double t0 = tab[k], t1 = tab[k + 1];
    return __dadd_rn(t0, __dmul_rn(__dsub_rn(x, (double)k), __dsub_rn(t1, t0)));
}

// bbarolo/galmod.py:38-46
__device__ __forceinline__ long long wround(double x) {
    if (!(fabs(x) < 1e18)) return -(1LL << 62);
    if (x >= 0) return (long long)__dadd_rn(x, 0.5);
    return -(long long)__dadd_rn(-x, 0.5);
}

// bbarolo/galmod.py:49-62: the channel of velocity v for line nl
__device__ __forceinline__ double wvelgrid(double v, const WindGridDev &g, int nl) {
    double w;
    if (g.axtyp == 4) w = v;
    else {
        const double f0 = g.lfreq0[nl];
        if (g.velsys == 1) w = __dmul_rn(f0, __dsub_rn(1.0, __ddiv_rn(v, W_C_MS)));
        else if (g.velsys == 2) w = __dmul_rn(f0, __ddiv_rn(W_C_MS, __dadd_rn(W_C_MS, v)));
        else w = __dmul_rn(f0, __dsqrt_rn(__ddiv_rn(__dsub_rn(W_C_MS, v), __dadd_rn(W_C_MS, v))));
        if (g.axtyp == 2) w = __ddiv_rn(W_C_MS, w);
    }
    return __dsub_rn(__dadd_rn(__ddiv_rn(__dsub_rn(w, g.crval3), g.cdelt3), g.crpix3), 1.0);
}

// bbarolo/windmodel.py:212-222: ys(xs) at r, linear, constant beyond the ends
__device__ __forceinline__ double winterp(double r, const double *__restrict__ xs, const double *__restrict__ ys,
                                          int n) {
    if (n == 1 || r <= xs[0]) return ys[0];
    if (r >= xs[n - 1]) return ys[n - 1];
    int j = 1;
    while (xs[j] < r) j++;
    const double t = __ddiv_rn(__dsub_rn(r, xs[j - 1]), __dsub_rn(xs[j], xs[j - 1]));
    return __dadd_rn(ys[j - 1], __dmul_rn(t, __dsub_rn(ys[j], ys[j - 1])));
}

// the clipped extent of cell k (bbarolo/windmodel.py:232-236); false if the cone leaves nothing of it
__device__ __forceinline__ bool wclip(const double *__restrict__ c, const WindParsDev &p, double &r0, double &r1,
                                      double &t0, double &t1) {
    r0 = c[1];
    r1 = p.rmax < c[2] ? p.rmax : c[2];
    t0 = p.th_in > c[3] ? p.th_in : c[3];
    t1 = p.th_out < c[4] ? p.th_out : c[4];
    return !(r1 <= r0 || t1 <= t0);
}

// bbarolo/windmodel.py:225-270 (the points; the normalisation is k_wind_cells). rad: radii, vw, vd, vr (nrad each).
__global__ void __launch_bounds__(256) k_wind_points(const double *__restrict__ cells, const int4 *__restrict__ qn,
                                                     const long long *__restrict__ qoff, const int *__restrict__ pcell,
                                                     long long npts, WindParsDev p, const double *__restrict__ rad,
                                                     WindGridDev g, double *__restrict__ gx, double *__restrict__ gy,
                                                     double *__restrict__ vel, double *__restrict__ sig,
                                                     double *__restrict__ w, double *__restrict__ rr) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    const int k = pcell[i];
    const double *c = cells + 7 * (size_t)k;
    double r0, r1, t0, t1;
    if (!wclip(c, p, r0, r1, t0, t1)) {
        gx[i] = -1e9; gy[i] = -1e9; vel[i] = 0.; sig[i] = 1.; w[i] = 0.; rr[i] = r0;
        return;
    }
    const int4 q = qn[k];
    const long long j = i - qoff[k];
    const long long tp = (long long)q.y * q.z;
    const long long a = j / tp;
    const long long rem = j - a * tp;
    const long long b = rem / q.z, cc = rem - b * q.z;
    const double cs = c[0], p0 = c[5], p1 = c[6];
    const double dr = __ddiv_rn(__dsub_rn(r1, r0), (double)q.x);
    const double dt = __ddiv_rn(__dsub_rn(t1, t0), (double)q.y);
    const double dp = __ddiv_rn(__dsub_rn(p1, p0), (double)q.z);
    const double r = __dadd_rn(r0, __dmul_rn(__dadd_rn((double)a, 0.5), dr));
    const int n = p.nrad;
    const double vrad = __dmul_rn(winterp(r, rad, rad + n, n), 1000.);
    const double disp = __dmul_rn(winterp(r, rad, rad + 2 * n, n), 1000.);
    const double vrot = __dmul_rn(winterp(r, rad, rad + 3 * n, n), 1000.);
    const double s = __dsqrt_rn(__dadd_rn(__dmul_rn(disp, disp), __dmul_rn(g.sig_instr, g.sig_instr)));
    const double th = __dadd_rn(t0, __dmul_rn(__dadd_rn((double)b, 0.5), dt));
    const double ph = __dadd_rn(p0, __dmul_rn(__dadd_rn((double)cc, 0.5), dp));
    double st, ct, sp, cp;
    sincos(th, &st, &ct);
    sincos(ph, &sp, &cp);
    const double R = __dmul_rn(r, st);
    const double z = __dmul_rn(__dmul_rn(cs, r), ct);
    const double x = __dmul_rn(R, cp);
    const double ys = __dsub_rn(__dmul_rn(__dmul_rn(R, sp), p.cinc), __dmul_rn(z, p.sinc));
    gx[i] = __dadd_rn(p.x0, __ddiv_rn(__dsub_rn(__dmul_rn(x, p.spa), __dmul_rn(ys, p.cpa)), g.cd0));
    gy[i] = __dadd_rn(p.y0, __ddiv_rn(__dadd_rn(__dmul_rn(x, p.cpa), __dmul_rn(ys, p.spa)), g.cd1));
    const double geo = __dadd_rn(__dmul_rn(__dmul_rn(cs, ct), p.cinc), __dmul_rn(__dmul_rn(st, sp), p.sinc));
    vel[i] = __dadd_rn(__dadd_rn(p.vsys, __dmul_rn(vrad, geo)), __dmul_rn(__dmul_rn(vrot, cp), p.sinc));
    sig[i] = s;
    w[i] = __dmul_rn(__dmul_rn(r, r), st);
    rr[i] = r;
}

// The same points with one CTA per cell: the values that depend on the radial, polar or azimuthal sample alone
// (radius, velocities and dispersion; sin and cos of theta; sin and cos of phi) computed once per sample into shared
// memory, then combined per point with the same operations as k_wind_points (bit-identical results).
__global__ void __launch_bounds__(256) k_wind_points_cell(const double *__restrict__ cells, const int4 *__restrict__ qn,
                                                          const long long *__restrict__ qoff, WindParsDev p,
                                                          const double *__restrict__ rad, WindGridDev g,
                                                          double *__restrict__ gx, double *__restrict__ gy,
                                                          double *__restrict__ vel, double *__restrict__ sig,
                                                          double *__restrict__ w, double *__restrict__ rr) {
    extern __shared__ double tab[];
    const int k = blockIdx.x;
    const double *c = cells + 7 * (size_t)k;
    const long long i0 = qoff[k], i1 = qoff[k + 1];
    double r0, r1, t0, t1;
    if (!wclip(c, p, r0, r1, t0, t1)) {
        for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
            gx[i] = -1e9; gy[i] = -1e9; vel[i] = 0.; sig[i] = 1.; w[i] = 0.; rr[i] = r0;
        }
        return;
    }
    const int4 q = qn[k];
    double *tr = tab, *tvr = tab + q.x, *tds = tab + 2 * q.x, *tvo = tab + 3 * q.x, *tst = tab + 4 * q.x;
    double *tct = tst + q.y, *tsp = tct + q.y, *tcp = tsp + q.z;
    const double cs = c[0], p0 = c[5], p1 = c[6];
    const double dr = __ddiv_rn(__dsub_rn(r1, r0), (double)q.x);
    const double dt = __ddiv_rn(__dsub_rn(t1, t0), (double)q.y);
    const double dp = __ddiv_rn(__dsub_rn(p1, p0), (double)q.z);
    const int n = p.nrad;
    for (int a = threadIdx.x; a < q.x; a += blockDim.x) {
        const double r = __dadd_rn(r0, __dmul_rn(__dadd_rn((double)a, 0.5), dr));
        tr[a] = r;
        tvr[a] = __dmul_rn(winterp(r, rad, rad + n, n), 1000.);
        const double disp = __dmul_rn(winterp(r, rad, rad + 2 * n, n), 1000.);
        tvo[a] = __dmul_rn(winterp(r, rad, rad + 3 * n, n), 1000.);
        tds[a] = __dsqrt_rn(__dadd_rn(__dmul_rn(disp, disp), __dmul_rn(g.sig_instr, g.sig_instr)));
    }
    for (int b = threadIdx.x; b < q.y; b += blockDim.x)
        sincos(__dadd_rn(t0, __dmul_rn(__dadd_rn((double)b, 0.5), dt)), tst + b, tct + b);
    for (int cc = threadIdx.x; cc < q.z; cc += blockDim.x)
        sincos(__dadd_rn(p0, __dmul_rn(__dadd_rn((double)cc, 0.5), dp)), tsp + cc, tcp + cc);
    __syncthreads();
    const int tp = q.y * q.z;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int j = (int)(i - i0);
        const int a = j / tp, rem = j - a * tp;
        const int b = rem / q.z, cc = rem - b * q.z;
        const double r = tr[a], st = tst[b], ct = tct[b], sp = tsp[cc], cp = tcp[cc];
        const double R = __dmul_rn(r, st);
        const double z = __dmul_rn(__dmul_rn(cs, r), ct);
        const double x = __dmul_rn(R, cp);
        const double ys = __dsub_rn(__dmul_rn(__dmul_rn(R, sp), p.cinc), __dmul_rn(z, p.sinc));
        gx[i] = __dadd_rn(p.x0, __ddiv_rn(__dsub_rn(__dmul_rn(x, p.spa), __dmul_rn(ys, p.cpa)), g.cd0));
        gy[i] = __dadd_rn(p.y0, __ddiv_rn(__dadd_rn(__dmul_rn(x, p.cpa), __dmul_rn(ys, p.spa)), g.cd1));
        const double geo = __dadd_rn(__dmul_rn(__dmul_rn(cs, ct), p.cinc), __dmul_rn(__dmul_rn(st, sp), p.sinc));
        vel[i] = __dadd_rn(__dadd_rn(p.vsys, __dmul_rn(tvr[a], geo)), __dmul_rn(__dmul_rn(tvo[a], cp), p.sinc));
        sig[i] = tds[a];
        w[i] = __dmul_rn(__dmul_rn(r, r), st);
        rr[i] = r;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
    return v;
}

// bbarolo/windmodel.py:271-288: one warp per cell: the clipped volume, the weights normalised to it, the mean radius
__global__ void __launch_bounds__(256) k_wind_cells(const double *__restrict__ cells, const long long *__restrict__ qoff,
                                                    int ncell, WindParsDev p, double *__restrict__ w,
                                                    const double *__restrict__ rr, double *__restrict__ vol,
                                                    double *__restrict__ rbar) {
    const int k = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (k >= ncell) return;
    const double *c = cells + 7 * (size_t)k;
    double r0, r1, t0, t1;
    if (!wclip(c, p, r0, r1, t0, t1)) {
        if (lane == 0) {
            vol[k] = 0.;
            rbar[k] = r1 > r0 ? __dmul_rn(0.5, __dadd_rn(r0, r1)) : r0;
        }
        return;
    }
    const long long i0 = qoff[k], i1 = qoff[k + 1];
    double ws = 0.;
    for (long long i = i0 + lane; i < i1; i += 32) ws += w[i];
    ws = warp_sum(ws);
    const double V = __dmul_rn(__dmul_rn(__ddiv_rn(__dsub_rn(pow(r1, 3.0), pow(r0, 3.0)), 3.),
                                         __dsub_rn(cos(t0), cos(t1))), __dsub_rn(c[6], c[5]));
    const double f = ws > 0 ? __ddiv_rn(V, ws) : 0.;
    double rs = 0.;
    for (long long i = i0 + lane; i < i1; i += 32) {
        const double wi = __dmul_rn(w[i], f);
        w[i] = wi;
        rs += wi * rr[i];
    }
    rs = warp_sum(rs);
    if (lane == 0) {
        vol[k] = V;
        rbar[k] = V > 0 ? __ddiv_rn(rs, V) : __dmul_rn(0.5, __dadd_rn(r0, r1));
    }
}

// the weight of point i in the columns (the normalised weight times the caller's weight of the point, if any)
__device__ __forceinline__ double wpoint(const double *__restrict__ w, const double *__restrict__ wt, long long i) {
    return wt ? __dmul_rn(w[i], wt[i]) : w[i];
}

__device__ __forceinline__ bool wpoint_ok(double wi, double gx, double gy) {
    return wi > 0. && fabs(gx) < 1e8 && fabs(gy) < 1e8;
}

__device__ __forceinline__ int clamp30(long long v) {
    return (int)(v < -(1LL << 30) ? -(1LL << 30) : (v > (1LL << 30) ? (1LL << 30) : v));
}

// bbarolo/windmodel.py:291-319: one warp per cell; lim: the raw limits (the cube box grown by the beam)
__global__ void __launch_bounds__(256) k_wind_rawbox(const long long *__restrict__ qoff, int ncell,
                                                     const double *__restrict__ gx, const double *__restrict__ gy,
                                                     const double *__restrict__ vel, const double *__restrict__ sig,
                                                     const double *__restrict__ w, const double *__restrict__ wt,
                                                     WindGridDev g, WindLim lim, long long *__restrict__ rbox) {
    const int k = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (k >= ncell) return;
    int bx0 = 1 << 30, bx1 = -(1 << 30), by0 = 1 << 30, by1 = -(1 << 30), bk0 = 1 << 30, bk1 = -(1 << 30);
    for (long long i = qoff[k] + lane; i < qoff[k + 1]; i += 32) {
        const double x = gx[i], y = gy[i];
        if (!wpoint_ok(wpoint(w, wt, i), x, y)) continue;
        const int ix = (int)floor(x), iy = (int)floor(y);
        bx0 = min(bx0, ix);
        bx1 = max(bx1, ix + 2);
        by0 = min(by0, iy);
        by1 = max(by1, iy + 2);
        const long long K = (long long)__ddiv_rn(__dmul_rn(5.0, sig[i]), g.chmin) + 2;
        for (int nl = 0; nl < g.nlines; nl++) {
            const long long kc = wround(wvelgrid(vel[i], g, nl));
            bk0 = min(bk0, clamp30(kc - K));
            bk1 = max(bk1, clamp30(kc + K + 1));
        }
    }
    bx0 = __reduce_min_sync(FULLMASK, bx0);
    bx1 = __reduce_max_sync(FULLMASK, bx1);
    by0 = __reduce_min_sync(FULLMASK, by0);
    by1 = __reduce_max_sync(FULLMASK, by1);
    bk0 = __reduce_min_sync(FULLMASK, bk0);
    bk1 = __reduce_max_sync(FULLMASK, bk1);
    if (lane) return;
    long long o[6] = {std::max((long long)bx0, lim.x0), std::min((long long)bx1, lim.x1),
                      std::max((long long)by0, lim.y0), std::min((long long)by1, lim.y1),
                      std::max((long long)bk0, lim.k0), std::min((long long)bk1, lim.k1)};
    if (o[1] <= o[0] || o[3] <= o[2] || o[5] <= o[4]) {
        o[0] = o[1] = lim.x0;
        o[2] = o[3] = lim.y0;
        o[4] = o[5] = lim.k0;
    }
    for (int j = 0; j < 6; j++) rbox[6 * (size_t)k + j] = o[j];
}

// the deposits of point i (bbarolo/windmodel.py:335-366): the channel-integrated line of each line times the
// bilinear weights, lanes over the channels of the line window; put(offset in the raw box, value)
template <class Put>
__device__ __forceinline__ void deposit_point(long long i, double wi, const double *__restrict__ gx,
                                              const double *__restrict__ gy, const double *__restrict__ vel,
                                              const double *__restrict__ sig, const long long *B,
                                              const double *__restrict__ vedges, const double *__restrict__ ptab,
                                              const WindGridDev &g, int lane, Put put) {
    const int x0 = (int)B[0], x1 = (int)B[1], y0 = (int)B[2], y1 = (int)B[3], k0 = (int)B[4], k1 = (int)B[5];
    const int bx = x1 - x0, by = y1 - y0;
    const double px = gx[i], py = gy[i];
    const int ix = (int)floor(px), iy = (int)floor(py);
    const double fx = __dsub_rn(px, (double)ix), fy = __dsub_rn(py, (double)iy);
    double s = sig[i];
    const double smin = __dmul_rn(1e-6, g.chmin);
    if (s < smin) s = smin;
    const long long K = (long long)__ddiv_rn(__dmul_rn(5.0, s), g.chmin) + 2;
    const double inv = __ddiv_rn(1.0, s);
    const double v = vel[i];
    for (int nl = 0; nl < g.nlines; nl++) {
        const long long kc = wround(wvelgrid(v, g, nl));
        long long a0 = kc - K, a1 = kc + K + 1;
        if (a0 < k0) a0 = k0;                 // (the window clipped to the cube, then to the box)
        if (a1 > k1) a1 = k1;
        if (a1 <= a0) continue;
        const double *ve = vedges + (size_t)nl * (g.nz + 1);
        const double amp = __dmul_rn(wi, g.relint[nl]);
        for (int kz = (int)a0 + lane; kz < (int)a1; kz += 32) {
            const double f = __dsub_rn(wphi(__dmul_rn(__dsub_rn(ve[kz + 1], v), inv), ptab),
                                       wphi(__dmul_rn(__dsub_rn(ve[kz], v), inv), ptab));
            const double pv = __dmul_rn(amp, f >= 0 ? f : -f);
            if (pv == 0.) continue;
            for (int dy = 0; dy < 2; dy++) {
                const int yy = iy + dy;
                if (yy < y0 || yy >= y1) continue;
                const double wy = dy == 1 ? fy : __dsub_rn(1., fy);
                const int row = ((kz - k0) * by + (yy - y0)) * bx - x0;
                for (int dx = 0; dx < 2; dx++) {
                    const int xx = ix + dx;
                    if (xx < x0 || xx >= x1) continue;
                    const double wx = dx == 1 ? fx : __dsub_rn(1., fx);
                    put(row + xx, __dmul_rn(__dmul_rn(pv, wx), wy));
                }
            }
        }
    }
}

__device__ __forceinline__ long long box_size(const long long *B) {
    return (B[1] - B[0]) * (B[3] - B[2]) * (B[5] - B[4]);
}

// one CTA per cell whose raw box holds at most maxvals values: its points deposited in shared memory in 64-bit
// fixed point (units of 2^(E-62), 2^E above the sum of the cell's weights times the lines' |relint|: no overflow;
// exact sums, independent of their order), the box written once
__global__ void __launch_bounds__(512) k_wind_deposit_cell(const long long *__restrict__ qoff,
                                                           const double *__restrict__ gx,
                                                           const double *__restrict__ gy,
                                                           const double *__restrict__ vel,
                                                           const double *__restrict__ sig,
                                                           const double *__restrict__ w,
                                                           const double *__restrict__ wt,
                                                           const long long *__restrict__ rbox,
                                                           const long long *__restrict__ roffs,
                                                           const double *__restrict__ vedges,
                                                           const double *__restrict__ ptab, WindGridDev g,
                                                           long long maxvals, double *__restrict__ rbuf) {
    extern __shared__ unsigned long long acc[];
    __shared__ double red[16];
    const int k = blockIdx.x;
    const long long *B = rbox + 6 * (size_t)k;
    if (B[1] <= B[0] || B[3] <= B[2] || B[5] <= B[4]) return;
    const int size = (int)box_size(B);
    if (size > maxvals) return;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = threadIdx.x; j < size; j += blockDim.x) acc[j] = 0ull;
    const long long i0 = qoff[k], i1 = qoff[k + 1];
    double sw = 0.;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double wi = wpoint(w, wt, i);
        if (wpoint_ok(wi, gx[i], gy[i])) sw += wi;
    }
    sw = warp_sum(sw);
    if (lane == 0) red[wid] = sw;
    __syncthreads();
    sw = 0.;
    for (int j = 0; j < nw; j++) sw += red[j];
    double rs = 0.;
    for (int nl = 0; nl < g.nlines; nl++) rs += fabs(g.relint[nl]);
    int E = 0;
    frexp(sw * rs * 1.0000001 + 1e-300, &E);
    const double scale = ldexp(1.0, 62 - E), unit = ldexp(1.0, E - 62);
    // a thread per point: its line window channel by channel (the CDF carried from one edge to the next, as the
    // reference), the four bilinear weights times the fixed-point scale computed once per point
    const int x0 = (int)B[0], x1 = (int)B[1], y0 = (int)B[2], y1 = (int)B[3], k0 = (int)B[4], k1 = (int)B[5];
    const int bx = x1 - x0, by = y1 - y0;
    const double smin = __dmul_rn(1e-6, g.chmin);
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double wi = wpoint(w, wt, i), px = gx[i], py = gy[i];
        if (!wpoint_ok(wi, px, py)) continue;
        const int ix = (int)floor(px), iy = (int)floor(py);
        const double fx = __dsub_rn(px, (double)ix), fy = __dsub_rn(py, (double)iy);
        const double wx[2] = {__dsub_rn(1., fx), fx}, wy[2] = {__dsub_rn(1., fy), fy};
        double c4[4];
        int o4[4];
        int nc = 0;
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                const int xx = ix + dx, yy = iy + dy;
                if (xx < x0 || xx >= x1 || yy < y0 || yy >= y1) continue;
                c4[nc] = wx[dx] * wy[dy] * scale;
                o4[nc++] = (yy - y0) * bx + (xx - x0);
            }
        if (nc == 0) continue;
        double sg = sig[i];
        if (sg < smin) sg = smin;
        const long long K = (long long)__ddiv_rn(__dmul_rn(5.0, sg), g.chmin) + 2;
        const double inv = __ddiv_rn(1.0, sg);
        const double v = vel[i];
        for (int nl = 0; nl < g.nlines; nl++) {
            const long long kc = wround(wvelgrid(v, g, nl));
            long long a0 = kc - K, a1 = kc + K + 1;
            if (a0 < k0) a0 = k0;
            if (a1 > k1) a1 = k1;
            if (a1 <= a0) continue;
            const double *ve = vedges + (size_t)nl * (g.nz + 1);
            const double amp = __dmul_rn(wi, g.relint[nl]);
            double pp = wphi(__dmul_rn(__dsub_rn(ve[a0], v), inv), ptab);
            for (int kz = (int)a0; kz < (int)a1; kz++) {
                const double pn = wphi(__dmul_rn(__dsub_rn(ve[kz + 1], v), inv), ptab);
                const double f = __dsub_rn(pn, pp);
                pp = pn;
                const double pv = __dmul_rn(amp, f >= 0 ? f : -f);
                if (pv == 0.) continue;
                unsigned long long *plane = acc + (size_t)(kz - k0) * by * bx;
                for (int c = 0; c < nc; c++)
                    atomicAdd(plane + o4[c], (unsigned long long)__double2ll_rn(pv * c4[c]));
            }
        }
    }
    __syncthreads();
    double *out = rbuf + roffs[k];
    for (int j = threadIdx.x; j < size; j += blockDim.x) out[j] = (double)(long long)acc[j] * unit;
}

// one warp per point of the cells whose raw box holds more than maxvals values: float64 atomics in global memory
__global__ void __launch_bounds__(256) k_wind_deposit(const int *__restrict__ pcell, long long npts,
                                                      const double *__restrict__ gx, const double *__restrict__ gy,
                                                      const double *__restrict__ vel, const double *__restrict__ sig,
                                                      const double *__restrict__ w, const double *__restrict__ wt,
                                                      const long long *__restrict__ rbox,
                                                      const long long *__restrict__ roffs,
                                                      const double *__restrict__ vedges,
                                                      const double *__restrict__ ptab, WindGridDev g,
                                                      long long maxvals, double *__restrict__ rbuf) {
    const long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= npts) return;
    const double wi = wpoint(w, wt, i);
    if (!wpoint_ok(wi, gx[i], gy[i])) return;
    const int k = pcell[i];
    const long long *B = rbox + 6 * (size_t)k;
    if (B[1] <= B[0] || B[3] <= B[2] || B[5] <= B[4] || box_size(B) <= maxvals) return;
    double *base = rbuf + roffs[k];
    deposit_point(i, wi, gx, gy, vel, sig, B, vedges, ptab, g, lane,
                  [&](int o, double val) { atomicAdd(base + o, val); });
}

// The beam convolution of the raw boxes: one CTA row block per (box, blockIdx.y), a warp per output row, lanes
// over its columns; each sum over the taps in the reference's order (raw columns, then raw rows, ascending). The
// float64 pipe of this GPU does two fused multiply-adds per clock per SM, so the sums run in float-float on the
// float32 pipes (an unevaluated sum hi + lo of two float32: products with their exact rounding error from an FMA,
// sums by an error-free two-sum, the low parts accumulated apart; relative error ~1e-14 of the box's peak) on the
// values of each raw box scaled by a power of two into [0, 1) (k_wind_to_ff), and the result converted back to
// float64 and unscaled.

// a += x * k in float-float (x, k: hi, lo); the low-order terms of the product and the rounding error of the sum
// are gathered in al
__device__ __forceinline__ void ff_fma(float &ah, float &al, float2 x, float2 k) {
    const float p = __fmul_rn(x.x, k.x);
    const float e = fmaf(x.x, k.x, -p);
    const float c = fmaf(x.x, k.y, fmaf(x.y, k.x, e));
    const float s = __fadd_rn(ah, p);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    ah = s;
    al = __fadd_rn(al, __fadd_rn(err, c));
}

__device__ __forceinline__ float2 ff_norm(float ah, float al) {
    const float h = __fadd_rn(ah, al);
    return make_float2(h, __fsub_rn(al, __fsub_rn(h, ah)));
}

// one CTA per raw box: its values times 2^-E (2^E above the box's largest magnitude) as float-float, and E
__global__ void __launch_bounds__(256) k_wind_to_ff(const double *__restrict__ rbuf, const long long *__restrict__ roffs,
                                                    float2 *__restrict__ rff, int *__restrict__ bexp) {
    __shared__ unsigned long long red[8];
    const int k = blockIdx.x;
    const long long j0 = roffs[k], j1 = roffs[k + 1];
    if (j1 == j0) return;
    unsigned long long m = 0;
    for (long long j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        const unsigned long long a = (unsigned long long)__double_as_longlong(rbuf[j]) & 0x7fffffffffffffffull;
        if (a < 0x7ff0000000000000ull) m = max(m, a);
    }
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(FULLMASK, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = max(m, red[i]);
    int E = 0;
    if (m) frexp(__longlong_as_double((long long)m), &E);
    const double sc = ldexp(1.0, -E);
    for (long long j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        const double v = __dmul_rn(rbuf[j], sc);
        const float h = __double2float_rn(v);
        rff[j] = make_float2(h, __double2float_rn(__dsub_rn(v, (double)h)));
    }
    if (threadIdx.x == 0) bexp[k] = E;
}

// bbarolo/windmodel.py:380-393, the x pass of a separable beam: tmp (box k: raw channels x raw rows x grown columns)
__global__ void __launch_bounds__(256) k_wind_conv_x(const float2 *__restrict__ rff, const long long *__restrict__ roffs,
                                                     const long long *__restrict__ rbox,
                                                     const long long *__restrict__ box,
                                                     const long long *__restrict__ toffs,
                                                     const float2 *__restrict__ kx, int hx, float2 *__restrict__ tmp) {
    const int k = blockIdx.x;
    if (toffs[k + 1] == toffs[k]) return;
    const long long *R = rbox + 6 * (size_t)k, *B = box + 6 * (size_t)k;
    const int rx0 = (int)R[0], rx1 = (int)R[1], rby = (int)(R[3] - R[2]), rbz = (int)(R[5] - R[4]);
    const int rbx = rx1 - rx0, x0 = (int)B[0], bx = (int)(B[1] - B[0]);
    const int lane = threadIdx.x & 31, nw = (blockDim.x >> 5) * gridDim.y;
    const float2 *src = rff + roffs[k];
    float2 *dst = tmp + toffs[k];
    for (int row = (threadIdx.x >> 5) + (blockDim.x >> 5) * blockIdx.y; row < rbz * rby; row += nw) {
        const float2 *a = src + (size_t)row * rbx - rx0;
        float2 *o = dst + (size_t)row * bx;
        for (int c = lane; c < bx; c += 32) {
            const int xx = x0 + c;
            const int xa = max(rx0, xx - hx), xb = min(rx1 - 1, xx + hx);
            float ah = 0.f, al = 0.f;
            for (int x = xa; x <= xb; x++) ff_fma(ah, al, a[x], kx[xx - x + hx]);
            o[c] = ff_norm(ah, al);
        }
    }
}

// bbarolo/windmodel.py:394-401, the y pass of a separable beam: buf (box k, float64) from tmp
__global__ void __launch_bounds__(256) k_wind_conv_y(const float2 *__restrict__ tmp, const long long *__restrict__ toffs,
                                                     const long long *__restrict__ rbox,
                                                     const long long *__restrict__ box,
                                                     const long long *__restrict__ offs,
                                                     const int *__restrict__ bexp, const float2 *__restrict__ ky,
                                                     int hy, double *__restrict__ buf) {
    const int k = blockIdx.x;
    if (offs[k + 1] == offs[k] || toffs[k + 1] == toffs[k]) return;
    const long long *R = rbox + 6 * (size_t)k, *B = box + 6 * (size_t)k;
    const int ry0 = (int)R[2], ry1 = (int)R[3], rby = ry1 - ry0;
    const int bx = (int)(B[1] - B[0]), by = (int)(B[3] - B[2]), bz = (int)(B[5] - B[4]), y0 = (int)B[2];
    const int lane = threadIdx.x & 31, nw = (blockDim.x >> 5) * gridDim.y;
    const double sc = ldexp(1.0, bexp[k]);
    const float2 *src = tmp + toffs[k];
    double *dst = buf + offs[k];
    for (int row = (threadIdx.x >> 5) + (blockDim.x >> 5) * blockIdx.y; row < bz * by; row += nw) {
        const int kz = row / by, yy = y0 + (row - kz * by);
        const int ya = max(ry0, yy - hy), yb = min(ry1 - 1, yy + hy);
        const float2 *t = src + (size_t)kz * rby * bx;
        double *o = dst + (size_t)row * bx;
        for (int c = lane; c < bx; c += 32) {
            float ah = 0.f, al = 0.f;
            for (int y = ya; y <= yb; y++) ff_fma(ah, al, t[(size_t)(y - ry0) * bx + c], ky[yy - y + hy]);
            o[c] = __dmul_rn(__dadd_rn((double)ah, (double)al), sc);
        }
    }
}

// bbarolo/windmodel.py:402-423: the 2D beam (not separable), kern (2hy+1, 2hx+1)
__global__ void __launch_bounds__(256) k_wind_conv_2d(const float2 *__restrict__ rff, const long long *__restrict__ roffs,
                                                      const long long *__restrict__ rbox,
                                                      const long long *__restrict__ box,
                                                      const long long *__restrict__ offs,
                                                      const int *__restrict__ bexp,
                                                      const float2 *__restrict__ kern, int hy, int hx,
                                                      double *__restrict__ buf) {
    const int k = blockIdx.x;
    if (offs[k + 1] == offs[k]) return;
    const long long *R = rbox + 6 * (size_t)k, *B = box + 6 * (size_t)k;
    const int rx0 = (int)R[0], rx1 = (int)R[1], ry0 = (int)R[2], ry1 = (int)R[3];
    const int rbx = rx1 - rx0, rby = ry1 - ry0;
    if (rbx <= 0 || rby <= 0 || R[5] <= R[4]) return;
    const int x0 = (int)B[0], bx = (int)(B[1] - B[0]), by = (int)(B[3] - B[2]), bz = (int)(B[5] - B[4]);
    const int y0 = (int)B[2], kw = 2 * hx + 1;
    const int lane = threadIdx.x & 31, nw = (blockDim.x >> 5) * gridDim.y;
    const double sc = ldexp(1.0, bexp[k]);
    const float2 *src = rff + roffs[k];
    double *dst = buf + offs[k];
    for (int row = (threadIdx.x >> 5) + (blockDim.x >> 5) * blockIdx.y; row < bz * by; row += nw) {
        const int kz = row / by, yy = y0 + (row - kz * by);
        const int ya = max(ry0, yy - hy), yb = min(ry1 - 1, yy + hy);
        const float2 *plane = src + (size_t)kz * rby * rbx;
        double *o = dst + (size_t)row * bx;
        for (int c = lane; c < bx; c += 32) {
            const int xx = x0 + c;
            const int xa = max(rx0, xx - hx), xb = min(rx1 - 1, xx + hx);
            float ah = 0.f, al = 0.f;
            for (int y = ya; y <= yb; y++) {
                const float2 *r = plane + (size_t)(y - ry0) * rbx - rx0;
                const float2 *kr = kern + (yy - y + hy) * kw + hx + xx;
                for (int x = xa; x <= xb; x++) ff_fma(ah, al, r[x], kr[-x]);
            }
            o[c] = __dmul_rn(__dadd_rn((double)ah, (double)al), sc);
        }
    }
}

// rel x the peak |value| of each column (one CTA per column)
__global__ void __launch_bounds__(256) k_wind_thr(const double *__restrict__ buf, const long long *__restrict__ offs,
                                                  double rel, double *__restrict__ thr) {
    __shared__ unsigned long long red[8];
    const int k = blockIdx.x;
    // (the magnitudes compared as integers: the bit patterns of non-negative doubles order as their values)
    unsigned long long m = 0;
    for (long long j = offs[k] + threadIdx.x; j < offs[k + 1]; j += blockDim.x) {
        const unsigned long long a = (unsigned long long)__double_as_longlong(buf[j]) & 0x7fffffffffffffffull;
        if (a <= 0x7ff0000000000000ull) m = max(m, a);              // (NaN never raises the peak)
    }
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(FULLMASK, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) m = max(m, red[i]);
        thr[k] = __dmul_rn(rel, __longlong_as_double((long long)m));
    }
}

// The voxel lists of the columns within lim (bbarolo/windmodel.py:477-527): an entry per column value that is
// != 0, at least thr[k] in magnitude and on a voxel with W != 0. pass 0 counts the entries of each voxel of lim;
// pass 1 writes them (cell, value) from the voxels' cursors. One CTA per column, a warp per row of its box.
__global__ void __launch_bounds__(256) k_wind_lists(int pass, const double *__restrict__ buf,
                                                    const long long *__restrict__ offs,
                                                    const long long *__restrict__ box,
                                                    const double *__restrict__ thr, const double *__restrict__ W,
                                                    int ny, int nx, WindLim lim, int *__restrict__ cnt,
                                                    int *__restrict__ cursor, int *__restrict__ ecell,
                                                    double *__restrict__ eval) {
    const int k = blockIdx.x;
    const long long *B = box + 6 * (size_t)k;
    const int bx = (int)(B[1] - B[0]), by = (int)(B[3] - B[2]), bz = (int)(B[5] - B[4]);
    if (bx <= 0 || by <= 0 || bz <= 0) return;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int lx = (int)(lim.x1 - lim.x0), ly = (int)(lim.y1 - lim.y0);
    // (the tests as integers on the bit patterns: |v| >= t for t >= 0, v != 0 and W != 0, off the float64 pipe)
    const unsigned long long t = (unsigned long long)__double_as_longlong(thr[k]);
    const double *col = buf + offs[k];
    for (int row = threadIdx.x >> 5; row < by * bz; row += nw) {
        const int zr = row / by, yr = row - zr * by;
        const int z = (int)B[4] + zr, y = (int)B[2] + yr;
        const double *a = col + (size_t)row * bx;
        const double *wr = W + ((size_t)z * ny + y) * nx + B[0];
        const int vrow = ((z - (int)lim.k0) * ly + (y - (int)lim.y0)) * lx + (int)(B[0] - lim.x0);
        for (int x = lane; x < bx; x += 32) {
            const double v = a[x];
            const unsigned long long av = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
            const unsigned long long aw = (unsigned long long)__double_as_longlong(wr[x]) & 0x7fffffffffffffffull;
            if (av == 0 || av < t || av > 0x7ff0000000000000ull || aw == 0) continue;
            if (pass == 0) {
                atomicAdd(cnt + vrow + x, 1);
            } else {
                const int j = atomicAdd(cursor + vrow + x, 1);
                ecell[j] = k;
                eval[j] = v;
            }
        }
    }
}

// bbarolo/windmodel.py:530-554: one warp per voxel of lim: b[k] += A_k Wd over its entries and, for every pair of
// its entries (k <= l), G[k, l] += (W A_k) A_l (float64 atomics; G is made symmetric afterwards)
__global__ void __launch_bounds__(256) k_wind_lists_gram(const int *__restrict__ cnt, const int *__restrict__ start,
                                                         const int *__restrict__ ecell,
                                                         const double *__restrict__ eval, int nvox,
                                                         const double *__restrict__ W, const double *__restrict__ Wd,
                                                         int ny, int nx, WindLim lim, int ncell,
                                                         double *__restrict__ G, double *__restrict__ b) {
    const long long wv = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wv >= nvox) return;
    const int i = (int)wv;
    const int n = cnt[i];
    if (n == 0) return;
    const int lx = (int)(lim.x1 - lim.x0), ly = (int)(lim.y1 - lim.y0);
    const int x = (int)lim.x0 + i % lx, t = i / lx;
    const int y = (int)lim.y0 + t % ly, z = (int)lim.k0 + t / ly;
    const size_t cv = ((size_t)z * ny + y) * nx + x;
    const double w = W[cv], d = Wd[cv];
    const int j0 = start[i];
    for (int p = lane; p < n; p += 32) atomicAdd(b + ecell[j0 + p], __dmul_rn(eval[j0 + p], d));
    for (int p = 0; p < n; p++) {
        const int kp = ecell[j0 + p];
        const double ap = eval[j0 + p];
        for (int q = p + lane; q < n; q += 32) {
            const int kq = ecell[j0 + q];
            const double aq = eval[j0 + q];
            // (the reference's order: the weight times the value of the lower cell, times the other)
            if (kp <= kq) atomicAdd(G + (size_t)kp * ncell + kq, __dmul_rn(__dmul_rn(w, ap), aq));
            else atomicAdd(G + (size_t)kq * ncell + kp, __dmul_rn(__dmul_rn(w, aq), ap));
        }
    }
}

// G[l, k] = G[k, l] for l > k
__global__ void __launch_bounds__(256) k_wind_sym(double *__restrict__ G, int n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * n) return;
    const int r = (int)(i / n), c = (int)(i - (long long)r * n);
    if (r > c) G[i] = G[(size_t)c * n + r];
}

// bbarolo/windmodel.py:584-602: out (nz, ny, nx) += amp[k] A_k (one CTA row block per column, float64 atomics)
__global__ void __launch_bounds__(256) k_wind_scatter(const double *__restrict__ buf, const long long *__restrict__ offs,
                                                      const long long *__restrict__ box,
                                                      const double *__restrict__ amp, int ny, int nx,
                                                      double *__restrict__ out) {
    const int k = blockIdx.x;
    const double a = amp[k];
    if (a == 0. || offs[k + 1] == offs[k]) return;
    const long long *B = box + 6 * (size_t)k;
    const int bx = (int)(B[1] - B[0]), by = (int)(B[3] - B[2]), bz = (int)(B[5] - B[4]);
    const int lane = threadIdx.x & 31, nw = (blockDim.x >> 5) * gridDim.y;
    const double *src = buf + offs[k];
    for (int row = (threadIdx.x >> 5) + (blockDim.x >> 5) * blockIdx.y; row < bz * by; row += nw) {
        const int zr = row / by, z = (int)B[4] + zr, y = (int)B[2] + (row - zr * by);
        double *o = out + ((size_t)z * ny + y) * nx + B[0];
        const double *r = src + (size_t)row * bx;
        for (int c = lane; c < bx; c += 32) {
            const double v = r[c];
            if (v != 0.) atomicAdd(o + c, __dmul_rn(a, v));
        }
    }
}

unsigned grid_of(long long n, int per) {
    return (unsigned)((n + per - 1) / per);
}

int fail(bbgpu_wind *w, int code, const std::string &msg) {
    w->err = msg;
    return code;
}

int cuda_check(bbgpu_wind *w, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return BBGPU_OK;
    return fail(w, BBGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
int grow(bbgpu_wind *w, T **p, size_t &cap, size_t n) {
    if (n <= cap && *p) return BBGPU_OK;
    cudaFree(*p);
    *p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(n + n / 4, 1024);
    if (cudaMalloc((void **)p, sizeof(T) * want) != cudaSuccess) {
        cudaGetLastError();
        return fail(w, BBGPU_ERR_NOMEM, "device allocation failed");
    }
    cap = want;
    return BBGPU_OK;
}

}  // namespace

// PHI table (bbarolo/galmod.py:176-180) for the wind engine: 0.5 erfc(-t/sqrt 2) at t = -6 + k/512
static void wind_phi_table(std::vector<double> &t) {
    t.resize(WIND_PHI_N);
    for (int k = 0; k < WIND_PHI_N; k++) t[k] = 0.5 * erfc(-(-6.0 + k / 512.0) / sqrt(2.0));
}

extern "C" int bbgpu_wind_create(bbgpu_wind **out, int device, const bbgpu_wind_grid *g, const double *lfreq0,
                                 const double *relint, const double *vedges, const double *kern, int hy, int hx,
                                 const double *kx, const double *ky, int separable) {
    if (!out || !g || !lfreq0 || !relint || !vedges || !kern) return BBGPU_ERR_ARG;
    *out = nullptr;
    if (g->nx < 1 || g->ny < 1 || g->nz < 1 || g->nlines < 1 || g->nlines > WIND_MAXL || hx < 0 || hy < 0 ||
        hx > 255 || hy > 255 || !(g->chmin > 0) || g->cdelt0 == 0 || g->cdelt1 == 0 || g->cdelt3 == 0 ||
        (long long)g->nx * g->ny * g->nz >= (1LL << 31))
        return BBGPU_ERR_ARG;
    if (separable && (!kx || !ky)) return BBGPU_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return BBGPU_ERR_CUDA;
    bbgpu_wind *w = new bbgpu_wind();
    w->device = device;
    WindGridDev &d = w->g;
    d.nx = g->nx; d.ny = g->ny; d.nz = g->nz; d.nlines = g->nlines; d.axtyp = g->axtyp; d.velsys = g->velsys;
    d.cd0 = g->cdelt0; d.cd1 = g->cdelt1; d.sig_instr = g->sig_instr; d.chmin = g->chmin;
    d.crval3 = g->crval3; d.cdelt3 = g->cdelt3; d.crpix3 = g->crpix3;
    for (int i = 0; i < g->nlines; i++) {
        d.lfreq0[i] = lfreq0[i];
        d.relint[i] = relint[i];
    }
    w->hx = hx;
    w->hy = hy;
    w->separable = separable ? 1 : 0;
    std::vector<double> ptab;
    wind_phi_table(ptab);
    const size_t nk = (size_t)(2 * hy + 1) * (2 * hx + 1), ne = (size_t)g->nlines * (g->nz + 1);
    bool ok = cudaStreamCreateWithFlags(&w->s, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&w->d_kern, sizeof(float2) * nk) == cudaSuccess &&
              cudaMalloc(&w->d_kx, sizeof(float2) * (2 * hx + 1)) == cudaSuccess &&
              cudaMalloc(&w->d_ky, sizeof(float2) * (2 * hy + 1)) == cudaSuccess &&
              cudaMalloc(&w->d_vedges, sizeof(double) * ne) == cudaSuccess &&
              cudaMalloc(&w->d_ptab, sizeof(double) * WIND_PHI_N) == cudaSuccess &&
              cudaMalloc(&w->d_rad, sizeof(double) * 4 * WIND_MAXRAD) == cudaSuccess;
    auto split = [](const double *v, size_t n) {
        std::vector<float2> o(n);
        for (size_t i = 0; i < n; i++) {
            const float h = (float)v[i];
            o[i] = make_float2(h, (float)(v[i] - (double)h));
        }
        return o;
    };
    const std::vector<float2> k2 = split(kern, nk);
    const std::vector<float2> kx2 = separable ? split(kx, 2 * hx + 1) : std::vector<float2>(2 * hx + 1);
    const std::vector<float2> ky2 = separable ? split(ky, 2 * hy + 1) : std::vector<float2>(2 * hy + 1);
    ok = ok && cudaMemcpy(w->d_kern, k2.data(), sizeof(float2) * nk, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(w->d_vedges, vedges, sizeof(double) * ne, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(w->d_ptab, ptab.data(), sizeof(double) * WIND_PHI_N, cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && separable)
        ok = cudaMemcpy(w->d_kx, kx2.data(), sizeof(float2) * (2 * hx + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(w->d_ky, ky2.data(), sizeof(float2) * (2 * hy + 1), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        bbgpu_wind_destroy(w);
        return BBGPU_ERR_NOMEM;
    }
    if (cudaFuncSetAttribute(k_wind_deposit_cell, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(unsigned long long) * WIND_SMEM_VALS)) != cudaSuccess ||
        cudaFuncSetAttribute(k_wind_points_cell, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double) * WIND_SMEM_VALS)) != cudaSuccess) {
        cudaGetLastError();
        bbgpu_wind_destroy(w);
        return BBGPU_ERR_CUDA;
    }
    *out = w;
    return BBGPU_OK;
}

static void free_cells(bbgpu_wind *w) {
    void *ps[] = {w->d_cells, w->d_qn, w->d_qoff, w->d_pcell, w->d_gx, w->d_gy, w->d_vel, w->d_sig, w->d_w,
                  w->d_rr, w->d_vol, w->d_rbar, w->d_weight, w->d_rbox, w->d_box, w->d_roffs, w->d_offs,
                  w->d_toffs, w->d_thr, w->d_G, w->d_b, w->d_bexp};
    for (void *p : ps) cudaFree(p);
    w->d_cells = nullptr; w->d_qn = nullptr; w->d_qoff = nullptr; w->d_pcell = nullptr;
    w->d_gx = w->d_gy = w->d_vel = w->d_sig = w->d_w = w->d_rr = w->d_vol = w->d_rbar = w->d_weight = nullptr;
    w->d_rbox = w->d_box = w->d_roffs = w->d_offs = w->d_toffs = nullptr;
    w->d_thr = w->d_G = w->d_b = nullptr;
    w->d_bexp = nullptr;
    w->ncell = 0;
    w->npts = 0;
    w->have_points = w->have_boxes = false;
}

extern "C" int bbgpu_wind_destroy(bbgpu_wind *w) {
    if (!w) return BBGPU_ERR_ARG;
    cudaSetDevice(w->device);
    if (w->s) cudaStreamSynchronize(w->s);
    free_cells(w);
    void *ps[] = {w->d_kern, w->d_kx, w->d_ky, w->d_vedges, w->d_ptab, w->d_rad, w->d_rbuf, w->d_buf, w->d_tmp,
                  w->d_rff,
                  w->d_W, w->d_Wd, w->d_out, w->d_cnt, w->d_start, w->d_cursor, w->d_scan, w->d_ecell, w->d_eval};
    for (void *p : ps) cudaFree(p);
    if (w->s) cudaStreamDestroy(w->s);
    delete w;
    return BBGPU_OK;
}

extern "C" const char *bbgpu_wind_last_error(const bbgpu_wind *w) {
    return w ? w->err.c_str() : "null handle";
}

extern "C" int64_t bbgpu_wind_launch_count(const bbgpu_wind *w) {
    return w ? w->launches : -1;
}

extern "C" int bbgpu_wind_set_cells(bbgpu_wind *w, int ncell, const double *cells, const int64_t *qn,
                                    const int64_t *qoff) {
    if (!w || ncell < 1 || ncell > WIND_MAXCELL || !cells || !qn || !qoff) return BBGPU_ERR_ARG;
    if (qoff[0] != 0) return fail(w, BBGPU_ERR_ARG, "qoff[0] must be 0");
    std::vector<int4> q(ncell);
    for (int k = 0; k < ncell; k++) {
        const int64_t a = qn[3 * k], b = qn[3 * k + 1], c = qn[3 * k + 2];
        if (a < 1 || b < 1 || c < 1 || a > (1 << 20) || b > (1 << 20) || c > (1 << 20) ||
            qoff[k + 1] - qoff[k] != a * b * c)
            return fail(w, BBGPU_ERR_ARG, "the quadrature counts of a cell do not match its offsets");
        q[k] = make_int4((int)a, (int)b, (int)c, 0);
        if (cells[7 * (size_t)k] != 1.0 && cells[7 * (size_t)k] != -1.0)
            return fail(w, BBGPU_ERR_ARG, "the cone of a cell must be 1 or -1");
    }
    const long long np = qoff[ncell];
    if (np < 1 || np > (1LL << 31) - 1) return fail(w, BBGPU_ERR_ARG, "quadrature points out of range");
    std::vector<int> pc(np);
    for (int k = 0; k < ncell; k++)
        for (long long i = qoff[k]; i < qoff[k + 1]; i++) pc[i] = k;
    cudaSetDevice(w->device);
    cudaStreamSynchronize(w->s);
    free_cells(w);
    const size_t n = (size_t)np;
    bool ok = cudaMalloc(&w->d_cells, sizeof(double) * 7 * ncell) == cudaSuccess &&
              cudaMalloc(&w->d_qn, sizeof(int4) * ncell) == cudaSuccess &&
              cudaMalloc(&w->d_qoff, sizeof(long long) * (ncell + 1)) == cudaSuccess &&
              cudaMalloc(&w->d_pcell, sizeof(int) * n) == cudaSuccess;
    double **pts[] = {&w->d_gx, &w->d_gy, &w->d_vel, &w->d_sig, &w->d_w, &w->d_rr, &w->d_weight};
    for (double **p : pts) ok = ok && cudaMalloc(p, sizeof(double) * n) == cudaSuccess;
    ok = ok && cudaMalloc(&w->d_vol, sizeof(double) * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_rbar, sizeof(double) * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_thr, sizeof(double) * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_bexp, sizeof(int) * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_b, sizeof(double) * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_G, sizeof(double) * ncell * (size_t)ncell) == cudaSuccess;
    ok = ok && cudaMalloc(&w->d_rbox, sizeof(long long) * 6 * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_box, sizeof(long long) * 6 * ncell) == cudaSuccess &&
         cudaMalloc(&w->d_roffs, sizeof(long long) * (ncell + 1)) == cudaSuccess &&
         cudaMalloc(&w->d_offs, sizeof(long long) * (ncell + 1)) == cudaSuccess &&
         cudaMalloc(&w->d_toffs, sizeof(long long) * (ncell + 1)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_cells(w);
        return fail(w, BBGPU_ERR_NOMEM, "device allocation of the cells failed");
    }
    ok = cudaMemcpy(w->d_cells, cells, sizeof(double) * 7 * ncell, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(w->d_qn, q.data(), sizeof(int4) * ncell, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(w->d_qoff, qoff, sizeof(long long) * (ncell + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(w->d_pcell, pc.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        free_cells(w);
        return fail(w, BBGPU_ERR_CUDA, "upload of the cells failed");
    }
    w->ncell = ncell;
    w->npts = np;
    w->tabmax = 0;
    for (int k = 0; k < ncell; k++) w->tabmax = std::max(w->tabmax, 5 * q[k].x + 2 * q[k].y + 2 * q[k].z);
    w->h_rbox.assign(6 * (size_t)ncell, 0);
    w->h_box.assign(6 * (size_t)ncell, 0);
    w->h_offs.assign(ncell + 1, 0);
    w->h_roffs.assign(ncell + 1, 0);
    w->h_toffs.assign(ncell + 1, 0);
    return BBGPU_OK;
}

static int download_points(bbgpu_wind *w, double *gx, double *gy, double *vel, double *sig, double *wt, double *r,
                           double *vol, double *rbar) {
    const size_t n = sizeof(double) * (size_t)w->npts, c = sizeof(double) * (size_t)w->ncell;
    struct { double *h; double *d; size_t b; } cp[] = {{gx, w->d_gx, n}, {gy, w->d_gy, n}, {vel, w->d_vel, n},
                                                       {sig, w->d_sig, n}, {wt, w->d_w, n}, {r, w->d_rr, n},
                                                       {vol, w->d_vol, c}, {rbar, w->d_rbar, c}};
    for (auto &e : cp)
        if (e.h) {
            int rc = cuda_check(w, cudaMemcpyAsync(e.h, e.d, e.b, cudaMemcpyDeviceToHost, w->s), "points download");
            if (rc) return rc;
        }
    return cuda_check(w, cudaStreamSynchronize(w->s), "points");
}

extern "C" int bbgpu_wind_points(bbgpu_wind *w, const bbgpu_wind_pars *p, int nrad, const double *radii,
                                 const double *vwind, const double *vdisp, const double *vrot, double *gx, double *gy,
                                 double *vel, double *sig, double *wt, double *r, double *vol, double *rbar) {
    if (!w || !p || nrad < 1 || nrad > WIND_MAXRAD || !radii || !vwind || !vdisp || !vrot) return BBGPU_ERR_ARG;
    if (!w->ncell) return fail(w, BBGPU_ERR_STATE, "no cells (bbgpu_wind_set_cells)");
    for (int i = 1; i < nrad; i++)
        if (!(radii[i] > radii[i - 1])) return fail(w, BBGPU_ERR_ARG, "the radii must be increasing");
    cudaSetDevice(w->device);
    std::vector<double> rad(4 * (size_t)nrad);
    for (int i = 0; i < nrad; i++) {
        rad[i] = radii[i];
        rad[nrad + i] = vwind[i];
        rad[2 * nrad + i] = vdisp[i];
        rad[3 * nrad + i] = vrot[i];
    }
    int rc = cuda_check(w, cudaMemcpyAsync(w->d_rad, rad.data(), sizeof(double) * rad.size(), cudaMemcpyHostToDevice,
                                           w->s), "radii upload");
    if (rc) return rc;
    WindParsDev d{p->x0, p->y0, p->vsys, p->sinc, p->cinc, p->spa, p->cpa, p->th_in, p->th_out, p->rmax, nrad};
    if (w->tabmax <= WIND_SMEM_VALS)        // (the sample tables fit in shared memory: one CTA per cell)
        k_wind_points_cell<<<w->ncell, 256, sizeof(double) * w->tabmax, w->s>>>(
            w->d_cells, w->d_qn, w->d_qoff, d, w->d_rad, w->g, w->d_gx, w->d_gy, w->d_vel, w->d_sig, w->d_w, w->d_rr);
    else
        k_wind_points<<<grid_of(w->npts, 256), 256, 0, w->s>>>(w->d_cells, w->d_qn, w->d_qoff, w->d_pcell, w->npts,
                                                                d, w->d_rad, w->g, w->d_gx, w->d_gy, w->d_vel,
                                                                w->d_sig, w->d_w, w->d_rr);
    k_wind_cells<<<grid_of((long long)w->ncell * 32, 256), 256, 0, w->s>>>(w->d_cells, w->d_qoff, w->ncell, d, w->d_w,
                                                                          w->d_rr, w->d_vol, w->d_rbar);
    w->launches += 2;
    rc = cuda_check(w, cudaGetLastError(), "k_wind_points");
    if (rc) return rc;
    // the rad upload reads a host vector that goes out of scope: wait for it before returning
    rc = cuda_check(w, cudaStreamSynchronize(w->s), "points");
    if (rc) return rc;
    w->have_points = true;               // (the columns of the last bbgpu_wind_boxes stay valid)
    if (gx || gy || vel || sig || wt || r || vol || rbar) return download_points(w, gx, gy, vel, sig, wt, r, vol, rbar);
    return BBGPU_OK;
}

extern "C" int bbgpu_wind_set_points(bbgpu_wind *w, const double *gx, const double *gy, const double *vel,
                                     const double *sig, const double *wt) {
    if (!w || !gx || !gy || !vel || !sig || !wt) return BBGPU_ERR_ARG;
    if (!w->ncell) return fail(w, BBGPU_ERR_STATE, "no cells (bbgpu_wind_set_cells)");
    cudaSetDevice(w->device);
    const size_t n = sizeof(double) * (size_t)w->npts;
    struct { const double *h; double *d; } cp[] = {{gx, w->d_gx}, {gy, w->d_gy}, {vel, w->d_vel}, {sig, w->d_sig},
                                                   {wt, w->d_w}};
    for (auto &e : cp) {
        int rc = cuda_check(w, cudaMemcpyAsync(e.d, e.h, n, cudaMemcpyHostToDevice, w->s), "points upload");
        if (rc) return rc;
    }
    int rc = cuda_check(w, cudaStreamSynchronize(w->s), "points upload");
    if (rc) return rc;
    w->have_points = true;               // (the columns of the last bbgpu_wind_boxes stay valid)
    return BBGPU_OK;
}

extern "C" int bbgpu_wind_boxes(bbgpu_wind *w, const int64_t *lim, const double *weight, int64_t *boxes,
                                int64_t *total) {
    if (!w || !lim) return BBGPU_ERR_ARG;
    if (!w->have_points) return fail(w, BBGPU_ERR_STATE, "no points (bbgpu_wind_points or bbgpu_wind_set_points)");
    if (lim[0] > lim[1] || lim[2] > lim[3] || lim[4] > lim[5] || lim[0] < 0 || lim[2] < 0 || lim[4] < 0 ||
        lim[1] > w->g.nx || lim[3] > w->g.ny || lim[5] > w->g.nz)
        return fail(w, BBGPU_ERR_ARG, "lim must lie within the cube");
    cudaSetDevice(w->device);
    w->have_boxes = false;                  // (until these columns are complete)
    const int n = w->ncell, hx = w->hx, hy = w->hy;
    int rc;
    const double *wt = nullptr;
    if (weight) {
        rc = cuda_check(w, cudaMemcpyAsync(w->d_weight, weight, sizeof(double) * (size_t)w->npts,
                                           cudaMemcpyHostToDevice, w->s), "weight upload");
        if (rc) return rc;
        wt = w->d_weight;
    }
    const WindLim rl{lim[0] - hx, lim[1] + hx, lim[2] - hy, lim[3] + hy, lim[4], lim[5]};
    k_wind_rawbox<<<grid_of((long long)n * 32, 256), 256, 0, w->s>>>(w->d_qoff, n, w->d_gx, w->d_gy, w->d_vel,
                                                                     w->d_sig, w->d_w, wt, w->g, rl, w->d_rbox);
    w->launches++;
    rc = cuda_check(w, cudaGetLastError(), "k_wind_rawbox");
    if (!rc) rc = cuda_check(w, cudaMemcpyAsync(w->h_rbox.data(), w->d_rbox, sizeof(long long) * 6 * n,
                                                cudaMemcpyDeviceToHost, w->s), "boxes download");
    if (!rc) rc = cuda_check(w, cudaStreamSynchronize(w->s), "raw boxes");
    if (rc) return rc;
    // offsets of the raw boxes; the grown boxes (bbarolo/windmodel.py:846-859) and their offsets
    const long long *R = w->h_rbox.data();
    long long *B = w->h_box.data();
    const bool conv = hx > 0 || hy > 0;
    w->h_roffs[0] = w->h_offs[0] = w->h_toffs[0] = 0;
    for (int k = 0; k < n; k++) {
        const long long *r = R + 6 * (size_t)k;
        long long *b = B + 6 * (size_t)k;
        const long long rsz = std::max(0LL, (r[1] - r[0]) * (r[3] - r[2]) * (r[5] - r[4]));
        w->h_roffs[k + 1] = w->h_roffs[k] + rsz;
        if (!conv) {
            const long long lo[6] = {lim[0], lim[0], lim[2], lim[2], lim[4], lim[4]};
            const long long hi[6] = {lim[1], lim[1], lim[3], lim[3], lim[5], lim[5]};
            for (int j = 0; j < 6; j++) b[j] = std::min(std::max(r[j], lo[j]), hi[j]);
        } else {
            b[0] = std::min(std::max(r[0] - hx, (long long)lim[0]), (long long)lim[1]);
            b[1] = std::min(std::max(r[1] + hx, (long long)lim[0]), (long long)lim[1]);
            b[2] = std::min(std::max(r[2] - hy, (long long)lim[2]), (long long)lim[3]);
            b[3] = std::min(std::max(r[3] + hy, (long long)lim[2]), (long long)lim[3]);
            b[4] = r[4];
            b[5] = r[5];
            if (r[1] <= r[0] || b[1] <= b[0] || b[3] <= b[2]) {
                b[0] = b[1] = lim[0];
                b[2] = b[3] = lim[2];
                b[4] = b[5] = lim[4];
            }
        }
        const long long sz = std::max(0LL, (b[1] - b[0]) * (b[3] - b[2]) * (b[5] - b[4]));
        w->h_offs[k + 1] = w->h_offs[k] + sz;
        const bool live = !(r[1] <= r[0] || r[3] <= r[2] || r[5] <= r[4] || b[1] <= b[0] || b[3] <= b[2] ||
                            b[5] <= b[4]);
        const long long tsz = live ? (r[5] - r[4]) * (r[3] - r[2]) * (b[1] - b[0]) : 0;
        w->h_toffs[k + 1] = w->h_toffs[k] + tsz;
    }
    const long long rtot = w->h_roffs[n], tot = conv ? w->h_offs[n] : rtot, ttot = w->h_toffs[n];
    if (!conv) w->h_offs = w->h_roffs;
    rc = grow(w, &w->d_rbuf, w->cap_rbuf, (size_t)rtot);
    if (!rc && conv) rc = grow(w, &w->d_buf, w->cap_buf, (size_t)tot);
    if (!rc && conv && w->separable) rc = grow(w, &w->d_tmp, w->cap_tmp, (size_t)ttot);
    if (!rc && conv) rc = grow(w, &w->d_rff, w->cap_rff, (size_t)rtot);
    if (rc) return rc;
    rc = cuda_check(w, cudaMemcpyAsync(w->d_box, B, sizeof(long long) * 6 * n, cudaMemcpyHostToDevice, w->s), "up");
    if (!rc) rc = cuda_check(w, cudaMemcpyAsync(w->d_roffs, w->h_roffs.data(), sizeof(long long) * (n + 1),
                                                cudaMemcpyHostToDevice, w->s), "up");
    if (!rc) rc = cuda_check(w, cudaMemcpyAsync(w->d_offs, w->h_offs.data(), sizeof(long long) * (n + 1),
                                                cudaMemcpyHostToDevice, w->s), "up");
    if (!rc) rc = cuda_check(w, cudaMemcpyAsync(w->d_toffs, w->h_toffs.data(), sizeof(long long) * (n + 1),
                                                cudaMemcpyHostToDevice, w->s), "up");
    if (rc) return rc;
    if (rtot) {
        // cells whose raw box fits in shared memory: one CTA each; the others: float64 atomics in global memory
        long long big = 0;
        for (int k = 0; k < n; k++) big = std::max(big, w->h_roffs[k + 1] - w->h_roffs[k]);
        const long long maxvals = std::min(big, (long long)WIND_SMEM_VALS);
        if (big > maxvals) {        // (the global path accumulates: its boxes start at zero; the others are written)
            rc = cuda_check(w, cudaMemsetAsync(w->d_rbuf, 0, sizeof(double) * rtot, w->s), "memset");
            if (rc) return rc;
        }
        if (maxvals > 0) {
            k_wind_deposit_cell<<<n, 512, sizeof(unsigned long long) * maxvals, w->s>>>(
                w->d_qoff, w->d_gx, w->d_gy, w->d_vel, w->d_sig, w->d_w, wt, w->d_rbox, w->d_roffs, w->d_vedges,
                w->d_ptab, w->g, maxvals, w->d_rbuf);
            w->launches++;
        }
        if (big > maxvals) {
            k_wind_deposit<<<grid_of(w->npts * 32, 256), 256, 0, w->s>>>(w->d_pcell, w->npts, w->d_gx, w->d_gy,
                                                                         w->d_vel, w->d_sig, w->d_w, wt, w->d_rbox,
                                                                         w->d_roffs, w->d_vedges, w->d_ptab, w->g,
                                                                         maxvals, w->d_rbuf);
            w->launches++;
        }
    }
    if (conv && tot) {
        const dim3 cg((unsigned)n, 4);
        k_wind_to_ff<<<n, 256, 0, w->s>>>(w->d_rbuf, w->d_roffs, w->d_rff, w->d_bexp);
        if (w->separable) {
            if (ttot)
                k_wind_conv_x<<<cg, 256, 0, w->s>>>(w->d_rff, w->d_roffs, w->d_rbox, w->d_box, w->d_toffs,
                                                    w->d_kx, hx, w->d_tmp);
            k_wind_conv_y<<<cg, 256, 0, w->s>>>(w->d_tmp, w->d_toffs, w->d_rbox, w->d_box, w->d_offs, w->d_bexp,
                                                w->d_ky, hy, w->d_buf);
            w->launches += 3;
        } else {
            k_wind_conv_2d<<<cg, 256, 0, w->s>>>(w->d_rff, w->d_roffs, w->d_rbox, w->d_box, w->d_offs, w->d_bexp,
                                                 w->d_kern, hy, hx, w->d_buf);
            w->launches += 2;
        }
    }
    rc = cuda_check(w, cudaGetLastError(), "wind deposit/convolution");
    if (rc) return rc;
    w->total = tot;
    w->have_boxes = true;
    if (boxes) std::copy(B, B + 6 * (size_t)n, boxes);
    if (total) *total = tot;
    return BBGPU_OK;
}

static const double *columns_ptr(const bbgpu_wind *w) {
    return (w->hx > 0 || w->hy > 0) ? w->d_buf : w->d_rbuf;
}

extern "C" int bbgpu_wind_columns(bbgpu_wind *w, double *buf, int64_t *offs) {
    if (!w) return BBGPU_ERR_ARG;
    if (!w->have_boxes) return fail(w, BBGPU_ERR_STATE, "no columns (bbgpu_wind_boxes)");
    cudaSetDevice(w->device);
    if (offs) std::copy(w->h_offs.begin(), w->h_offs.end(), offs);
    int rc = BBGPU_OK;
    if (buf && w->total)
        rc = cuda_check(w, cudaMemcpyAsync(buf, columns_ptr(w), sizeof(double) * (size_t)w->total,
                                           cudaMemcpyDeviceToHost, w->s), "columns download");
    if (!rc) rc = cuda_check(w, cudaStreamSynchronize(w->s), "columns");
    return rc;
}

extern "C" int bbgpu_wind_set_weights(bbgpu_wind *w, const double *wm, const double *wd) {
    if (!w || !wm || !wd) return BBGPU_ERR_ARG;
    cudaSetDevice(w->device);
    const size_t n = (size_t)w->g.nx * w->g.ny * w->g.nz;
    if (!w->d_W) {
        if (cudaMalloc(&w->d_W, sizeof(double) * n) != cudaSuccess ||
            cudaMalloc(&w->d_Wd, sizeof(double) * n) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(w->d_W);
            w->d_W = nullptr;
            return fail(w, BBGPU_ERR_NOMEM, "device allocation of the weights failed");
        }
    }
    int rc = cuda_check(w, cudaMemcpyAsync(w->d_W, wm, sizeof(double) * n, cudaMemcpyHostToDevice, w->s), "W");
    if (!rc) rc = cuda_check(w, cudaMemcpyAsync(w->d_Wd, wd, sizeof(double) * n, cudaMemcpyHostToDevice, w->s), "Wd");
    if (!rc) rc = cuda_check(w, cudaStreamSynchronize(w->s), "weights");
    if (!rc) w->have_weights = true;
    return rc;
}

extern "C" int bbgpu_wind_normal(bbgpu_wind *w, const int64_t *lim, double rel, double *G, double *b) {
    if (!w || !(rel >= 0.)) return BBGPU_ERR_ARG;
    if (!w->have_boxes) return fail(w, BBGPU_ERR_STATE, "no columns (bbgpu_wind_boxes)");
    if (!w->have_weights) return fail(w, BBGPU_ERR_STATE, "no weights (bbgpu_wind_set_weights)");
    cudaSetDevice(w->device);
    const int n = w->ncell;
    const int64_t cube[6] = {0, w->g.nx, 0, w->g.ny, 0, w->g.nz};
    if (!lim) lim = cube;
    if (lim[0] < 0 || lim[2] < 0 || lim[4] < 0 || lim[1] > w->g.nx || lim[3] > w->g.ny || lim[5] > w->g.nz ||
        lim[0] > lim[1] || lim[2] > lim[3] || lim[4] > lim[5])
        return fail(w, BBGPU_ERR_ARG, "lim must lie within the cube");
    for (int k = 0; k < n; k++) {
        const long long *B = w->h_box.data() + 6 * (size_t)k;
        if (B[1] <= B[0] || B[3] <= B[2] || B[5] <= B[4]) continue;
        if (B[0] < lim[0] || B[1] > lim[1] || B[2] < lim[2] || B[3] > lim[3] || B[4] < lim[4] || B[5] > lim[5])
            return fail(w, BBGPU_ERR_ARG, "the columns reach outside lim");
    }
    const WindLim L{lim[0], lim[1], lim[2], lim[3], lim[4], lim[5]};
    const long long nvox = (lim[1] - lim[0]) * (lim[3] - lim[2]) * (lim[5] - lim[4]);
    if (w->total >= (1LL << 31)) return fail(w, BBGPU_ERR_ARG, "more than 2^31 column values");
    const double *buf = columns_ptr(w);
    int rc = grow(w, &w->d_cnt, w->cap_cnt, (size_t)nvox + 1);
    if (!rc) rc = grow(w, &w->d_start, w->cap_start, (size_t)nvox + 1);
    if (!rc) rc = grow(w, &w->d_cursor, w->cap_cursor, (size_t)nvox + 1);
    if (!rc) rc = grow(w, &w->d_scan, w->cap_scan, (size_t)(nvox + 1023) / 1024 + 1);
    if (!rc) rc = grow(w, &w->d_ecell, w->cap_ecell, (size_t)w->total + 1);
    if (!rc) rc = grow(w, &w->d_eval, w->cap_eval, (size_t)w->total + 1);
    if (rc) return rc;
    rc = cuda_check(w, cudaMemsetAsync(w->d_G, 0, sizeof(double) * n * (size_t)n, w->s), "memset G");
    if (!rc) rc = cuda_check(w, cudaMemsetAsync(w->d_b, 0, sizeof(double) * n, w->s), "memset b");
    if (!rc) rc = cuda_check(w, cudaMemsetAsync(w->d_cnt, 0, sizeof(int) * (size_t)nvox, w->s), "memset counts");
    if (!rc && rel == 0.) rc = cuda_check(w, cudaMemsetAsync(w->d_thr, 0, sizeof(double) * n, w->s), "memset thr");
    if (rc) return rc;
    if (w->total && nvox) {
        if (rel > 0.) {
            k_wind_thr<<<n, 256, 0, w->s>>>(buf, w->d_offs, rel, w->d_thr);
            w->launches++;
        }
        k_wind_lists<<<n, 256, 0, w->s>>>(0, buf, w->d_offs, w->d_box, w->d_thr, w->d_W, w->g.ny, w->g.nx, L,
                                          w->d_cnt, nullptr, nullptr, nullptr);
        launch_scan_tiles(w->s, w->d_cnt, w->d_start, w->d_cursor, (int)nvox, w->d_scan);
        k_wind_lists<<<n, 256, 0, w->s>>>(1, buf, w->d_offs, w->d_box, w->d_thr, w->d_W, w->g.ny, w->g.nx, L,
                                          nullptr, w->d_cursor, w->d_ecell, w->d_eval);
        k_wind_lists_gram<<<grid_of(nvox * 32, 256), 256, 0, w->s>>>(w->d_cnt, w->d_start, w->d_ecell, w->d_eval,
                                                                      (int)nvox, w->d_W, w->d_Wd, w->g.ny, w->g.nx,
                                                                      L, n, w->d_G, w->d_b);
        k_wind_sym<<<grid_of((long long)n * n, 256), 256, 0, w->s>>>(w->d_G, n);
        w->launches += 7;
    }
    rc = cuda_check(w, cudaGetLastError(), "wind normal equations");
    if (!rc && G) rc = cuda_check(w, cudaMemcpyAsync(G, w->d_G, sizeof(double) * n * (size_t)n,
                                                     cudaMemcpyDeviceToHost, w->s), "G download");
    if (!rc && b) rc = cuda_check(w, cudaMemcpyAsync(b, w->d_b, sizeof(double) * n, cudaMemcpyDeviceToHost, w->s),
                                  "b download");
    if (!rc) rc = cuda_check(w, cudaStreamSynchronize(w->s), "normal equations");
    return rc;
}

extern "C" int bbgpu_wind_model(bbgpu_wind *w, const double *amp, double *out) {
    if (!w || !amp || !out) return BBGPU_ERR_ARG;
    if (!w->have_boxes) return fail(w, BBGPU_ERR_STATE, "no columns (bbgpu_wind_boxes)");
    cudaSetDevice(w->device);
    const size_t nv = (size_t)w->g.nx * w->g.ny * w->g.nz;
    int rc = grow(w, &w->d_out, w->cap_out, nv + w->ncell);
    if (rc) return rc;
    double *d_amp = w->d_out + nv;
    rc = cuda_check(w, cudaMemcpyAsync(d_amp, amp, sizeof(double) * w->ncell, cudaMemcpyHostToDevice, w->s), "a");
    if (!rc) rc = cuda_check(w, cudaMemsetAsync(w->d_out, 0, sizeof(double) * nv, w->s), "memset");
    if (rc) return rc;
    if (w->total) {
        k_wind_scatter<<<dim3((unsigned)w->ncell, 4), 256, 0, w->s>>>(columns_ptr(w), w->d_offs, w->d_box, d_amp,
                                                                       w->g.ny, w->g.nx, w->d_out);
        w->launches++;
    }
    rc = cuda_check(w, cudaGetLastError(), "k_wind_scatter");
    if (!rc) rc = cuda_check(w, cudaMemcpyAsync(out, w->d_out, sizeof(double) * nv, cudaMemcpyDeviceToHost, w->s),
                             "model download");
    if (!rc) rc = cuda_check(w, cudaStreamSynchronize(w->s), "model");
    return rc;
}
