// Host set-up of the bbgpu runtime: random-stream layouts of the MC model and the per-sub-ring constants.
//
// Compiled with -ffp-contract=off: the float64 expressions below round exactly as the reference's
// (bbarolo/galmod.py), and its transcendental functions are the C library's, as numba's.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/bbgpu.h"
#include "internal.h"

#include <unordered_map>

// sin and cos of an angle from the C library, remembered per value: a batch repeats the inclinations and
// position angles of its members' sub-rings (the values are the library's, computed once each).
static void sincos_memo(double x, double &s, double &c) {
    thread_local std::unordered_map<uint64_t, std::pair<double, double>> memo;
    uint64_t key;
    memcpy(&key, &x, sizeof key);
    auto it = memo.find(key);
    if (it != memo.end()) {
        s = it->second.first;
        c = it->second.second;
        return;
    }
    s = sin(x);
    c = cos(x);
    if (memo.size() > 65536) memo.clear();
    memo.emplace(key, std::make_pair(s, c));
}

namespace {

// ---------------------------------------------------------------- ziggurat tables (bbarolo/_rng.py:17-38)
struct Zig {
    int64_t kn[128];
    double wn[128], fn[128];
    Zig() {
        double dn = 3.442619855899, tn = dn;
        const double vn = 9.91256303526217e-3, m1 = 2147483648.0;
        const double q = vn / exp(-.5 * dn * dn);
        kn[0] = (int64_t)((dn / q) * m1);
        kn[1] = 0;
        wn[0] = q / m1;
        wn[127] = dn / m1;
        fn[0] = 1.;
        fn[127] = exp(-.5 * dn * dn);
        for (int i = 126; i >= 1; i--) {
            dn = sqrt(-2. * log(vn / dn + exp(-.5 * dn * dn)));
            kn[i + 1] = (int64_t)((dn / tn) * m1);
            tn = dn;
            fn[i] = exp(-.5 * dn * dn);
            wn[i] = dn / m1;
        }
    }
};
const Zig &zig() {
    static Zig z;
    return z;
}

// ---------------------------------------------------------------- the stream (bbarolo/_rng.py:49-100)
struct Stream {
    uint64_t s0, s1;
    explicit Stream(uint64_t seed) {
        // splitmix64 seeding: two outputs of the splitmix sequence started at seed + golden gamma
        uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
        uint64_t out[2];
        for (int i = 0; i < 2; i++) {
            z += 0x9E3779B97F4A7C15ULL;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
            out[i] = x ^ (x >> 31);
        }
        s0 = out[0];
        s1 = out[1];
        if (s0 == 0 && s1 == 0) s0 = 1;
    }
    inline uint64_t next() {   // xoroshiro128+
        uint64_t a = s0, b = s1, r = a + b;
        b ^= a;
        s0 = ((a << 24) | (a >> 40)) ^ b ^ (b << 16);
        s1 = (b << 37) | (b >> 27);
        return r;
    }
    inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // Ziggurat normal. first_hz: the high word (minus 2^31) of its first draw; slow: it did not take the
    // one-draw path (its value must then be recorded).
    inline double normal(int32_t *first_hz, bool *slow) {
        const Zig &Z = zig();
        bool first = true;
        *slow = false;
        for (;;) {
            int64_t hz = (int64_t)(next() >> 32) - 2147483648LL;
            if (first) { *first_hz = (int32_t)hz; first = false; }
            int64_t iz = hz & 127;
            int64_t ahz = hz < 0 ? -hz : hz;
            if (ahz < Z.kn[iz]) return (double)hz * Z.wn[iz];
            *slow = true;
            double x = (double)hz * Z.wn[iz];
            if (iz == 0) {
                double xx, yy;
                for (;;) {
                    xx = -log(1.0 - uniform()) * 0.2904764;
                    yy = -log(1.0 - uniform());
                    if (yy + yy >= xx * xx) break;
                }
                return hz > 0 ? 3.442620 + xx : -3.442620 - xx;
            }
            if (Z.fn[iz] + uniform() * (Z.fn[iz - 1] - Z.fn[iz]) < exp(-.5 * x * x)) return x;
        }
    }
    inline double normal() {
        int32_t h;
        bool s;
        return normal(&h, &s);
    }
};

inline int64_t lround_ref(double x) {   // bbarolo/galmod.py:38-46
    if (!(fabs(x) < 1e18)) return -((int64_t)1 << 62);
    if (x >= 0) return (int64_t)(x + 0.5);
    return -(int64_t)(-x + 0.5);
}

// layer deviate (bbarolo/galmod.py:76-89)
inline double layer_deviate(int ltype, Stream &st) {
    if (ltype == 1) return st.normal();
    double x = 2.0 * st.uniform() - 1.0;
    if (ltype == 2) return atanh(x);
    if (ltype == 3) return x >= 0.0 ? -log(x) : log(-x);
    if (ltype == 4) return tan(0.5 * M_PI * x);
    return x;
}

template <class T>
T *dup(const std::vector<T> &v) {
    T *p = (T *)malloc(sizeof(T) * (v.size() ? v.size() : 1));
    if (p && !v.empty()) memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
}

}  // namespace

void bbh_zig_tables(int64_t *kn, double *wn, double *fn) {
    const Zig &Z = zig();
    memcpy(kn, Z.kn, sizeof Z.kn);
    memcpy(wn, Z.wn, sizeof Z.wn);
    memcpy(fn, Z.fn, sizeof Z.fn);
}

// Phi(t) on the 1/512 grid of bbarolo/galmod.py:176-180
void bbh_phi_table(double *tab) {
    for (int k = 0; k < 6146; k++) tab[k] = 0.5 * erfc(-(-6.0 + k / 512.0) / sqrt(2.0));
}

uint64_t bbh_layout_key(uint64_t seed, int ltype, int nsub, const int *nc, const int *nv, const double *R0,
                        double radsep) {
    uint64_t h = 1469598103934665603ULL;
    auto mix = [&h](const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t i = 0; i < n; i++) { h ^= c[i]; h *= 1099511628211ULL; }
    };
    mix(&seed, sizeof seed);
    mix(&ltype, sizeof ltype);
    mix(&nsub, sizeof nsub);
    mix(nc, sizeof(int) * nsub);
    mix(nv, sizeof(int) * nsub);
    mix(R0, sizeof(double) * nsub);
    mix(&radsep, sizeof radsep);
    return h;
}

// Parses the stream of _galmod_wind (bbarolo/galmod.py:546-590): per shell its cloud count and constants (each
// in the reference's float64 operation order, with the C library's sin and cos), per cloud the three uniforms
// made into its radius, azimuth (cos, sin) and polar angle (sin, cos), and its velocity deviates (the first word of
// each, and the values of the rare ones that took the ziggurat's slow path).
int bbh_wind_clouds(WindClouds *W, uint64_t seed, const double *sr, int nsub, int lo, int hi, double sep,
                    const int64_t *nv, const GridDev *g) {
    if (!W || !sr || !nv || lo < 0 || hi > nsub || lo > hi) return -1;
    *W = WindClouds();
    Stream st(seed);
    auto SRV = [&](int row, int ir) { return sr[(size_t)row * nsub + ir]; };
    auto count = [&](int ir) {
        return lround_ref(g->cdens * pow(SRV(4, ir), (double)g->cmode) * 2 * M_PI * SRV(0, ir) * sep / g->pixarea);
    };
    // (the arrays sized first: the clouds and deviates of every shell)
    size_t ncl = 0, nnrm = 0;
    for (int ir = lo; ir < hi; ir++) {
        const int64_t nc = count(ir);
        if (nc < 0 || nc > (1LL << 31) || nv[ir] < 1 || nv[ir] > (1 << 20)) return -2;
        ncl += (size_t)nc;
        nnrm += (size_t)nc * (size_t)nv[ir];
    }
    W->shell.resize(ncl);
    W->geo.resize(5 * ncl);
    W->nbase.resize(ncl);
    W->sbase.resize(ncl);
    W->hz.resize(nnrm);
    W->slow.reserve(nnrm / 50 + 16);
    size_t icl = 0, inr = 0;
    for (int ir = lo; ir < hi; ir++) {
        const double rtmp = SRV(0, ir);
        const int64_t nc = count(ir);
        if (nc == 0) continue;
        WindShell s{};
        s.vrot = SRV(1, ir);
        s.vsph = SRV(2, ir);
        const double opentmp = SRV(7, ir) / 2.;
        s.vdisp = sqrt(SRV(3, ir) * SRV(3, ir) + g->sig_instr * g->sig_instr);
        s.vsys = SRV(10, ir);
        s.sinc = sin(SRV(5, ir));
        s.cinc = cos(SRV(5, ir));
        const double pa = SRV(6, ir);
        s.spa = sin(pa) * cos(g->crota2) + cos(pa) * sin(g->crota2);
        s.cpa = cos(pa) * cos(g->crota2) - sin(pa) * sin(g->crota2);
        s.xpos = SRV(8, ir);
        s.ypos = SRV(9, ir);
        s.nvr = (int)nv[ir];
        s.fluxsc = SRV(4, ir) * 2 * M_PI * rtmp * sep / (double)(nc * nv[ir]);
        const int si = (int)W->shells.size();
        W->shells.push_back(s);
        const double r_in2 = pow(rtmp - 0.5 * sep, 2.0);
        int *shp = W->shell.data();
        double *geo = W->geo.data();
        int32_t *hz = W->hz.data();
        long long *nb = W->nbase.data(), *sb = W->sbase.data();
        for (int64_t ic = 0; ic < nc; ic++, icl++) {
            const double rad = sqrt(r_in2 + 2 * sep * rtmp * fabs(2.0 * st.uniform() - 1.0));
            const double az = 2 * M_PI * fabs(2.0 * st.uniform() - 1.0);
            double ph = opentmp * fabs(2.0 * st.uniform() - 1.0);
            if (ic % 2 == 0) ph = M_PI - ph;
            shp[icl] = si;
            double *gc = geo + 5 * icl;
            gc[0] = rad;
            gc[1] = cos(az);
            gc[2] = sin(az);
            gc[3] = sin(ph);
            gc[4] = cos(ph);
            nb[icl] = (long long)inr;
            sb[icl] = (long long)W->slow.size();
            for (int iv = 0; iv < s.nvr; iv++) {
                bool slow;
                const double v = st.normal(hz + inr++, &slow);
                if (slow) W->slow.push_back(v);
            }
        }
        W->total += (double)nc * s.nvr * fabs(s.fluxsc);
    }
    return 0;
}

// Parses the stream of _galmod_mc (bbarolo/galmod.py:100-144) for clouds counts nc and velocity samples nv
// per sub-ring: the draws are the same whatever the ring velocities, geometry and box, so each cloud's
// radius, azimuth, layer deviate and the first word of each of its normals are recorded once.
int bbh_layout_build(LayoutHost *L, uint64_t seed, int ltype, int nsub, const int *nc, const int *nv,
                     const double *R0, double radsep) {
    memset(L, 0, sizeof *L);
    L->key = bbh_layout_key(seed, ltype, nsub, nc, nv, R0, radsep);
    L->nsub = nsub;
    long long ncl = 0, nsc = 0;
    std::vector<int> vnc(nsub), vnv(nsub), vcb(nsub);
    std::vector<long long> vsb(nsub);
    for (int i = 0; i < nsub; i++) {
        vnc[i] = nc[i];
        vnv[i] = nv[i];
        vcb[i] = (int)ncl;
        vsb[i] = nsc;
        ncl += nc[i];
        nsc += (long long)nc[i] * nv[i];
    }
    if (ncl > 0x7fffffffLL) return -1;
    L->ncloud = (int)ncl;
    L->nsubcloud = nsc;
    std::vector<double> R(ncl), caz(ncl), saz(ncl), fd(ncl);
    std::vector<int> sub(ncl), slow_base(ncl);
    int32_t *hz = (int32_t *)malloc(sizeof(int32_t) * (nsc ? nsc : 1));
    if (!hz) return -1;
    std::vector<double> slow;
    slow.reserve((size_t)(nsc / 20 + 16));
    Stream st(seed);
    long long c = 0, q = 0;
    for (int ir = 0; ir < nsub; ir++) {
        if (nc[ir] <= 0) continue;
        double r_inner = R0[ir] - 0.5 * radsep;
        double r_inner_sq = r_inner * r_inner;
        double r_cross = 2.0 * radsep * R0[ir];
        for (int ic = 0; ic < nc[ir]; ic++, c++) {
            R[c] = sqrt(r_inner_sq + r_cross * fabs(2.0 * st.uniform() - 1.0));
            double az = 2 * M_PI * fabs(2.0 * st.uniform() - 1.0);
            saz[c] = sin(az);
            caz[c] = cos(az);
            fd[c] = layer_deviate(ltype, st);
            sub[c] = ir;
            slow_base[c] = (int)slow.size();
            for (int iv = 0; iv < nv[ir]; iv++, q++) {
                bool s;
                double v = st.normal(&hz[q], &s);
                if (s) slow.push_back(v);
            }
        }
    }
    L->nc = dup(vnc);
    L->nv = dup(vnv);
    L->cloud_base = dup(vcb);
    L->sub_base = dup(vsb);
    L->R = dup(R);
    L->caz = dup(caz);
    L->saz = dup(saz);
    L->fdev = dup(fd);
    L->sub = dup(sub);
    L->slow_base = dup(slow_base);
    L->hz = hz;
    L->slow_val = dup(slow);
    L->nslow = (long long)slow.size();
    return 0;
}

void bbh_layout_free(LayoutHost *L) {
    free(L->nc); free(L->nv); free(L->cloud_base); free(L->sub_base);
    free(L->R); free(L->caz); free(L->saz); free(L->fdev); free(L->sub); free(L->slow_base);
    free(L->hz); free(L->slow_val);
    memset(L, 0, sizeof *L);
}

// Cloud counts of _galmod_mc (bbarolo/galmod.py:107-114): 0 for the sub-rings without density.
void bbh_cloud_counts(const double *sr, int nsub, const int64_t *nv_in, const GridDev *g, int *nc, int *nv) {
    for (int ir = 0; ir < nsub; ir++) {
        double R0 = sr[0 * nsub + ir], dens = sr[5 * nsub + ir];
        nv[ir] = (int)nv_in[ir];
        if (dens == 0) { nc[ir] = 0; continue; }
        double ring_area_pix = 2 * M_PI * R0 * g->radsep / g->pixarea;
        double dp = g->cmode == 1 ? pow(dens, 1.0) : pow(dens, (double)g->cmode);
        int64_t n = lround_ref(g->cdens * dp * ring_area_pix);
        if ((double)lround_ref((double)n / ring_area_pix) < 10.) n = lround_ref(10 * ring_area_pix);
        nc[ir] = n > 0x3fffffff ? 0x3fffffff : (n < 0 ? 0 : (int)n);
    }
}

// The per-sub-ring constants of one member (bbarolo/galmod.py:111-127 and the cloud loop's invariants).
// Returns e: the deposits are fixed-point numbers in units of 2^-e.
void bbh_column_diff(const double *a, const double *b, int nsub, uint16_t *mask) {
    memset(mask, 0, sizeof(uint16_t) * (size_t)nsub);
    for (int r = 0; r < BBGPU_NSR; r++) {
        const double *x = a + (size_t)r * nsub, *y = b + (size_t)r * nsub;
        if (!memcmp(x, y, sizeof(double) * (size_t)nsub)) continue;       // (most rows of a step are equal)
        for (int i = 0; i < nsub; i++) {
            uint64_t u, v;
            memcpy(&u, x + i, 8);
            memcpy(&v, y + i, 8);
            if (u != v) mask[i] |= (uint16_t)(1u << r);
        }
    }
}

bool bbh_map_same(uint16_t m, const double *a, int nsub, int ir) {
    const unsigned rows = (1u << 0) | (1u << 6) | (1u << 7) | (1u << 9) | (1u << 10) | (1u << 11) | (1u << 12) |
                          (1u << 14) | (1u << 15);
    return !(m & rows) && (a[(size_t)7 * nsub + ir] == 0.0 || !(m & (1u << 4)));
}

// the rows that differ from the reference table's, per column (thread-local scratch), or nullptr without one
static const uint16_t *diff_of(const double *sr, const double *sr_ref, int nsub) {
    if (!sr_ref) return nullptr;
    thread_local std::vector<uint16_t> d;
    d.resize((size_t)nsub);
    bbh_column_diff(sr, sr_ref, nsub, d.data());
    return d.data();
}

int bbh_submc(const double *sr, int nsub, const int *nc, const int *nv, const GridDev *g, SubMC *out,
              const double *sr_ref, const SubMC *out_ref, signed char *reused, const uint16_t *diff_in) {
    double bound = 0.;
    const uint16_t *diff = out_ref ? (diff_in ? diff_in : diff_of(sr, sr_ref, nsub)) : nullptr;
    double scr, ccr;
    sincos_memo(g->crota2, scr, ccr);
    for (int ir = 0; ir < nsub; ir++) {
        SubMC &S = out[ir];
        if (reused) reused[ir] = 0;
        if (diff && !diff[ir]) {     // (the values of another member: same constants)
            const SubMC &T = out_ref[ir];
            if (reused) reused[ir] = 1;
            else S = T;
            if (T.active) {
                const double wmax = fmax(fabs(T.wrec), fabs(T.wapp));
                for (int nl = 0; nl < g->nlines && nl < BBGPU_MAXL; nl++)
                    bound += (double)nc[ir] * (double)nv[ir] * fabs(T.valrel[nl]) * wmax;
            }
            continue;
        }
        memset(&S, 0, sizeof S);
#define R_(row) sr[(size_t)(row) * nsub + ir]
        double R0 = R_(0), dens = R_(5);
        S.nc = nc[ir];
        S.nv = nv[ir];
        S.active = dens != 0 && nc[ir] > 0;
        if (!S.active) continue;
        double ring_area_pix = 2 * M_PI * R0 * g->radsep / g->pixarea;
        double fluxsc = (double)(float)(dens * ring_area_pix * g->pixarea / (double)((int64_t)nc[ir] * nv[ir]));
        S.vdisptmp = sqrt(R_(4) * R_(4) + g->sig_instr * g->sig_instr);
        S.vrot = R_(1); S.vrad = R_(2); S.vvert = R_(3);
        S.z0 = R_(6); S.dvdz = R_(7); S.zcyl = R_(8);
        sincos_memo(R_(9), S.sinc, S.cinc);
        double phi = R_(10);
        double sphi, cphi;
        sincos_memo(phi, sphi, cphi);
        S.spa = sphi * ccr + cphi * scr;
        S.cpa = cphi * ccr - sphi * scr;
        S.xpos = R_(11); S.ypos = R_(12); S.vsys = R_(13);
        S.wrec = R_(14); S.wapp = R_(15);
#undef R_
        double wmax = fmax(fabs(S.wrec), fabs(S.wapp));
        for (int nl = 0; nl < g->nlines && nl < BBGPU_MAXL; nl++) {
            S.valrel[nl] = g->relint[nl] * fluxsc;
            bound += (double)nc[ir] * (double)nv[ir] * fabs(S.valrel[nl]) * wmax;
        }
        // fast-path coefficients (any rounding: the error is bounded in the kernel)
        S.P1 = (float)(S.spa / g->cdelt0);
        S.P2 = (float)(S.cinc * S.cpa / g->cdelt0);
        S.P3 = (float)(S.sinc * S.cpa / g->cdelt0);
        S.Q1 = (float)(S.cpa / g->cdelt1);
        S.Q2 = (float)(S.cinc * S.spa / g->cdelt1);
        S.Q3 = (float)(-S.sinc * S.spa / g->cdelt1);
        S.xposf = (float)S.xpos;
        S.yposf = (float)S.ypos;
        for (int nl = 0; nl < g->nlines && nl < BBGPU_MAXL; nl++) {
            double ia = g->axtyp == 4 ? g->ia : (double)g->lia[nl];
            double ib = g->axtyp == 4 ? g->ib : (double)g->lib[nl];
            S.c0[nl] = (float)((S.vsys + S.vvert * S.cinc) * ia + ib);
            S.sia[nl] = (float)(S.sinc * ia);
            S.sg[nl] = (float)(S.vdisptmp * ia);
        }
        S.z0f = (float)S.z0;
        S.zcylf = (float)S.zcyl;
        S.dvdzf = (float)S.dvdz;
        S.vrotf = (float)S.vrot;
        S.vradf = (float)S.vrad;
    }
    // fixed point: every voxel sum stays below 2^62
    double Q = bound > 0 ? ldexp(1.0, (int)floor(62.0 - log2(bound))) : 1.0;
    int cb = 0;
    for (int ir = 0; ir < nsub; ir++) {
        if (reused && reused[ir]) {                              // (set on the device: k_fill_submc)
            cb += out_ref[ir].active ? out_ref[ir].nc : 0;
            continue;
        }
        SubMC &S = out[ir];
        S.cloud_base = cb;
        cb += S.active ? S.nc : 0;
        if (!S.active) continue;
        for (int nl = 0; nl < g->nlines && nl < BBGPU_MAXL; nl++) {
            S.fix[0][nl] = llrint(S.valrel[nl] * S.wrec * Q);
            S.fix[1][nl] = llrint(S.valrel[nl] * S.wapp * Q);
        }
    }
    return bound > 0 ? (int)floor(62.0 - log2(bound)) : 0;
}

// The ring footprint of _norm (bbarolo/galfit.py:62-93): the reference's float64 expressions and C library calls.
void bbh_norm_footprint(int bsy, int bsx, double x0, double y0, double phi, double inc, double r1, double r2,
                        double wpow, int side, int foot, double hmax, uint8_t *inside, double *wmap) {
    const double F = M_PI / 180.;
    const double sphi = sin(F * phi), cphi = cos(F * phi), cinc = cos(F * inc);
    const int usesin = wpow < 0;
    const double apow = fabs(wpow);
    for (int y = 0; y < bsy; y++)
        for (int x = 0; x < bsx; x++) {
            const int p = y * bsx + x;
            inside[p] = 0;
            wmap[p] = 0.0;
            const double xr = -(x - x0) * sphi + (y - y0) * cphi;
            const double ys = -(x - x0) * cphi - (y - y0) * sphi;
            const double yr = ys / cinc;
            const double r = sqrt(xr * xr + yr * yr);
            double th = r < 0.1 ? 0.0 : atan2(yr, xr) / F;
            if (foot == 1) {
                if (!(fabs(xr) >= r1 && fabs(xr) <= r2 && fabs(ys) <= hmax)) continue;
                th = xr >= 0 ? 0.0 : 180.0;
            } else if (!(r >= r1 && r <= r2)) {
                continue;
            }
            if (side == 1 && !(fabs(th) <= 90.0)) continue;
            if (side == 2 && !(fabs(th) >= 90.0)) continue;
            inside[p] = 1;
            if (foot == 1) {
                wmap[p] = 1.0;
                continue;
            }
            const double wf = usesin ? fabs(sin(th * F)) : fabs(cos(th * F));
            wmap[p] = pow(wf, apow);
        }
}

// ------------------------------------------------------------------------------------------- ANALYTIC
// The vertical layers of the ANALYTIC models (bbarolo/galmod.py:217-259): the cumulative flux below x (units
// of z0), the height beyond which less than 1e-6 of the flux remains, the height where the density falls
// below 1e-3 of its peak.
static double layer_cdf(int ltype, double x) {
    if (ltype == 1) return 0.5 * (1.0 + erf(x / sqrt(2.0)));
    if (ltype == 2) return 0.5 * (1.0 + tanh(x));
    if (ltype == 3) return x >= 0 ? 1.0 - 0.5 * exp(-x) : 0.5 * exp(x);
    if (ltype == 4) return 0.5 + atan(x) / M_PI;
    const double c = x < -1.0 ? -1.0 : (x > 1.0 ? 1.0 : x);
    return 0.5 * (c + 1.0);
}

static double layer_extent(int ltype) {
    return ltype == 1 ? 5.0 : ltype == 2 ? 7.6 : ltype == 3 ? 14.0 : ltype == 4 ? 1e30 : 1.0;
}

static double layer_core(int ltype) {
    return ltype == 1 ? 3.717 : ltype == 2 ? 4.147 : ltype == 3 ? 6.908 : ltype == 4 ? 31.61 : 1e30;
}

int bbh_zgrid(double *zq, double *wq, int nmax, int ltype, double z0, double sinc, double pixsize, double dvdz,
              double sig, double R0, double radsep, double xpos, double ypos, double cdelt0, double cdelt1,
              long long blo0, long long blo1, long long bhi0, long long bhi1, double zstep) {
    const double s = fabs(sinc);
    if (z0 <= 0 || nmax < 2 || s < 1e-6) {
        zq[0] = 0.0;
        wq[0] = 1.0;
        return 1;
    }
    const double dx = std::max(fabs((double)blo0 - 0.5 - xpos), fabs((double)bhi0 - 0.5 - xpos)) * fabs(cdelt0);
    const double dy = std::max(fabs((double)blo1 - 0.5 - ypos), fabs((double)bhi1 - 0.5 - ypos)) * fabs(cdelt1);
    const double zlim = std::min(layer_extent(ltype), (R0 + radsep + sqrt(dx * dx + dy * dy)) / (s * z0));
    double step = zstep * pixsize / (z0 * s);
    if (dvdz != 0) step = std::min(step, 0.5 * sig / (fabs(dvdz) * z0 * s));
    const double zc = layer_core(ltype);
    long long nin, nout;
    for (;;) {
        nin = std::max((long long)ceil(std::min(zc, zlim) / step), 1LL);
        nout = std::max((long long)ceil((zlim - (double)nin * step) / (4.0 * step)), 0LL);
        if (2 * (nin + nout) <= nmax) break;
        step *= 1.01 * (double)(nin + nout) / (double)(nmax / 2);
    }
    const long long half = nin + nout;
    for (long long j = 0; j < half; j++) {
        const double lo = j < nin ? (double)j * step : (double)(nin + 4 * (j - nin)) * step;
        const double hi = std::min(lo + (j < nin ? step : 4.0 * step), zlim);
        const double w = layer_cdf(ltype, hi) - layer_cdf(ltype, lo);
        zq[half + j] = 0.5 * (lo + hi);
        wq[half + j] = w;
        zq[half - 1 - j] = -0.5 * (lo + hi);
        wq[half - 1 - j] = w;
    }
    return (int)(2 * half);
}

static long long an_naz(double R0, double pixarea) {   // bbarolo/galmod.py:345-346
    const double circ_pix = 2 * M_PI * R0 / sqrt(pixarea);
    return std::max((long long)(3 * circ_pix + 0.5), 16LL);
}

void bbh_an_samples(const double *R0, int nsub, const GridDev *g, std::vector<int> &sbase, std::vector<int> &ssub,
                    std::vector<double> &cs) {
    sbase.assign(nsub + 1, 0);
    long long n = 0;
    for (int ir = 0; ir < nsub; ir++) {
        sbase[ir] = (int)n;
        n += 2 * an_naz(R0[ir], g->pixarea);
    }
    sbase[nsub] = (int)n;
    ssub.resize(n ? n : 1);
    cs.resize(2 * (n ? n : 1));
    for (int ir = 0; ir < nsub; ir++) {
        const long long naz = an_naz(R0[ir], g->pixarea);
        const double daz = 2 * M_PI / (double)naz;
        const double cd = cos(daz), sd = sin(daz);
        for (int kr = 0; kr < 2; kr++) {
            const double az0 = 2 * M_PI * (0.5 * ((kr + 1) % 2) + 0.25) / (double)naz;
            double caz = cos(az0), saz = sin(az0);
            for (long long ka = 0; ka < naz; ka++) {
                if (ka > 0) {
                    const double c2 = caz * cd - saz * sd, s2 = saz * cd + caz * sd;
                    caz = c2;
                    saz = s2;
                }
                const long long q = sbase[ir] + kr * naz + ka;
                ssub[q] = ir;
                cs[2 * q] = caz;
                cs[2 * q + 1] = saz;
            }
        }
    }
}

// The grid of _zgrid's inputs, from the cache or computed and appended to it: (offset, samples).
static std::pair<int, int> zgrid_cached(ZgridCache &zc, std::vector<double> &tz, std::vector<double> &tw, int nzq,
                                        int ltype, double z0, double sinc, double pixsize, double dvdz, double sig,
                                        double R0, double radsep, double xpos, double ypos, double cdelt0,
                                        double cdelt1, long long blo0, long long blo1, long long bhi0, long long bhi1,
                                        double zstep) {
    ZKey key;
    memset(&key, 0, sizeof key);
    if (z0 <= 0 || nzq < 2 || fabs(sinc) < 1e-6) {
        key.iv[0] = -1;
    } else {
        // (the dispersion enters the grid only with a velocity gradient)
        const double dv[] = {z0, sinc, pixsize, dvdz, dvdz != 0 ? sig : 0.0, R0, radsep, xpos, ypos, cdelt0, cdelt1,
                             zstep};
        const long long iv[] = {nzq, ltype, blo0, blo1, bhi0, bhi1};
        memcpy(key.dv, dv, sizeof dv);
        memcpy(key.iv, iv, sizeof iv);
    }
    auto it = zc.map.find(key);
    if (it != zc.map.end()) return it->second;
    const int n = bbh_zgrid(tz.data(), tw.data(), nzq, ltype, z0, sinc, pixsize, dvdz, sig, R0, radsep, xpos, ypos,
                            cdelt0, cdelt1, blo0, blo1, bhi0, bhi1, zstep);
    const std::pair<int, int> v((int)zc.zq.size(), n);
    zc.zq.insert(zc.zq.end(), tz.begin(), tz.begin() + n);
    zc.wq.insert(zc.wq.end(), tw.begin(), tw.begin() + n);
    zc.map.emplace(key, v);
    return v;
}

void bbh_an_samples_f32(const std::vector<double> &cs, std::vector<float> &csf) {
    csf.resize(cs.size());
    for (size_t q = 0; q + 1 < cs.size(); q += 2) {
        float cx = (float)cs[q];
        cx = cs[q] >= 0.0 ? fabsf(cx) : -fabsf(cx);    // (a negative value that rounds to -0 keeps its sign)
        if (cs[q] < 0.0 && cx == 0.0f) cx = -1e-30f;
        csf[q] = cx;
        csf[q + 1] = (float)cs[q + 1];
    }
}

int bbh_an_subs(const double *sr, int nsub, const GridDev *g, int nzq, int blo0, int blo1, int bhi0, int bhi1,
                const double *cd2i, int maps, const int64_t *widx, const double *wval, AnSub *out, ZgridCache &zc,
                const double *sr_ref, const AnSub *out_ref, signed char *reused, const uint16_t *diff_in) {
#define SR(r, i) sr[(size_t)(r) * nsub + (i)]
    const int nb = nzq > 1 ? nzq : 1;
    std::vector<double> tz(nb), tw(nb);
    const double pixsize = sqrt(g->pixarea);
    double cmax = 0.0, lsum = 0.0, bound = 0.0;
    for (int k = 0; k < g->nz; k++) cmax = std::max(cmax, fabs(cd2i[k]));
    for (int nl = 0; nl < g->nlines; nl++) lsum += fabs(g->relint[nl]);
    const uint16_t *diff = out_ref ? (diff_in ? diff_in : diff_of(sr, sr_ref, nsub)) : nullptr;
    double scr, ccr;
    sincos_memo(g->crota2, scr, ccr);
    for (int ir = 0; ir < nsub; ir++) {
        AnSub &S = out[ir];
        if (reused) reused[ir] = 0;
        if (diff && !diff[ir]) {     // (the values of another member: same constants)
            const AnSub &T = out_ref[ir];
            if (reused) reused[ir] = 1;
            else S = T;
            if (T.active) {
                const double ws = std::max(fabs(T.wrec), fabs(T.wapp));
                double per = lsum * cmax;
                if (maps) per = std::max(fabs(wval[2 * ir]), fabs(wval[2 * ir + 1]));
                bound += fabs(T.fluxsc) * ws * per * (double)((long long)T.naz * 2);
            }
            continue;
        }
        memset(&S, 0, sizeof S);
        S.sub = ir;
        const double R0 = SR(0, ir), dens = SR(5, ir);
        S.active = maps ? (widx[2 * ir] >= 0 || widx[2 * ir + 1] >= 0) : dens != 0;
        const double ring_area_pix = 2 * M_PI * R0 * g->radsep / g->pixarea;
        const long long naz = an_naz(R0, g->pixarea);
        const int nrad = 2;
        S.naz = (int)naz;
        S.vrot = SR(1, ir); S.vrad = SR(2, ir); S.vvert = SR(3, ir);
        const double sig = std::max(sqrt(SR(4, ir) * SR(4, ir) + g->sig_instr * g->sig_instr), 1e-6 * fabs(g->chwidth));
        S.inv = 1.0 / sig;
        S.K = (long long)(5.0 * sig / g->chwidth) + 2;
        S.z0 = SR(6, ir); S.dvdz = SR(7, ir); S.zcyl = SR(8, ir);
        sincos_memo(SR(9, ir), S.sinc, S.cinc);
        const double phi = SR(10, ir);
        double sphi, cphi;
        sincos_memo(phi, sphi, cphi);
        S.spa = sphi * ccr + cphi * scr;
        S.cpa = cphi * ccr - sphi * scr;
        S.xpos = SR(11, ir); S.ypos = SR(12, ir); S.vsys = SR(13, ir);
        S.wrec = SR(14, ir); S.wapp = SR(15, ir);
        S.zq_off = 0;
        if (S.active) {
            const std::pair<int, int> zg = zgrid_cached(zc, tz, tw, nzq, g->ltype, S.z0, S.sinc, pixsize, S.dvdz, sig,
                                                        R0, g->radsep, S.xpos, S.ypos, g->cdelt0, g->cdelt1, blo0,
                                                        blo1, bhi0, bhi1, g->zstep);
            S.zq_off = zg.first;
            S.nzz = zg.second;
        }
        S.fluxsc = maps ? ring_area_pix * g->pixarea / (double)(naz * nrad)
                        : dens * ring_area_pix * g->pixarea / (double)(naz * nrad);
        for (int nl = 0; nl < g->nlines; nl++) S.a[nl] = g->relint[nl] * S.fluxsc;
        S.zdep = 0;
        if (!maps && S.active && S.dvdz != 0 && S.nzz > 1)
            for (int kz = 0; kz < S.nzz; kz++)
                if (fabs(zc.zq[S.zq_off + kz] * S.z0) > S.zcyl) { S.zdep = 1; break; }
        const double r_inner = R0 - 0.5 * g->radsep;
        for (int kr = 0; kr < nrad; kr++) {
            const double u = (kr + 0.5) / nrad;
            S.R[kr] = sqrt(r_inner * r_inner + 2.0 * g->radsep * R0 * u);
        }
        {
            auto split = [](double v, float &hi, float &lo) {
                hi = (float)v;
                lo = (float)(v - (double)hi);
            };
            split(S.spa / g->cdelt0, S.P1, S.P1l);
            split(S.cinc * S.cpa / g->cdelt0, S.P2, S.P2l);
            split(S.sinc * S.cpa / g->cdelt0, S.P3, S.P3l);
            split(S.cpa / g->cdelt1, S.Q1, S.Q1l);
            split(S.cinc * S.spa / g->cdelt1, S.Q2, S.Q2l);
            split(-S.sinc * S.spa / g->cdelt1, S.Q3, S.Q3l);
            split(S.xpos, S.xposf, S.xposl);
            split(S.ypos, S.yposf, S.yposl);
            split(S.z0, S.z0f, S.z0l);
            split(S.R[0], S.Rf[0], S.Rl[0]);
            split(S.R[1], S.Rf[1], S.Rl[1]);
        }
        S.wzero = (S.wrec == 0.0 ? 1 : 0) | (S.wapp == 0.0 ? 2 : 0);
        S.invf = (float)S.inv;
        S.anfast = !maps && !S.zdep && g->nlines == 1 && g->fast_ok;
        {
            auto split = [](double v, float &hi, float &lo) {
                hi = (float)v;
                lo = (float)(v - (double)hi);
            };
            split(S.vsys, S.vsysh, S.vsysl);
            split(S.vrot, S.vroth, S.vrotl);
            split(S.vrad, S.vradh, S.vradl);
            split(S.vvert, S.vverth, S.vvertl);
            split(S.sinc, S.sinch, S.sincl);
            split(S.cinc, S.cinch, S.cincl);
            S.af = (float)S.a[0];
        }
        S.fluxscf = (float)S.fluxsc;
        S.wrecf = (float)S.wrec;
        S.wappf = (float)S.wapp;
        if (!S.active) continue;
        // every deposit of the sub-ring is at most |fluxsc| x |wside| x (line: sum of relint x max cd2i; map:
        // max wval) per sample, the vertical weights and the channel profile summing to at most 1
        const double ws = std::max(fabs(S.wrec), fabs(S.wapp));
        double per = lsum * cmax;
        if (maps) per = std::max(fabs(wval[2 * ir]), fabs(wval[2 * ir + 1]));
        bound += fabs(S.fluxsc) * ws * per * (double)(naz * nrad);
    }
#undef SR
    if (!std::isfinite(bound)) return -10000;
    if (bound == 0) return 0;
    int ex = 0;
    frexp(bound * 1.01, &ex);       // bound * 1.01 < 2^ex
    return std::min(62 - ex, 1000);
}

// ------------------------------------------------------------------------------------------- profile prior
// The second differences of the profile at the radii R (n: the rings then the exterior annulus), as
// bbarolo/profile.py:60-85 and :141-151: for row i (0 .. n-3) the columns lc[3i..3i+2] and weights lv[3i..3i+2];
// ord the order of the radii; near[i] when the radii around row i are closer than a quarter of the median ring
// distance d (bbarolo/profile.py:134-136); norm the sum of the squared weights of the relative prior.
static void second_differences(double d1, double d2, double *w) {
    w[0] = (1. / d1) * 2. / (d1 + d2);
    w[1] = (-1. / d1 - 1. / d2) * 2. / (d1 + d2);
    w[2] = (1. / d2) * 2. / (d1 + d2);
}

void bbh_profile_consts(const double *R, int n, int *lc, double *lv, int *ord, unsigned char *near, double *d,
                        double *norm) {
    std::vector<int> o(n);
    for (int i = 0; i < n; i++) o[i] = i;
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return R[a] < R[b]; });
    std::vector<double> Rs(n);
    for (int i = 0; i < n; i++) {
        Rs[i] = R[o[i]];
        ord[i] = o[i];
    }
    double mx = R[0], mn = R[0];
    for (int i = 1; i < n; i++) {
        mx = std::max(mx, R[i]);
        mn = std::min(mn, R[i]);
    }
    const double tiny = 1e-6 * std::max(mx - mn, 1e-300);
    // the distances between the rings (all but the last radius), sorted
    std::vector<double> rr(R, R + (n > 1 ? n - 1 : 0));
    std::sort(rr.begin(), rr.end());
    std::vector<double> dr;
    for (size_t i = 1; i < rr.size(); i++) dr.push_back(rr[i] - rr[i - 1]);
    double dmin = tiny;
    if (n > 2 && !dr.empty()) dmin = std::max(0.25 * *std::min_element(dr.begin(), dr.end()), tiny);
    double med = 0.0;
    if (!dr.empty()) {
        std::vector<double> s = dr;
        std::sort(s.begin(), s.end());
        const size_t m = s.size();
        med = m % 2 ? s[m / 2] : (s[m / 2 - 1] + s[m / 2]) / 2.0;
    }
    *d = med;
    double nrm = 0.0;
    for (int i = 1; i < n - 1; i++) {
        const double d1 = std::max(Rs[i] - Rs[i - 1], tiny), d2 = std::max(Rs[i + 1] - Rs[i], tiny);
        double w[3];
        second_differences(d1, d2, w);
        for (int a = 0; a < 3; a++) {
            lc[3 * (i - 1) + a] = o[i - 1 + a];
            lv[3 * (i - 1) + a] = w[a];
        }
        double wr[3];
        second_differences(std::max(d1, dmin), std::max(d2, dmin), wr);
        nrm += (wr[0] * wr[0] + wr[1] * wr[1]) + wr[2] * wr[2];
        const double dl = Rs[i] - Rs[i - 1], dh = Rs[i + 1] - Rs[i];
        near[i - 1] = std::min(dl, dh) < 0.25 * med;
    }
    *norm = nrm;
}

// The sub-ring tables of a batch of thin-disk ring sets on one radius grid (bbarolo/galmod.py:761-851, the
// interpolation v0 + ((v1 - v0) / dur) dr per sub-ring, constant before the first radius), in the float64
// operations and order of the reference: member 0 in full, every other member from member 0's table and the
// sub-rings next to a ring whose values differ from member 0's (the rest are member 0's values).
extern "C" int bbgpu_subrings_rows(const double *rows, int nb, int nr, int nsub, const int64_t *i1, const double *dr,
                                   const double *dseg, const uint8_t *cst, const double *radii, const double *edgew,
                                   const double *side, int64_t nvtmp, double *sr, int64_t *nv, double *ms, int nsm) {
    if (nb < 1 || nr < 2 || nsub < 1 || !rows || !i1 || !dr || !dseg || !cst || !radii || !side || !sr || !nv ||
        (ms && nsm < nsub))
        return BBGPU_ERR_ARG;
    for (int s = 0; s < nsub; s++)
        if (i1[s] < 1 || i1[s] >= nr) return BBGPU_ERR_ARG;
    constexpr int NV = 13;                     // interpolated rows 1 .. 13 of the table
    // (the ring-value row of each interpolated row, RING_KEYS order, and its transform)
    static const int src[NV] = {4, 6, 7, 5, 10, 11, 8, 9, 12, 13, 1, 2, 3};
    const double d2r = 3.141592653589793 / 180.0;
    std::vector<double> V0((size_t)NV * nr), V((size_t)NV * nr);
    std::vector<unsigned char> D((size_t)nr);
    auto values = [&](const double *rw, double *out) {
        for (int f = 0; f < NV; f++) {
            const double *x = rw + (size_t)src[f] * nr;
            double *o = out + (size_t)f * nr;
            switch (f) {
                case 0: case 1: case 2: case 3: case 12:
                    for (int j = 0; j < nr; j++) o[j] = x[j] * 1000.;
                    break;
                case 5: case 7:
                    for (int j = 0; j < nr; j++) o[j] = x[j] / 60.;
                    break;
                case 6:
                    for (int j = 0; j < nr; j++) o[j] = x[j] * 1000. * 60.;
                    break;
                case 8: case 9:
                    for (int j = 0; j < nr; j++) o[j] = x[j] * d2r;
                    break;
                default:
                    memcpy(o, x, sizeof(double) * nr);
                    break;
            }
        }
    };
    auto interp = [&](const double *Vv, int f, int s) -> double {
        const double *v = Vv + (size_t)f * nr;
        if (cst[s]) return v[0];
        const int64_t j = i1[s];
        const double v0 = v[j - 1];
        return v0 + ((v[j] - v0) / dseg[j - 1]) * dr[s];
    };
    const size_t tsz = (size_t)BBGPU_NSR * nsub;
    values(rows, V0.data());
    for (int k = 0; k < nb; k++) {
        double *t = sr + (size_t)k * tsz;
        if (k == 0) {
            memcpy(t, radii, sizeof(double) * nsub);
            for (int f = 0; f < NV; f++)
                for (int s = 0; s < nsub; s++) t[(size_t)(f + 1) * nsub + s] = interp(V0.data(), f, s);
            if (edgew)
                for (int s = 0; s < nsub; s++) t[(size_t)5 * nsub + s] *= edgew[s];
            memcpy(t + (size_t)14 * nsub, side, sizeof(double) * 2 * nsub);
        } else {
            const double *rw = rows + (size_t)k * 17 * nr;
            memcpy(t, sr, sizeof(double) * tsz);
            // the rings whose values (of the interpolated rows) differ from member 0's
            bool any = false;
            for (int j = 0; j < nr; j++) D[j] = 0;
            for (int f = 0; f < NV; f++) {
                const double *a = rw + (size_t)src[f] * nr, *b = rows + (size_t)src[f] * nr;
                if (!memcmp(a, b, sizeof(double) * nr)) continue;
                for (int j = 0; j < nr; j++)
                    if (memcmp(a + j, b + j, sizeof(double))) D[j] = 1, any = true;
            }
            if (any) {
                values(rw, V.data());
                for (int s = 0; s < nsub; s++) {
                    const bool chg = cst[s] ? D[0] : (D[i1[s] - 1] || D[i1[s]]);
                    if (!chg) continue;
                    for (int f = 0; f < NV; f++) t[(size_t)(f + 1) * nsub + s] = interp(V.data(), f, s);
                    if (edgew) t[(size_t)5 * nsub + s] *= edgew[s];
                }
            }
        }
        for (int s = 0; s < nsub; s++) nv[(size_t)k * nsub + s] = t[(size_t)4 * nsub + s] == 0.0 ? 1 : nvtmp;
        if (ms)
            for (int r = 0; r < BBGPU_NSR; r++)
                memcpy(ms + ((size_t)k * BBGPU_NSR + r) * nsm, t + (size_t)r * nsub, sizeof(double) * nsub);
    }
    return BBGPU_OK;
}
