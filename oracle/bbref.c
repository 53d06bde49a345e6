/*
 * CPU restatement of BBarolo 2's model-evaluation kernels: the ORACLE of the GPU path.
 *
 * This file is test infrastructure. Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it, as the checker; the product never links or calls it.
 *
 * Each function restates, in plain C with the reference's operation order (compile with
 * -ffp-contract=off: no fused multiply-adds, so every operation rounds as in the reference's float64),
 * the numba kernel cited beside it. The reference runs these kernels through numba, whose math
 * functions are the C library's (exp, log, sin, cos, sqrt, atanh, tan, erf, erfc, tanh, atan): the same
 * functions are called here.
 *
 * Pinned against the reference itself: the golden fixtures under tests/golden/ were produced by running
 * the reference's Python kernels (bbarolo/_rng.py, bbarolo/galmod.py, bbarolo/smooth.py,
 * bbarolo/galfit.py, bbarolo/bayesian/likelihood.py) and the CPU tests check this file against them.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define C_MS 2.99792458e08

/* ------------------------------------------------------------------ RNG (bbarolo/_rng.py) */
static int64_t KN[128];
static double WN[128], FN[128];
static int zig_ready = 0;

/* bbarolo/_rng.py:17-38 */
static void zig_tables(void) {
    double dn = 3.442619855899, tn = dn, vn = 9.91256303526217e-3, m1 = 2147483648.0;
    double q = vn / exp(-.5 * dn * dn);
    KN[0] = (int64_t)((dn / q) * m1);
    KN[1] = 0;
    WN[0] = q / m1;
    WN[127] = dn / m1;
    FN[0] = 1.;
    FN[127] = exp(-.5 * dn * dn);
    for (int i = 126; i >= 1; i--) {
        dn = sqrt(-2. * log(vn / dn + exp(-.5 * dn * dn)));
        KN[i + 1] = (int64_t)((dn / tn) * m1);
        tn = dn;
        FN[i] = exp(-.5 * dn * dn);
        WN[i] = dn / m1;
    }
    zig_ready = 1;
}

void ref_zig_tables(int64_t *kn, double *wn, double *fn) {
    if (!zig_ready) zig_tables();
    memcpy(kn, KN, sizeof KN); memcpy(wn, WN, sizeof WN); memcpy(fn, FN, sizeof FN);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* bbarolo/_rng.py:49-63 (splitmix64) */
void ref_rng_init(uint64_t seed, uint64_t *s) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
    for (int i = 0; i < 2; i++) {
        z = z + 0x9E3779B97F4A7C15ULL;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
        x = x ^ (x >> 31);
        s[i] = x;
    }
    if (s[0] == 0 && s[1] == 0) s[0] = 1;
}

/* bbarolo/_rng.py:66-74 (xoroshiro128+) */
uint64_t ref_rng_next(uint64_t *s) {
    uint64_t s0 = s[0], s1 = s[1], r = s0 + s1;
    s1 ^= s0;
    s[0] = rotl(s0, 24) ^ s1 ^ (s1 << 16);
    s[1] = rotl(s1, 37);
    return r;
}

/* bbarolo/_rng.py:77-80 */
double ref_rng_uniform(uint64_t *s) { return (double)(ref_rng_next(s) >> 11) * (1.0 / 9007199254740992.0); }

/* bbarolo/_rng.py:83-100 (Marsaglia & Tsang ziggurat) */
double ref_rng_normal(uint64_t *s) {
    if (!zig_ready) zig_tables();
    for (;;) {
        int64_t hz = (int64_t)(ref_rng_next(s) >> 32) - 2147483648LL;
        int64_t iz = hz & 127;
        int64_t ahz = hz < 0 ? -hz : hz;
        if (ahz < KN[iz]) return (double)hz * WN[iz];
        double x = (double)hz * WN[iz];
        if (iz == 0) {
            double xx, yy;
            for (;;) {
                xx = -log(1.0 - ref_rng_uniform(s)) * 0.2904764;
                yy = -log(1.0 - ref_rng_uniform(s));
                if (yy + yy >= xx * xx) break;
            }
            return hz > 0 ? 3.442620 + xx : -3.442620 - xx;
        }
        if (FN[iz] + ref_rng_uniform(s) * (FN[iz - 1] - FN[iz]) < exp(-.5 * x * x)) return x;
    }
}

/* ------------------------------------------------------------------ helpers (bbarolo/galmod.py:38-89) */
static inline int64_t lround_ref(double x) {
    if (!(fabs(x) < 1e18)) return -((int64_t)1 << 62);
    if (x >= 0) return (int64_t)(x + 0.5);
    return -(int64_t)(-x + 0.5);
}

static inline double velgrid(double v, int axtyp, int velsys, double freq0, double crval3, double cdelt3,
                             double crpix3) {
    double w;
    if (axtyp == 4) w = v;
    else {
        if (velsys == 1) w = freq0 * (1 - v / C_MS);
        else if (velsys == 2) w = freq0 * (C_MS / (C_MS + v));
        else w = freq0 * sqrt((C_MS - v) / (C_MS + v));
        if (axtyp == 2) w = C_MS / w;
    }
    return (w - crval3) / cdelt3 + crpix3 - 1;
}

static inline double lagged(double vrot, double dvdz, double dz) {
    double v = vrot - dvdz * dz;
    if (vrot >= 0.0) return (0.0 > v) ? 0.0 : v;
    return (0.0 < v) ? 0.0 : v;
}

static inline double fdev(int ltype, uint64_t *st) {
    if (ltype == 1) return ref_rng_normal(st);
    double x = 2.0 * ref_rng_uniform(st) - 1.0;
    if (ltype == 2) return atanh(x);
    if (ltype == 3) return x >= 0.0 ? -log(x) : log(-x);
    if (ltype == 4) return tan(0.5 * M_PI * x);
    return x;
}

#define SR(row, ir) sr[(size_t)(row) * nsub + (ir)]

/* ------------------------------------------------------------------ _galmod_mc (bbarolo/galmod.py:92-171)
 * out: (ny, nx, nz) float64, accumulated. sr: (16, nsub). */
void ref_galmod_mc(double *out, int ny, int nx, int nz, const double *sr, int nsub, int ring_lo, int ring_hi,
                   uint64_t seed, double radsep, const int64_t *nv, double cdens, int cmode, double pixarea,
                   double cdelt0, double cdelt1, double crota2, int64_t blo0, int64_t blo1, int64_t bhi0,
                   int64_t bhi1, int ltype, double sig_instr, int axtyp, int velsys, int nlines,
                   const double *lfreq0, double crval3, double cdelt3, double crpix3, const double *relint,
                   const double *cd2i) {
    (void)ny;
    uint64_t st[2];
    ref_rng_init(seed, st);
    int linear = axtyp == 4 && nlines == 1;
    double ia = 1.0 / cdelt3;
    double ib = -crval3 / cdelt3 + crpix3 - 1;
    for (int ir = ring_lo; ir < ring_hi; ir++) {
        double R0 = SR(0, ir), dens = SR(5, ir);
        if (dens == 0) continue;
        double ring_area_pix = 2 * M_PI * R0 * radsep / pixarea;
        double dpow = cmode == 1 ? pow(dens, 1.0) : pow(dens, (double)cmode);
        int64_t nc = lround_ref(cdens * dpow * ring_area_pix);
        if ((double)lround_ref((double)nc / ring_area_pix) < 10.) nc = lround_ref(10 * ring_area_pix);
        double vrot = SR(1, ir), vrad = SR(2, ir), vvert = SR(3, ir);
        double vdisptmp = sqrt(SR(4, ir) * SR(4, ir) + sig_instr * sig_instr);
        double z0 = SR(6, ir), dvdz = SR(7, ir), zcyl = SR(8, ir);
        double sinc = sin(SR(9, ir)), cinc = cos(SR(9, ir));
        double phi = SR(10, ir);
        double spa = sin(phi) * cos(crota2) + cos(phi) * sin(crota2);
        double cpa = cos(phi) * cos(crota2) - sin(phi) * sin(crota2);
        double xpos = SR(11, ir), ypos = SR(12, ir), vsys0 = SR(13, ir);
        int64_t nvr = nv[ir];
        double fluxsc = (double)(float)(dens * ring_area_pix * pixarea / (double)(nc * nvr));
        double r_inner = R0 - 0.5 * radsep;
        double r_inner_sq = r_inner * r_inner;
        double r_cross = 2.0 * radsep * R0;
        for (int64_t ic = 0; ic < nc; ic++) {
            double R = sqrt(r_inner_sq + r_cross * fabs(2.0 * ref_rng_uniform(st) - 1.0));
            double az = 2 * M_PI * fabs(2.0 * ref_rng_uniform(st) - 1.0);
            double saz = sin(az), caz = cos(az);
            double z = fdev(ltype, st) * z0;
            double x = R * caz;
            double y = R * saz * cinc - z * sinc;
            int64_t g0 = lround_ref(xpos + (x * spa - y * cpa) / cdelt0);
            int64_t g1 = lround_ref(ypos + (x * cpa + y * spa) / cdelt1);
            double wside = caz >= 0.0 ? SR(14, ir) : SR(15, ir);
            if (wside == 0.0 || g0 < blo0 || g0 >= bhi0 || g1 < blo1 || g1 >= bhi1) {
                for (int64_t iv = 0; iv < nvr; iv++) ref_rng_normal(st);
                continue;
            }
            int64_t px = g0 - blo0, py = g1 - blo1;
            double az_ = fabs(z), vs;
            if (az_ > zcyl) vs = vsys0 + (lagged(vrot, dvdz, az_ - zcyl) * caz + vrad * saz) * sinc;
            else vs = vsys0 + (vrot * caz + vrad * saz) * sinc;
            vs += vvert * cinc;
            double *o = out + ((size_t)py * nx + (size_t)px) * nz;
            if (linear) {
                double gz = vs * ia + ib, sg = vdisptmp * ia;
                double val = relint[0] * fluxsc * wside;
                for (int64_t iv = 0; iv < nvr; iv++) {
                    int64_t isubs = lround_ref(gz + ref_rng_normal(st) * sg);
                    if (isubs < 0 || isubs >= nz) continue;
                    o[isubs] += val * cd2i[isubs];
                }
            } else {
                for (int64_t iv = 0; iv < nvr; iv++) {
                    double v = vs + ref_rng_normal(st) * vdisptmp;
                    for (int nl = 0; nl < nlines; nl++) {
                        int64_t isubs = lround_ref(velgrid(v, axtyp, velsys, lfreq0[nl], crval3, cdelt3, crpix3));
                        if (isubs < 0 || isubs >= nz) continue;
                        o[isubs] += relint[nl] * fluxsc * wside * cd2i[isubs];
                    }
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ ANALYTIC (bbarolo/galmod.py:174-465) */
#define PHI_N 6146
static double PHI_TAB[PHI_N];
static int phi_ready = 0;

/* bbarolo/galmod.py:176-180 */
static void phi_table(void) {
    for (int k = 0; k < PHI_N; k++) PHI_TAB[k] = 0.5 * erfc(-(-6.0 + k / 512.0) / sqrt(2.0));
    phi_ready = 1;
}

void ref_phi_table(double *out) {
    if (!phi_ready) phi_table();
    memcpy(out, PHI_TAB, sizeof PHI_TAB);
}

/* bbarolo/galmod.py:183-191 */
static inline double phi_interp(double t) {
    double x = (t + 6.0) * 512.0;
    if (x <= 0.0) return 0.0;
    int64_t k = (int64_t)x;
    if (k >= PHI_N - 1) return 1.0;
    return PHI_TAB[k] + (x - (double)k) * (PHI_TAB[k + 1] - PHI_TAB[k]);
}

/* bbarolo/galmod.py:194-214 */
static inline int line_profile(double *prof, double v, double sig, const double *vedges, const double *cd2i,
                               int64_t kc, int64_t K, int64_t nz, int64_t *k0out) {
    int64_t k0 = kc - K;
    if (k0 < 0) k0 = 0;
    int64_t k1 = kc + K + 1;
    if (k1 > nz) k1 = nz;
    if (k1 <= k0) { *k0out = 0; return 0; }
    double inv = 1.0 / sig;
    double pp = phi_interp((vedges[k0] - v) * inv);
    for (int64_t k = k0; k < k1; k++) {
        double pn = phi_interp((vedges[k + 1] - v) * inv);
        double f = pn - pp;
        prof[k - k0] = (f >= 0 ? f : -f) * cd2i[k];
        pp = pn;
    }
    *k0out = k0;
    return (int)(k1 - k0);
}

/* bbarolo/galmod.py:217-259 */
static inline double layer_cdf(int ltype, double x) {
    if (ltype == 1) return 0.5 * (1.0 + erf(x / sqrt(2.0)));
    if (ltype == 2) return 0.5 * (1.0 + tanh(x));
    if (ltype == 3) return x >= 0 ? 1.0 - 0.5 * exp(-x) : 0.5 * exp(x);
    if (ltype == 4) return 0.5 + atan(x) / M_PI;
    double c = x < -1.0 ? -1.0 : x;
    c = c > 1.0 ? 1.0 : c;
    return 0.5 * (c + 1.0);
}

static inline double layer_extent(int ltype) {
    return ltype == 1 ? 5.0 : ltype == 2 ? 7.6 : ltype == 3 ? 14.0 : ltype == 4 ? 1e30 : 1.0;
}

static inline double layer_core(int ltype) {
    return ltype == 1 ? 3.717 : ltype == 2 ? 4.147 : ltype == 3 ? 6.908 : ltype == 4 ? 31.61 : 1e30;
}

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* bbarolo/galmod.py:276-323 */
int ref_zgrid(double *zq, double *wq, int nmax, int ltype, double z0, double sinc, double pixsize, double dvdz,
              double sig, double R0, double radsep, double xpos, double ypos, double cdelt0, double cdelt1,
              int64_t blo0, int64_t blo1, int64_t bhi0, int64_t bhi1, double zstep) {
    double s = fabs(sinc);
    if (z0 <= 0 || nmax < 2 || s < 1e-6) { zq[0] = 0.0; wq[0] = 1.0; return 1; }
    double dx = dmax(fabs((double)blo0 - 0.5 - xpos), fabs((double)bhi0 - 0.5 - xpos)) * fabs(cdelt0);
    double dy = dmax(fabs((double)blo1 - 0.5 - ypos), fabs((double)bhi1 - 0.5 - ypos)) * fabs(cdelt1);
    double zlim = dmin(layer_extent(ltype), (R0 + radsep + sqrt(dx * dx + dy * dy)) / (s * z0));
    double step = zstep * pixsize / (z0 * s);
    if (dvdz != 0) step = dmin(step, 0.5 * sig / (fabs(dvdz) * z0 * s));
    double zc = layer_core(ltype);
    int64_t nin, nout;
    for (;;) {
        nin = (int64_t)ceil(dmin(zc, zlim) / step);
        if (nin < 1) nin = 1;
        nout = (int64_t)ceil((zlim - (double)nin * step) / (4.0 * step));
        if (nout < 0) nout = 0;
        if (2 * (nin + nout) <= nmax) break;
        step *= 1.01 * (double)(nin + nout) / (double)(nmax / 2);
    }
    int64_t half = nin + nout;
    for (int64_t j = 0; j < half; j++) {
        double lo = j < nin ? (double)j * step : (double)(nin + 4 * (j - nin)) * step;
        double hi = dmin(lo + (j < nin ? step : 4.0 * step), zlim);
        double w = layer_cdf(ltype, hi) - layer_cdf(ltype, lo);
        zq[half + j] = 0.5 * (lo + hi); wq[half + j] = w;
        zq[half - 1 - j] = -0.5 * (lo + hi); wq[half - 1 - j] = w;
    }
    return (int)(2 * half);
}

/* bbarolo/galmod.py:326-465. vedges: (nlines, nz+1). */
void ref_galmod_analytic(double *out, int ny, int nx, int nz, const double *sr, int nsub, int ring_lo,
                         int ring_hi, double radsep, double cdens, double pixarea, double cdelt0, double cdelt1,
                         double crota2, int64_t blo0, int64_t blo1, int64_t bhi0, int64_t bhi1, int ltype,
                         double sig_instr, const double *vedges, const double *relint, const double *cd2i,
                         int nzq, int axtyp, int velsys, int nlines, const double *lfreq0, double crval3,
                         double cdelt3, double crpix3, double chwidth, double zstep) {
    (void)cdens; (void)ny;
    if (!phi_ready) phi_table();
    int nb = nzq > 1 ? nzq : 1;
    double pixsize = sqrt(pixarea);
    double *zq = malloc(sizeof(double) * nb), *wq = malloc(sizeof(double) * nb);
    double *prof = malloc(sizeof(double) * (nz + 1));
    int64_t *gx = malloc(sizeof(int64_t) * nb), *gy = malloc(sizeof(int64_t) * nb);
    for (int ir = ring_lo; ir < ring_hi; ir++) {
        double R0 = SR(0, ir), dens = SR(5, ir);
        if (dens == 0) continue;
        double ring_area_pix = 2 * M_PI * R0 * radsep / pixarea;
        double circ_pix = 2 * M_PI * R0 / sqrt(pixarea);
        int64_t naz = (int64_t)(3 * circ_pix + 0.5);
        if (naz < 16) naz = 16;
        int nrad = 2;
        double vrot = SR(1, ir), vrad = SR(2, ir), vvert = SR(3, ir);
        double sig = dmax(sqrt(SR(4, ir) * SR(4, ir) + sig_instr * sig_instr), 1e-6 * fabs(chwidth));
        int64_t K = (int64_t)(5.0 * sig / chwidth) + 2;
        double z0 = SR(6, ir), dvdz = SR(7, ir), zcyl = SR(8, ir);
        double sinc = sin(SR(9, ir)), cinc = cos(SR(9, ir));
        double phi = SR(10, ir);
        double spa = sin(phi) * cos(crota2) + cos(phi) * sin(crota2);
        double cpa = cos(phi) * cos(crota2) - sin(phi) * sin(crota2);
        double xpos = SR(11, ir), ypos = SR(12, ir), vsys0 = SR(13, ir);
        int nzz = ref_zgrid(zq, wq, nzq, ltype, z0, sinc, pixsize, dvdz, sig, R0, radsep, xpos, ypos, cdelt0,
                            cdelt1, blo0, blo1, bhi0, bhi1, zstep);
        double fluxsc = dens * ring_area_pix * pixarea / (double)(naz * nrad);
        int zdep = 0;
        if (dvdz != 0 && nzz > 1)
            for (int kz = 0; kz < nzz; kz++)
                if (fabs(zq[kz] * z0) > zcyl) { zdep = 1; break; }
        double r_inner = R0 - 0.5 * radsep;
        double daz = 2 * M_PI / (double)naz;
        double cd = cos(daz), sd = sin(daz);
        for (int kr = 0; kr < nrad; kr++) {
            double u = (kr + 0.5) / nrad;
            double R = sqrt(r_inner * r_inner + 2.0 * radsep * R0 * u);
            double az0 = 2 * M_PI * (0.5 * ((kr + 1) % 2) + 0.25) / (double)naz;
            double caz = cos(az0), saz = sin(az0);
            for (int64_t ka = 0; ka < naz; ka++) {
                if (ka > 0) {
                    double c2 = caz * cd - saz * sd, s2 = saz * cd + caz * sd;
                    caz = c2; saz = s2;
                }
                double wside = caz >= 0.0 ? SR(14, ir) : SR(15, ir);
                if (wside == 0.0) continue;
                double x = R * caz, yb = R * saz * cinc, xs = x * spa, xc = x * cpa;
                for (int kz = 0; kz < nzz; kz++) {
                    double z = nzz > 1 ? zq[kz] * z0 : 0.0;
                    double y = yb - z * sinc;
                    gx[kz] = lround_ref(xpos + (xs - y * cpa) / cdelt0);
                    gy[kz] = lround_ref(ypos + (xc + y * spa) / cdelt1);
                }
                double vplane = vsys0 + (vrot * caz + vrad * saz) * sinc + vvert * cinc;
                int inbox = 0;
                for (int kz = 0; kz < nzz; kz++)
                    if (blo0 <= gx[kz] && gx[kz] < bhi0 && blo1 <= gy[kz] && gy[kz] < bhi1) { inbox = 1; break; }
                if (!inbox) continue;
                for (int nl = 0; nl < nlines; nl++) {
                    double a = relint[nl] * fluxsc * wside;
                    const double *ve = vedges + (size_t)nl * (nz + 1);
                    int64_t k0;
                    if (!zdep) {
                        double v = vplane;
                        int64_t kc = lround_ref(velgrid(v, axtyp, velsys, lfreq0[nl], crval3, cdelt3, crpix3));
                        int nk = line_profile(prof, v, sig, ve, cd2i, kc, K, nz, &k0);
                        if (nk == 0) continue;
                        int kz = 0;
                        while (kz < nzz) {
                            int64_t g0 = gx[kz], g1 = gy[kz];
                            double ws = wq[kz];
                            int w = 1;
                            while (kz + w < nzz && gx[kz + w] == g0 && gy[kz + w] == g1) { ws += wq[kz + w]; w++; }
                            kz += w;
                            if (g0 < blo0 || g0 >= bhi0 || g1 < blo1 || g1 >= bhi1) continue;
                            double aw = a * ws;
                            double *o = out + ((size_t)(g1 - blo1) * nx + (size_t)(g0 - blo0)) * nz;
                            for (int j = 0; j < nk; j++) o[k0 + j] += aw * prof[j];
                        }
                    } else {
                        for (int kz = 0; kz < (nzz + 1) / 2; kz++) {
                            int kz2 = nzz - 1 - kz;
                            int in1 = !(gx[kz] < blo0 || gx[kz] >= bhi0 || gy[kz] < blo1 || gy[kz] >= bhi1);
                            int in2 = kz2 != kz && !(gx[kz2] < blo0 || gx[kz2] >= bhi0 || gy[kz2] < blo1 ||
                                                     gy[kz2] >= bhi1);
                            if (!(in1 || in2)) continue;
                            double az_ = fabs(zq[kz] * z0), v;
                            if (az_ > zcyl) v = vsys0 + (lagged(vrot, dvdz, az_ - zcyl) * caz + vrad * saz) * sinc +
                                                vvert * cinc;
                            else v = vplane;
                            int64_t kc = lround_ref(velgrid(v, axtyp, velsys, lfreq0[nl], crval3, cdelt3, crpix3));
                            int nk = line_profile(prof, v, sig, ve, cd2i, kc, K, nz, &k0);
                            if (nk == 0) continue;
                            if (in1 && in2 && gx[kz] == gx[kz2] && gy[kz] == gy[kz2]) {
                                double *o = out + ((size_t)(gy[kz] - blo1) * nx + (size_t)(gx[kz] - blo0)) * nz;
                                double aw = a * (wq[kz] + wq[kz2]);
                                for (int j = 0; j < nk; j++) o[k0 + j] += aw * prof[j];
                                continue;
                            }
                            if (in1) {
                                double *o = out + ((size_t)(gy[kz] - blo1) * nx + (size_t)(gx[kz] - blo0)) * nz;
                                double aw = a * wq[kz];
                                for (int j = 0; j < nk; j++) o[k0 + j] += aw * prof[j];
                            }
                            if (in2) {
                                double *o = out + ((size_t)(gy[kz2] - blo1) * nx + (size_t)(gx[kz2] - blo0)) * nz;
                                double aw = a * wq[kz2];
                                for (int j = 0; j < nk; j++) o[k0 + j] += aw * prof[j];
                            }
                        }
                    }
                }
            }
        }
    }
    free(zq); free(wq); free(prof); free(gx); free(gy);
}

/* bbarolo/galmod.py:468-536. out: (nr, ny, nx); widx, wval: (nsub, 2). */
void ref_ring_maps_analytic(double *out, int nr, int ny, int nx, const double *sr, int nsub, const int64_t *widx,
                            const double *wval, double radsep, double pixarea, double cdelt0, double cdelt1,
                            double crota2, int64_t blo0, int64_t blo1, int64_t bhi0, int64_t bhi1, int ltype,
                            int nzq, double sig_instr, double chwidth, double zstep) {
    (void)nr;
    int nb = nzq > 1 ? nzq : 1;
    double pixsize = sqrt(pixarea);
    double *zq = malloc(sizeof(double) * nb), *wq = malloc(sizeof(double) * nb);
    int64_t *gx = malloc(sizeof(int64_t) * nb), *gy = malloc(sizeof(int64_t) * nb);
    for (int ir = 0; ir < nsub; ir++) {
        if (widx[2 * ir] < 0 && widx[2 * ir + 1] < 0) continue;
        double R0 = SR(0, ir);
        double ring_area_pix = 2 * M_PI * R0 * radsep / pixarea;
        double circ_pix = 2 * M_PI * R0 / sqrt(pixarea);
        int64_t naz = (int64_t)(3 * circ_pix + 0.5);
        if (naz < 16) naz = 16;
        int nrad = 2;
        double z0 = SR(6, ir);
        double sinc = sin(SR(9, ir));
        double phi = SR(10, ir);
        double spa = sin(phi) * cos(crota2) + cos(phi) * sin(crota2);
        double cpa = cos(phi) * cos(crota2) - sin(phi) * sin(crota2);
        double xpos = SR(11, ir), ypos = SR(12, ir);
        double sig = dmax(sqrt(SR(4, ir) * SR(4, ir) + sig_instr * sig_instr), 1e-6 * fabs(chwidth));
        int nzz = ref_zgrid(zq, wq, nzq, ltype, z0, sinc, pixsize, SR(7, ir), sig, R0, radsep, xpos, ypos,
                            cdelt0, cdelt1, blo0, blo1, bhi0, bhi1, zstep);
        double cinc = cos(SR(9, ir));
        double fluxsc = ring_area_pix * pixarea / (double)(naz * nrad);
        double r_inner = R0 - 0.5 * radsep;
        double daz = 2 * M_PI / (double)naz;
        double cd = cos(daz), sd = sin(daz);
        for (int kr = 0; kr < nrad; kr++) {
            double u = (kr + 0.5) / nrad;
            double R = sqrt(r_inner * r_inner + 2.0 * radsep * R0 * u);
            double az0 = 2 * M_PI * (0.5 * ((kr + 1) % 2) + 0.25) / (double)naz;
            double caz = cos(az0), saz = sin(az0);
            for (int64_t ka = 0; ka < naz; ka++) {
                if (ka > 0) {
                    double c2 = caz * cd - saz * sd, s2 = saz * cd + caz * sd;
                    caz = c2; saz = s2;
                }
                double wside = caz >= 0.0 ? SR(14, ir) : SR(15, ir);
                if (wside == 0.0) continue;
                double x = R * caz, yb = R * saz * cinc, xs = x * spa, xc = x * cpa;
                for (int kz = 0; kz < nzz; kz++) {
                    double z = nzz > 1 ? zq[kz] * z0 : 0.0;
                    double y = yb - z * sinc;
                    gx[kz] = lround_ref(xpos + (xs - y * cpa) / cdelt0);
                    gy[kz] = lround_ref(ypos + (xc + y * spa) / cdelt1);
                }
                int kz = 0;
                while (kz < nzz) {
                    int64_t g0 = gx[kz], g1 = gy[kz];
                    double ws = wq[kz];
                    kz++;
                    while (kz < nzz && gx[kz] == g0 && gy[kz] == g1) { ws += wq[kz]; kz++; }
                    if (g0 < blo0 || g0 >= bhi0 || g1 < blo1 || g1 >= bhi1) continue;
                    for (int m = 0; m < 2; m++) {
                        int64_t r = widx[2 * ir + m];
                        if (r >= 0)
                            out[((size_t)r * ny + (size_t)(g1 - blo1)) * nx + (size_t)(g0 - blo0)] +=
                                fluxsc * ws * wval[2 * ir + m] * wside;
                    }
                }
            }
        }
    }
    free(zq); free(wq); free(gx); free(gy);
}

/* ------------------------------------------------------------------ beam convolution
 * Direct "same" linear convolution of each plane of a (nz, ny, nx) float64 array with the kernel (ky, kx):
 * out[y, x] = sum_{j,i} k[j, i] in[y + ky/2 - j, x + kx/2 - i] (zero outside), the crop of the full linear
 * convolution taken by FFTConvolver (bbarolo/smooth.py:145-165); then, as DiskModel.convolve
 * (bbarolo/galmod.py:1273-1283), values below 1e-12 set to zero and the flux scale applied. This is the
 * FP64 oracle of the smoothed cube: it agrees with the FFT of the reference to ~1e-16 of the peak. */
void ref_conv_same(const double *in, double *out, int nz, int ny, int nx, const double *k, int ky, int kx,
                   double scale, int threshold) {
    int hy = ky / 2, hx = kx / 2;
    for (int z = 0; z < nz; z++) {
        const double *p = in + (size_t)z * ny * nx;
        double *o = out + (size_t)z * ny * nx;
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                double s = 0.;
                for (int j = 0; j < ky; j++) {
                    int yy = y + hy - j;
                    if (yy < 0 || yy >= ny) continue;
                    for (int i = 0; i < kx; i++) {
                        int xx = x + hx - i;
                        if (xx < 0 || xx >= nx) continue;
                        s += k[j * kx + i] * p[(size_t)yy * nx + xx];
                    }
                }
                if (threshold && s < 1.E-12) s = 0.;
                else if (scale != 1.0) s *= scale;
                o[(size_t)y * nx + x] = s;
            }
    }
}

/* bbarolo/galmod.py:974-1037: model (ny, nx, nz) -> out (ny, nx, nz), out zeroed by the caller. */
void ref_conv_sparse(const double *model, double *out, int ny, int nx, int nz, const double *kern, int ky, int kx,
                     double scale) {
    int hy = ky / 2, hx = kx / 2;
    int nk = 0;
    for (int j = 0; j < ky * kx; j++) nk += kern[j] != 0;
    int64_t *kj = malloc(sizeof(int64_t) * (nk + 1)), *ki = malloc(sizeof(int64_t) * (nk + 1));
    double *kv = malloc(sizeof(double) * (nk + 1));
    nk = 0;
    for (int j = 0; j < ky; j++)
        for (int i = 0; i < kx; i++)
            if (kern[j * kx + i] != 0) { kj[nk] = j - hy; ki[nk] = i - hx; kv[nk] = kern[j * kx + i]; nk++; }
    int64_t *zl = malloc(sizeof(int64_t) * ny * nx), *zh = malloc(sizeof(int64_t) * ny * nx);
    for (int q = 0; q < ny * nx; q++) { zl[q] = nz; zh[q] = -1; }
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const double *m = model + ((size_t)y * nx + x) * nz;
            int64_t zlo = -1, zhi = -1;
            for (int z = 0; z < nz; z++)
                if (m[z] != 0) { if (zlo < 0) zlo = z; zhi = z; }
            if (zlo < 0) continue;
            for (int n = 0; n < nk; n++) {
                int64_t yy = y + kj[n], xx = x + ki[n];
                if (yy < 0 || yy >= ny || xx < 0 || xx >= nx) continue;
                size_t q = (size_t)yy * nx + xx;
                if (zlo < zl[q]) zl[q] = zlo;
                if (zhi > zh[q]) zh[q] = zhi;
                double kk = kv[n];
                double *o = out + q * nz;
                for (int64_t z = zlo; z <= zhi; z++) o[z] += kk * m[z];
            }
        }
    for (int q = 0; q < ny * nx; q++) {
        double *o = out + (size_t)q * nz;
        for (int64_t z = zl[q]; z <= zh[q]; z++) {
            double v = o[z];
            if (v < 1.E-12) o[z] = 0.;
            else if (scale != 1.0) o[z] = v * scale;
        }
    }
    free(kj); free(ki); free(kv); free(zl); free(zh);
}

/* ------------------------------------------------------------------ residuals (bbarolo/bayesian/likelihood.py:22-77)
 * model f64 (nz, ny, nx), data f32 and mask u8 with the same shape (views of the box), region u8 (ny, nx)
 * or NULL. */
double ref_sumsq_residuals(const double *model, const float *data, const uint8_t *mask, int maskmode,
                           const uint8_t *region, int nz, int ny, int nx) {
    double s = 0.;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                if (region && !region[j * nx + i]) continue;
                size_t q = ((size_t)k * ny + j) * nx + i;
                double d = data[q];
                if (d != d || d == 0.) continue;
                if (maskmode != 0 && !mask[q]) {
                    if (maskmode == 2) continue;
                    d = 0.;
                }
                double r = d - model[q];
                s += r * r;
            }
    return s;
}

void ref_residuals_fracerr(const double *model, const float *data, const uint8_t *mask, int maskmode,
                           const uint8_t *region, int nz, int ny, int nx, double sigma2, double eps2, double *out) {
    double s = 0., lg = 0.;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                if (region && !region[j * nx + i]) continue;
                size_t q = ((size_t)k * ny + j) * nx + i;
                double d = data[q];
                if (d != d || d == 0.) continue;
                if (maskmode != 0 && !mask[q]) {
                    if (maskmode == 2) continue;
                    d = 0.;
                }
                double m = model[q], r = d - m;
                if (m != 0.) {
                    double v = sigma2 + eps2 * m * m;
                    s += r * r / v;
                    lg += log(v / sigma2);
                } else s += r * r / sigma2;
            }
    out[0] = s;
    out[1] = lg;
}

/* ------------------------------------------------------------------ CLASSIC normalisation + residual
 * bbarolo/galfit.py:39-188. model (bsy, bsx, nz) f64 is MODIFIED (x factor) as in the reference; data f32
 * and mask u8 are (ny, nx, nz) full arrays ("yxz"); chan_noise (nz); pre (bsy, bsx, nz) or NULL; ilo/ihi (ky);
 * thr (nz); P work (ky, bsx+1, nz). */
double ref_norm(double *model, int bsy, int bsx, int nz, const float *data, const uint8_t *mask, int dny, int dnx,
                int64_t blo0, int64_t blo1, double x0, double y0, double phi, double inc, double r1, double r2,
                double wpow, int side, int ftype, const double *chan_noise, double data_noise, double bweight,
                int normtype, const double *pre, const int64_t *ilo, const int64_t *ihi, int ky, const double *thr,
                int foot, double hmax) {
    (void)dny;
    int trunc = pre != NULL;
    int hy = ky / 2;
    double *lam = calloc(nz, sizeof(double));
    double *P = trunc ? calloc((size_t)ky * (bsx + 1) * nz, sizeof(double)) : NULL;
    int64_t nextrow = 0;
    double F = M_PI / 180.;
    double sphi = sin(F * phi), cphi = cos(F * phi), cinc = cos(F * inc);
    int64_t numBlanks = 0, numPix_tot = 0;
    double minfunc = 0.0;
    int usesin = wpow < 0;
    double apow = fabs(wpow);
    uint8_t *inside = calloc((size_t)bsy * bsx, 1);
    double *wmap = calloc((size_t)bsy * bsx, sizeof(double));
#define DAT(y, x, z) data[(((size_t)(y) + blo1) * dnx + ((size_t)(x) + blo0)) * nz + (z)]
#define MSK(y, x, z) mask[(((size_t)(y) + blo1) * dnx + ((size_t)(x) + blo0)) * nz + (z)]
#define MOD(y, x, z) model[(((size_t)(y)) * bsx + (size_t)(x)) * nz + (z)]
    for (int y = 0; y < bsy; y++)
        for (int x = 0; x < bsx; x++) {
            double xr = -(x - x0) * sphi + (y - y0) * cphi;
            double ys = -(x - x0) * cphi - (y - y0) * sphi;
            double yr = ys / cinc;
            double r = sqrt(xr * xr + yr * yr);
            double th = r < 0.1 ? 0.0 : atan2(yr, xr) / F;
            if (foot == 1) {
                if (!(fabs(xr) >= r1 && fabs(xr) <= r2 && fabs(ys) <= hmax)) continue;
                th = xr >= 0 ? 0.0 : 180.0;
            } else if (!(r >= r1 && r <= r2)) continue;
            if (side == 1 && !(fabs(th) <= 90.0)) continue;
            if (side == 2 && !(fabs(th) >= 90.0)) continue;
            inside[y * bsx + x] = 1;
            if (foot == 1) { wmap[y * bsx + x] = 1.0; continue; }
            double wf = usesin ? fabs(sin(th * F)) : fabs(cos(th * F));
            wmap[y * bsx + x] = pow(wf, apow);
        }
    double factor = 1.0;
    if (normtype == 1) {
        double modSum = 0.0, obsSum = 0.0;
        for (int y = 0; y < bsy; y++)
            for (int x = 0; x < bsx; x++) {
                if (!inside[y * bsx + x]) continue;
                for (int z = 0; z < nz; z++) {
                    modSum += MOD(y, x, z);
                    if (MSK(y, x, z)) obsSum += DAT(y, x, z);
                }
            }
        factor = modSum != 0 ? obsSum / modSum : 0.0;
    }
    for (int y = 0; y < bsy; y++) {
        if (trunc) {
            int anyin = 0;
            for (int x = 0; x < bsx; x++) if (inside[y * bsx + x]) { anyin = 1; break; }
            if (anyin) {
                if (nextrow < y - hy) nextrow = y - hy;
                while (nextrow <= (y + hy < bsy - 1 ? y + hy : bsy - 1)) {
                    double *Pr = P + (size_t)(nextrow % ky) * (bsx + 1) * nz;
                    const double *pr = pre + (size_t)nextrow * bsx * nz;
                    for (int z = 0; z < nz; z++) Pr[z] = 0.;
                    for (int x = 0; x < bsx; x++)
                        for (int z = 0; z < nz; z++)
                            Pr[(size_t)(x + 1) * nz + z] = Pr[(size_t)x * nz + z] + pr[(size_t)x * nz + z];
                    nextrow++;
                }
            }
        }
        for (int x = 0; x < bsx; x++) {
            if (!inside[y * bsx + x]) continue;
            if (normtype == 0) {
                double modSum = 0.0, obsSum = 0.0;
                for (int z = 0; z < nz; z++) {
                    modSum += MOD(y, x, z);
                    double o = DAT(y, x, z);
                    if (o > 0 && MSK(y, x, z)) obsSum += o;
                }
                factor = modSum != 0 ? obsSum / modSum : 0.0;
            }
            double wi = wmap[y * bsx + x];
            if (trunc) {
                int ca = nz, cb = -1;
                for (int z = 0; z < nz; z++)
                    if (MOD(y, x, z) != 0 && !MSK(y, x, z)) { if (ca == nz) ca = z; cb = z; }
                for (int z = ca; z <= cb; z++) lam[z] = 0.;
                if (cb >= ca)
                    for (int j = 0; j < ky; j++) {
                        int yy = y + hy - j;
                        if (yy < 0 || yy >= bsy) continue;
                        int64_t xa = x + ilo[j] > 0 ? x + ilo[j] : 0;
                        int64_t xb = x + ihi[j] + 1 < bsx ? x + ihi[j] + 1 : bsx;
                        if (xb <= xa) continue;
                        const double *p1 = P + ((size_t)(yy % ky) * (bsx + 1) + xb) * nz;
                        const double *p0 = P + ((size_t)(yy % ky) * (bsx + 1) + xa) * nz;
                        for (int z = ca; z <= cb; z++) lam[z] += p1[z] - p0[z];
                    }
            }
            for (int z = 0; z < nz; z++) {
                if (normtype != 2) MOD(y, x, z) *= factor;
                double o = DAT(y, x, z);
                double obs = o > 0 ? o : data_noise;
                double mod = MOD(y, x, z);
                if (!MSK(y, x, z)) {
                    if (mod == 0) continue;
                    if (trunc && lam[z] < thr[z]) continue;
                    numBlanks++;
                }
                numPix_tot++;
                double nw = chan_noise[z];
                if (ftype == 1) minfunc += wi * ((mod - obs) * (mod - obs)) / sqrt(obs) / nw;
                else if (ftype == 2) minfunc += wi * fabs(mod - obs) / nw;
                else if (ftype == 3) minfunc += wi * fabs(mod - obs) / (mod + obs) / nw;
                else if (ftype == 4) minfunc += wi * ((mod - obs) * (mod - obs)) / nw;
            }
        }
    }
#undef DAT
#undef MSK
#undef MOD
    free(lam); free(P); free(inside); free(wmap);
    if (numPix_tot - numBlanks == 0) return INFINITY;
    return pow(1 + (double)numBlanks / (double)numPix_tot, bweight) * minfunc / (double)(numPix_tot - numBlanks);
}

/* ------------------------------------------------------------------ WindModel (bbarolo/windmodel.py:212-602)
 * The columns of the bi-conical wind model of WINDFIT: quadrature points of the cells, their bilinear deposit in
 * the raw box of each cell, the beam convolution of the boxes and the normal equations of the columns. Boxes are
 * (x0, x1, y0, y1, k0, k1), [lo, hi), their values in (channel, y, x) order from the offset of the box. */

/* bbarolo/windmodel.py:212-222: ys(xs) at r, linear, constant beyond the ends */
static double wind_interp(double r, const double *xs, const double *ys, int n) {
    if (n == 1 || r <= xs[0]) return ys[0];
    if (r >= xs[n - 1]) return ys[n - 1];
    int j = 0;
    while (xs[j] < r) j++;                      /* numpy searchsorted, side='left' */
    double t = (r - xs[j - 1]) / (xs[j] - xs[j - 1]);
    return ys[j - 1] + t * (ys[j] - ys[j - 1]);
}

/* bbarolo/windmodel.py:225-288. cells: (ncell, 7) = cone, r0, r1, t0, t1, p0, p1; qn: (ncell, 3). */
void ref_wind_points(const double *cells, const int64_t *qn, const int64_t *qoff, int ncell, const double *radii,
                     const double *vw, const double *vd, const double *vr, int nrad, double x0, double y0,
                     double vsys, double sinc, double cinc, double spa, double cpa, double cd0, double cd1,
                     double th_in, double th_out, double rmax, double sig_instr, double *gx, double *gy, double *vel,
                     double *sig, double *w, double *rr, double *vol, double *rbar) {
    for (int k = 0; k < ncell; k++) {
        const double *c = cells + (size_t)k * 7;
        double cs = c[0], r0 = c[1];
        double r1 = rmax < c[2] ? rmax : c[2];
        double t0 = th_in > c[3] ? th_in : c[3];
        double t1 = th_out < c[4] ? th_out : c[4];
        double p0 = c[5], p1 = c[6];
        int64_t nqr = qn[3 * k], nqt = qn[3 * k + 1], nqp = qn[3 * k + 2];
        int64_t i0 = qoff[k], i1 = qoff[k + 1];
        if (r1 <= r0 || t1 <= t0) {
            for (int64_t i = i0; i < i1; i++) {
                gx[i] = -1e9; gy[i] = -1e9; vel[i] = 0.; sig[i] = 1.; w[i] = 0.; rr[i] = r0;
            }
            vol[k] = 0.;
            rbar[k] = r1 > r0 ? 0.5 * (r0 + r1) : r0;
            continue;
        }
        double dr = (r1 - r0) / (double)nqr, dt = (t1 - t0) / (double)nqt, dp = (p1 - p0) / (double)nqp;
        int64_t i = i0;
        double wsum = 0.;
        for (int64_t a = 0; a < nqr; a++) {
            double r = r0 + ((double)a + 0.5) * dr;
            double vrad = wind_interp(r, radii, vw, nrad) * 1000.;
            double disp = wind_interp(r, radii, vd, nrad) * 1000.;
            double vrot = wind_interp(r, radii, vr, nrad) * 1000.;
            double s = sqrt(disp * disp + sig_instr * sig_instr);
            for (int64_t b = 0; b < nqt; b++) {
                double th = t0 + ((double)b + 0.5) * dt;
                double st = sin(th), ct = cos(th);
                for (int64_t q = 0; q < nqp; q++) {
                    double ph = p0 + ((double)q + 0.5) * dp;
                    double sp = sin(ph), cp = cos(ph);
                    double R = r * st, z = cs * r * ct;
                    double x = R * cp;
                    double ys = R * sp * cinc - z * sinc;
                    gx[i] = x0 + (x * spa - ys * cpa) / cd0;
                    gy[i] = y0 + (x * cpa + ys * spa) / cd1;
                    vel[i] = vsys + vrad * (cs * ct * cinc + st * sp * sinc) + vrot * cp * sinc;
                    sig[i] = s;
                    w[i] = r * r * st;
                    rr[i] = r;
                    wsum += w[i];
                    i++;
                }
            }
        }
        double V = (pow(r1, 3.0) - pow(r0, 3.0)) / 3. * (cos(t0) - cos(t1)) * (p1 - p0);
        vol[k] = V;
        double f = wsum > 0 ? V / wsum : 0.;
        double rs = 0.;
        for (int64_t j = i0; j < i1; j++) {
            w[j] *= f;
            rs += w[j] * rr[j];
        }
        rbar[k] = V > 0 ? rs / V : 0.5 * (r0 + r1);
    }
}

static inline int wind_point_ok(double w, double gx, double gy) {
    return w > 0. && fabs(gx) < 1e8 && fabs(gy) < 1e8;
}

/* bbarolo/windmodel.py:291-319 */
void ref_wind_raw_boxes(const int64_t *qoff, int ncell, const double *gx, const double *gy, const double *vel,
                        const double *sig, const double *w, const int64_t *lim, double chmin, int axtyp, int velsys,
                        int nlines, const double *lfreq0, double crval3, double cdelt3, double crpix3,
                        int64_t *rboxes) {
    for (int k = 0; k < ncell; k++) {
        int64_t bx0 = 1 << 30, bx1 = -(1 << 30), by0 = 1 << 30, by1 = -(1 << 30), bk0 = 1 << 30, bk1 = -(1 << 30);
        for (int64_t i = qoff[k]; i < qoff[k + 1]; i++) {
            if (!wind_point_ok(w[i], gx[i], gy[i])) continue;
            int64_t ix = (int64_t)floor(gx[i]), iy = (int64_t)floor(gy[i]);
            if (ix < bx0) bx0 = ix;
            if (ix + 2 > bx1) bx1 = ix + 2;
            if (iy < by0) by0 = iy;
            if (iy + 2 > by1) by1 = iy + 2;
            int64_t K = (int64_t)(5.0 * sig[i] / chmin) + 2;
            for (int nl = 0; nl < nlines; nl++) {
                int64_t kc = lround_ref(velgrid(vel[i], axtyp, velsys, lfreq0[nl], crval3, cdelt3, crpix3));
                if (kc - K < bk0) bk0 = kc - K;
                if (kc + K + 1 > bk1) bk1 = kc + K + 1;
            }
        }
        if (bx0 < lim[0]) bx0 = lim[0];
        if (bx1 > lim[1]) bx1 = lim[1];
        if (by0 < lim[2]) by0 = lim[2];
        if (by1 > lim[3]) by1 = lim[3];
        if (bk0 < lim[4]) bk0 = lim[4];
        if (bk1 > lim[5]) bk1 = lim[5];
        if (bx1 <= bx0 || by1 <= by0 || bk1 <= bk0) {
            bx0 = bx1 = lim[0];
            by0 = by1 = lim[2];
            bk0 = bk1 = lim[4];
        }
        int64_t *o = rboxes + 6 * (size_t)k;
        o[0] = bx0; o[1] = bx1; o[2] = by0; o[3] = by1; o[4] = bk0; o[5] = bk1;
    }
}

/* bbarolo/windmodel.py:322-366. vedges: (nlines, nz + 1); cd2i: the channel factors (ones for the wind). */
void ref_wind_deposit_raw(double *rbuf, const int64_t *roffs, const int64_t *rboxes, const int64_t *qoff, int ncell,
                          const double *gx, const double *gy, const double *vel, const double *sig, const double *w,
                          const double *vedges, const double *relint, const double *cd2i, double chmin, int axtyp,
                          int velsys, int nlines, const double *lfreq0, double crval3, double cdelt3, double crpix3,
                          int nz) {
    if (!phi_ready) phi_table();
    double *prof = malloc(sizeof(double) * (size_t)(nz > 0 ? nz : 1));
    for (int k = 0; k < ncell; k++) {
        const int64_t *B = rboxes + 6 * (size_t)k;
        int64_t x0 = B[0], x1 = B[1], y0 = B[2], y1 = B[3], k0 = B[4], k1 = B[5];
        if (x1 <= x0 || y1 <= y0 || k1 <= k0) continue;
        int64_t bx = x1 - x0, by = y1 - y0, base = roffs[k];
        for (int64_t i = qoff[k]; i < qoff[k + 1]; i++) {
            if (!wind_point_ok(w[i], gx[i], gy[i])) continue;
            int64_t ix = (int64_t)floor(gx[i]), iy = (int64_t)floor(gy[i]);
            double fx = gx[i] - (double)ix, fy = gy[i] - (double)iy;
            double s = sig[i];
            if (s < 1e-6 * chmin) s = 1e-6 * chmin;
            int64_t K = (int64_t)(5.0 * s / chmin) + 2;
            for (int nl = 0; nl < nlines; nl++) {
                int64_t kc = lround_ref(velgrid(vel[i], axtyp, velsys, lfreq0[nl], crval3, cdelt3, crpix3));
                int64_t kk0;
                int nk = line_profile(prof, vel[i], s, vedges + (size_t)nl * (nz + 1), cd2i, kc, K, nz, &kk0);
                double amp = w[i] * relint[nl];
                for (int j = 0; j < nk; j++) {
                    int64_t kz = kk0 + j;
                    if (kz < k0 || kz >= k1) continue;
                    double pv = amp * prof[j];
                    if (pv == 0.) continue;
                    for (int dy = 0; dy < 2; dy++) {
                        int64_t yy = iy + dy;
                        if (yy < y0 || yy >= y1) continue;
                        double wy = dy == 1 ? fy : 1. - fy;
                        int64_t row = base + ((kz - k0) * by + (yy - y0)) * bx - x0;
                        for (int dx = 0; dx < 2; dx++) {
                            int64_t xx = ix + dx;
                            if (xx < x0 || xx >= x1) continue;
                            double wx = dx == 1 ? fx : 1. - fx;
                            rbuf[row + xx] += pv * wx * wy;
                        }
                    }
                }
            }
        }
    }
    free(prof);
}

/* bbarolo/windmodel.py:369-423. kern: (2hy+1, 2hx+1); kx, ky: the 1D kernels when separable. buf accumulated. */
void ref_wind_convolve_boxes(const double *rbuf, const int64_t *roffs, const int64_t *rboxes, int ncell,
                             const double *kern, int hy, int hx, const double *kx, const double *ky, int separable,
                             double *buf, const int64_t *offs, const int64_t *boxes) {
    int kw = 2 * hx + 1;
    for (int k = 0; k < ncell; k++) {
        const int64_t *R = rboxes + 6 * (size_t)k, *B = boxes + 6 * (size_t)k;
        int64_t rx0 = R[0], rx1 = R[1], ry0 = R[2], ry1 = R[3], rk0 = R[4], rk1 = R[5];
        int64_t x0 = B[0], x1 = B[1], y0 = B[2], y1 = B[3], k0 = B[4], k1 = B[5];
        if (rx1 <= rx0 || ry1 <= ry0 || rk1 <= rk0 || x1 <= x0 || y1 <= y0 || k1 <= k0) continue;
        int64_t rbx = rx1 - rx0, rby = ry1 - ry0, bx = x1 - x0, by = y1 - y0;
        int64_t za = rk0 > k0 ? rk0 : k0, zb = rk1 < k1 ? rk1 : k1;
        if (separable) {
            double *tmp = malloc(sizeof(double) * (size_t)(rby * bx));
            for (int64_t kz = za; kz < zb; kz++) {
                memset(tmp, 0, sizeof(double) * (size_t)(rby * bx));
                for (int64_t y = ry0; y < ry1; y++) {
                    const double *rrow = rbuf + roffs[k] + ((kz - rk0) * rby + (y - ry0)) * rbx - rx0;
                    for (int64_t x = rx0; x < rx1; x++) {
                        double v = rrow[x];
                        if (v == 0.) continue;
                        for (int jx = -hx; jx <= hx; jx++) {
                            int64_t xx = x + jx;
                            if (xx < x0 || xx >= x1) continue;
                            tmp[(y - ry0) * bx + (xx - x0)] += v * kx[jx + hx];
                        }
                    }
                }
                for (int64_t y = ry0; y < ry1; y++)
                    for (int jy = -hy; jy <= hy; jy++) {
                        int64_t yy = y + jy;
                        if (yy < y0 || yy >= y1) continue;
                        double f = ky[jy + hy];
                        double *row = buf + offs[k] + ((kz - k0) * by + (yy - y0)) * bx;
                        for (int64_t xx = 0; xx < bx; xx++) row[xx] += f * tmp[(y - ry0) * bx + xx];
                    }
            }
            free(tmp);
        } else {
            for (int64_t kz = za; kz < zb; kz++)
                for (int64_t y = ry0; y < ry1; y++) {
                    const double *rrow = rbuf + roffs[k] + ((kz - rk0) * rby + (y - ry0)) * rbx - rx0;
                    for (int64_t x = rx0; x < rx1; x++) {
                        double v = rrow[x];
                        if (v == 0.) continue;
                        for (int jy = -hy; jy <= hy; jy++) {
                            int64_t yy = y + jy;
                            if (yy < y0 || yy >= y1) continue;
                            double *row = buf + offs[k] + ((kz - k0) * by + (yy - y0)) * bx - x0;
                            for (int jx = -hx; jx <= hx; jx++) {
                                int64_t xx = x + jx;
                                if (xx < x0 || xx >= x1) continue;
                                row[xx] += v * kern[(jy + hy) * kw + jx + hx];
                            }
                        }
                    }
                }
        }
    }
}

/* bbarolo/windmodel.py:477-554: the voxel lists of the columns within lim (entries v != 0, |v| >= rel * the peak of
 * the column, wm != 0) and the normal equations from them: G[k, l] = sum(A_k A_l wm), b[k] = sum(A_k wd). wd, wm:
 * (nz, ny, nx). G (ncell x ncell) and b are overwritten. */
void ref_wind_normal(const double *buf, const int64_t *offs, const int64_t *boxes, int ncell, const double *wd,
                     const double *wm, int ny, int nx, const int64_t *lim, double rel, double *G, double *b) {
    int64_t lx = lim[1] - lim[0], ly = lim[3] - lim[2], nvox = lx * ly * (lim[5] - lim[4]);
    int64_t *start = calloc((size_t)nvox + 1, sizeof(int64_t));
    double *thr = malloc(sizeof(double) * (size_t)(ncell > 0 ? ncell : 1));
    for (int k = 0; k < ncell; k++) {
        double m = 0.;
        for (int64_t j = offs[k]; j < offs[k + 1]; j++) if (fabs(buf[j]) > m) m = fabs(buf[j]);
        thr[k] = rel * m;
    }
#define WIND_ENTRIES(BODY)                                                                                      \
    for (int k = 0; k < ncell; k++) {                                                                           \
        const int64_t *B = boxes + 6 * (size_t)k;                                                               \
        int64_t x0 = B[0], x1 = B[1], y0 = B[2], y1 = B[3], k0 = B[4], k1 = B[5];                               \
        if (x1 <= x0 || y1 <= y0 || k1 <= k0) continue;                                                         \
        int64_t bx = x1 - x0, by = y1 - y0;                                                                     \
        for (int64_t kz = k0; kz < k1; kz++)                                                                    \
            for (int64_t y = y0; y < y1; y++) {                                                                 \
                int64_t row = offs[k] + ((kz - k0) * by + (y - y0)) * bx - x0;                                  \
                int64_t vrow = ((kz - lim[4]) * ly + (y - lim[2])) * lx - lim[0];                               \
                for (int64_t x = x0; x < x1; x++) {                                                             \
                    double v = buf[row + x];                                                                    \
                    if (v != 0. && fabs(v) >= thr[k] && wm[((size_t)kz * ny + y) * nx + x] != 0.) { BODY }     \
                }                                                                                               \
            }                                                                                                   \
    }
    WIND_ENTRIES(start[vrow + x + 1]++;)
    for (int64_t i = 0; i < nvox; i++) start[i + 1] += start[i];
    int64_t ne = start[nvox];
    int32_t *cell = malloc(sizeof(int32_t) * (size_t)(ne > 0 ? ne : 1));
    double *val = malloc(sizeof(double) * (size_t)(ne > 0 ? ne : 1));
    int64_t *fill = malloc(sizeof(int64_t) * (size_t)(nvox > 0 ? nvox : 1));
    memcpy(fill, start, sizeof(int64_t) * (size_t)nvox);
    WIND_ENTRIES({ int64_t j = fill[vrow + x]; cell[j] = k; val[j] = v; fill[vrow + x] = j + 1; })
#undef WIND_ENTRIES
    memset(G, 0, sizeof(double) * (size_t)ncell * ncell);
    memset(b, 0, sizeof(double) * (size_t)ncell);
    for (int64_t i = 0; i < nvox; i++) {
        int64_t j0 = start[i], j1 = start[i + 1];
        if (j1 == j0) continue;
        int64_t x = lim[0] + i % lx, y = lim[2] + (i / lx) % ly, kz = lim[4] + i / (lx * ly);
        double wv = wm[((size_t)kz * ny + y) * nx + x], d = wd[((size_t)kz * ny + y) * nx + x];
        for (int64_t p = j0; p < j1; p++) {
            int kp = cell[p];
            double ap = val[p];
            b[kp] += ap * d;
            double wa = wv * ap;
            for (int64_t q = p; q < j1; q++) G[(size_t)kp * ncell + cell[q]] += wa * val[q];
        }
    }
    for (int k = 0; k < ncell; k++)
        for (int l = k + 1; l < ncell; l++) G[(size_t)l * ncell + k] = G[(size_t)k * ncell + l];
    free(start); free(thr); free(cell); free(val); free(fill);
}

/* bbarolo/windmodel.py:584-602: out (nz, ny, nx) += sum_k amp[k] A_k */
void ref_wind_scatter(double *out, int ny, int nx, const double *buf, const int64_t *offs, const int64_t *boxes,
                      int ncell, const double *amp) {
    for (int k = 0; k < ncell; k++) {
        double a = amp[k];
        if (a == 0.) continue;
        const int64_t *B = boxes + 6 * (size_t)k;
        int64_t x0 = B[0], x1 = B[1], y0 = B[2], y1 = B[3], k0 = B[4], k1 = B[5];
        if (x1 <= x0 || y1 <= y0 || k1 <= k0) continue;
        int64_t bx = x1 - x0, by = y1 - y0;
        for (int64_t kz = k0; kz < k1; kz++)
            for (int64_t y = y0; y < y1; y++) {
                int64_t row = offs[k] + ((kz - k0) * by + (y - y0)) * bx - x0;
                for (int64_t x = x0; x < x1; x++) out[((size_t)kz * ny + y) * nx + x] += a * buf[row + x];
            }
    }
}

/* ------------------------------------------------------------------ _galmod_wind (bbarolo/galmod.py:539-590)
 * GALWIND WTYPE 1: Monte-Carlo clouds on spherical shells of a bi-cone. out: (ny, nx, nz) float64, accumulated.
 * sr: (11, nsub): radius, vrot, vsph, vdisp, dens, inc, pa, openang, xpos, ypos, vsys (internal units). */
void ref_galmod_wind(double *out, int ny, int nx, int nz, const double *sr, int nsub, int ring_lo, int ring_hi,
                     uint64_t seed, double sep, const int64_t *nv, double cdens, int cmode, double pixarea,
                     double cdelt0, double cdelt1, double crota2, int64_t blo0, int64_t blo1, int64_t bhi0,
                     int64_t bhi1, double sig_instr, int axtyp, int velsys, int nlines, const double *lfreq0,
                     double crval3, double cdelt3, double crpix3, const double *relint, const double *cd2i) {
    (void)ny;
    uint64_t st[2];
    ref_rng_init(seed, st);
    for (int ir = ring_lo; ir < ring_hi; ir++) {
        double rtmp = SR(0, ir);
        int64_t nc = lround_ref(cdens * pow(SR(4, ir), (double)cmode) * 2 * M_PI * rtmp * sep / pixarea);
        if (nc == 0) continue;
        double vrottmp = SR(1, ir), vsphtmp = SR(2, ir);
        double opentmp = SR(7, ir) / 2.;
        double vdisptmp = sqrt(SR(3, ir) * SR(3, ir) + sig_instr * sig_instr);
        double vsystmp = SR(10, ir);
        double sinc = sin(SR(5, ir)), cinc = cos(SR(5, ir));
        double pa = SR(6, ir);
        double spa = sin(pa) * cos(crota2) + cos(pa) * sin(crota2);
        double cpa = cos(pa) * cos(crota2) - sin(pa) * sin(crota2);
        int64_t nvr = nv[ir];
        double fluxsc = SR(4, ir) * 2 * M_PI * rtmp * sep / (double)(nc * nvr);
        double r_in2 = pow(rtmp - 0.5 * sep, 2.0);           /* (the reference's float ** 2) */
        for (int64_t ic = 0; ic < nc; ic++) {
            double rad = sqrt(r_in2 + 2 * sep * rtmp * fabs(2.0 * ref_rng_uniform(st) - 1.0));
            double az = 2 * M_PI * fabs(2.0 * ref_rng_uniform(st) - 1.0);
            double saz = sin(az), caz = cos(az);
            double ph = opentmp * fabs(2.0 * ref_rng_uniform(st) - 1.0);
            if (ic % 2 == 0) ph = M_PI - ph;
            double sphi = sin(ph), cphi = cos(ph);
            double R = rad * sphi, z = rad * cphi;
            double x = R * caz;
            double y = R * saz * cinc - z * sinc;
            int64_t g0 = lround_ref(SR(8, ir) + (x * spa - y * cpa) / cdelt0);
            int64_t g1 = lround_ref(SR(9, ir) + (x * cpa + y * spa) / cdelt1);
            if (g0 < blo0 || g0 >= bhi0 || g1 < blo1 || g1 >= bhi1) {
                for (int64_t iv = 0; iv < nvr; iv++) ref_rng_normal(st);
                continue;
            }
            int64_t px = g0 - blo0, py = g1 - blo1;
            double vs = vsystmp + vsphtmp * (cphi * cinc + sphi * saz * sinc) + vrottmp * caz * sinc;
            double *o = out + ((size_t)py * nx + (size_t)px) * nz;
            for (int64_t iv = 0; iv < nvr; iv++) {
                double v = vs + ref_rng_normal(st) * vdisptmp;
                for (int nl = 0; nl < nlines; nl++) {
                    int64_t isubs = lround_ref(velgrid(v, axtyp, velsys, lfreq0[nl], crval3, cdelt3, crpix3));
                    if (isubs < 0 || isubs >= nz) continue;
                    o[isubs] += relint[nl] * fluxsc * cd2i[isubs];
                }
            }
        }
    }
}
