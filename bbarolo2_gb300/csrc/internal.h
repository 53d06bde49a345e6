// Shared definitions of the bbgpu runtime: host set-up (C++) and device kernels (CUDA).
#pragma once

#include <stdint.h>
#include <string.h>
#include <stddef.h>

#ifdef __cplusplus
#include <string>
#include <unordered_map>
#include <vector>
#endif

#define BBGPU_MAXL 4          // emission lines supported by the device path
#define BBGPU_MAXK 511        // largest beam kernel side (the reference's FFT convolver: below 512)
#define BBGPU_NSR 16          // rows of a sub-ring table

// Per (member, sub-ring) parameters of the MC deposit. f64 fields reproduce the reference's arithmetic
// exactly (exact path); f32 fields are the coefficients of the fast path, whose rounding is bounded.
struct SubMC {
    // exact (f64)
    double xpos, ypos, spa, cpa, sinc, cinc, z0, zcyl, dvdz, vrot, vrad, vvert, vsys, vdisptmp, wrec, wapp;
    double valrel[BBGPU_MAXL];      // relint[nl] * float32(fluxsc) (times wside at deposit)
    // fast path (f32)
    float P1, P2, P3, Q1, Q2, Q3, xposf, yposf;
    float c0[BBGPU_MAXL], sg[BBGPU_MAXL];   // channel = c0 + (vr caz + vrad saz) sia + n sg
    float sia[BBGPU_MAXL];
    float z0f, zcylf, dvdzf, vrotf, vradf, pad0;
    // deposits in fixed point: round(relint * fluxsc * wside * Q) for the receding / approaching half
    long long fix[2][BBGPU_MAXL];
    int nc, nv, cloud_base, active;
};

// Per (member, sub-ring) parameters of the ANALYTIC deposit (bbarolo/galmod.py:347-374), float64 as the
// reference. fluxsc: dens * ring area / samples for models, ring area / samples for ring maps.
struct AnSub {
    double xpos, ypos, spa, cpa, sinc, cinc, z0, zcyl, dvdz, vrot, vrad, vvert, vsys, inv, wrec, wapp, fluxsc;
    double R[2];                    // radius of the two radial samples
    double a[BBGPU_MAXL];           // relint[nl] * fluxsc (times wside at deposit)
    long long K;                    // half-width of the line profile in channels
    int naz, nzz, zq_off, zdep, active, sub;
    // float32 fast path of the pixels (ring maps of the flux normalisation; error bounded in the kernel):
    // x pixel = xposf + (R caz P1 - R saz P2) + z P3, y pixel = yposf + (R caz Q1 + R saz Q2) + z Q3
    float P1, P2, P3, Q1, Q2, Q3, xposf, yposf, z0f, fluxscf, wrecf, wappf;
    float Rf[2];
    // the float32 residuals of the same constants (value - float32 value): the float-float evaluation of the
    // pixel (about 44 bits) when the float32 one is too close to a rounding boundary
    float P1l, P2l, P3l, Q1l, Q2l, Q3l, xposl, yposl, z0l;
    float Rl[2];
    int wzero;                      // bit 0: wrec == 0, bit 1: wapp == 0 (the float64 tests, done on the host)
    // float32 fast path of a model (one line, a linear channel map, a velocity independent of the height):
    // anfast = 1 when it applies, invf = 1 / sig
    int anfast;
    float invf;
    // float-float (hi, lo) copies of the velocity terms and the line amplitude relint[0] fluxsc in float32 (the
    // fast path's line without float64 arithmetic)
    float vsysh, vsysl, vroth, vrotl, vradh, vradl, vverth, vvertl, sinch, sincl, cinch, cincl, af;
};

// The constants of a context, as the kernels see them.
struct GridDev {
    int nx, ny, nz, nlines, axtyp, velsys, ltype, cmode;
    int fast_ok;                    // the channel map is linear in velocity (fast path usable)
    int pad;
    double radsep, cdens, pixarea, cdelt0, cdelt1, crota2, sig_instr, crval3, cdelt3, crpix3, chwidth, zstep;
    double scalefactor, ia, ib;
    double lfreq0[BBGPU_MAXL], relint[BBGPU_MAXL];
    float lia[BBGPU_MAXL], lib[BBGPU_MAXL];  // channel = v * lia + lib per line (fast path)
    // ANALYTIC fast path (one line, linear map): channel = v ia0 + ib0 in float64 (ia0, ib0 of line 0), and the
    // reference velocity vref (the channel edges are kept relative to it in float-float)
    double ia0, ib0, vref;
    float ia0h, ia0l, ib0h, ib0l, vrefh, vrefl;  // (float-float copies)
};

// A parsed MC stream (host copy): everything about the clouds that does not depend on the ring parameters.
struct LayoutHost {
    uint64_t key;
    int nsub, ncloud;
    long long nsubcloud;
    // per sub-ring
    int *nc, *nv, *cloud_base;
    long long *sub_base;            // offset of the sub-ring's first sub-cloud in hz
    // per cloud
    double *R, *caz, *saz, *fdev;
    int *sub;                       // sub-ring of the cloud
    int *slow_base;                 // slow normals before this cloud
    // per sub-cloud: the high word (minus 2^31) of the first draw of its normal
    int32_t *hz;
    // the values of the normals that took the slow path of the ziggurat, in stream order
    double *slow_val;
    long long nslow;
};

#ifdef __cplusplus
// GALWIND WTYPE 1 (bbarolo/galmod.py:539-590): the constants of a shell with clouds, and the clouds of a stream
struct WindShell {
    double fluxsc, vdisp, vsys, vsph, vrot, sinc, cinc, spa, cpa, xpos, ypos;
    int nvr, pad;
};

#ifdef __cplusplus
struct WindClouds {
    std::vector<WindShell> shells;
    std::vector<int> shell;             // per cloud: its shell (index into shells)
    std::vector<double> geo;            // per cloud: rad, cos az, sin az, sin ph, cos ph
    std::vector<long long> nbase;       // per cloud: its first velocity deviate in hz
    std::vector<long long> sbase;       // per cloud: its first deviate in slow
    std::vector<int32_t> hz;            // the velocity deviates in stream order: the first word of each ziggurat
    std::vector<double> slow;           // the values of the deviates that left the ziggurat's one-word path
    double total = 0.;                  // sum over the clouds of nvr x fluxsc
};
#endif

extern "C++" {
// host_setup.cpp
// the stream of _galmod_wind for the shells [lo, hi) of sr (11, nsub): per cloud its radius, azimuth, polar angle
// and velocity deviates (all drawn, as the reference, also for clouds outside any box); 0 or a negative error
int bbh_wind_clouds(WindClouds *W, uint64_t seed, const double *sr, int nsub, int lo, int hi, double sep,
                    const int64_t *nv, const GridDev *g);
void bbh_zig_tables(int64_t *kn, double *wn, double *fn);
void bbh_phi_table(double *tab);      // 6146 entries
int bbh_layout_build(LayoutHost *L, uint64_t seed, int ltype, int nsub, const int *nc, const int *nv,
                     const double *R0, double radsep);
void bbh_layout_free(LayoutHost *L);
uint64_t bbh_layout_key(uint64_t seed, int ltype, int nsub, const int *nc, const int *nv, const double *R0,
                        double radsep);
// nc and nv of each sub-ring of a table (the reference's cloud count)
void bbh_cloud_counts(const double *sr, int nsub, const int64_t *nv_in, const GridDev *g, int *nc, int *nv);
// SubMC of one table; returns the exponent e of the fixed-point unit 2^-e of its deposits
// (sr_ref, out_ref: another member's table and constants, reused for the columns that are equal; may be NULL;
// reused: when given, those columns are only marked (1) and left unwritten, for the device to fill; diff: when
// given, bbh_column_diff(sr, sr_ref) computed by the caller)
int bbh_submc(const double *sr, int nsub, const int *nc, const int *nv, const GridDev *g, SubMC *out,
              const double *sr_ref = nullptr, const SubMC *out_ref = nullptr, signed char *reused = nullptr,
              const uint16_t *diff = nullptr);
// ANALYTIC: the vertical samples of a sub-ring (bbarolo/galmod.py:276-323); returns their number
int bbh_zgrid(double *zq, double *wq, int nmax, int ltype, double z0, double sinc, double pixsize, double dvdz,
              double sig, double R0, double radsep, double xpos, double ypos, double cdelt0, double cdelt1,
              long long blo0, long long blo1, long long bhi0, long long bhi1, double zstep);
// ANALYTIC: the azimuthal samples of the sub-rings of radii R0 (they depend on R0 and the pixel area only):
// sbase (nsub + 1) first sample of each sub-ring, ssub the sub-ring of each sample, cs (2 per sample) the
// cos/sin of its azimuth from the reference's rotation recurrence (bbarolo/galmod.py:384-391)
void bbh_an_samples(const double *R0, int nsub, const GridDev *g, std::vector<int> &sbase, std::vector<int> &ssub,
                    std::vector<double> &cs);
// float32 copy of cs with the half of each sample in the sign bit of its cosine: +0 / positive for caz >= 0
// (receding half, the reference's test on the float64 value), negative for caz < 0
void bbh_an_samples_f32(const std::vector<double> &cs, std::vector<float> &csf);
// ANALYTIC: the AnSub of each sub-ring of a table (maps: ring-map mode, active where widx has a ring), their
// vertical samples appended to zq/wq; returns the fixed-point exponent e (deposits in units of 2^-e) or
// -10000 when the total flux is not finite
// The vertical sample grids of the ANALYTIC sub-rings, shared by all the sub-rings with the same inputs of _zgrid:
// one table (append-only), each grid stored once (the fits change few geometries between evaluations).
// the inputs of _zgrid (a thin layer: all zero but iv[0] = -1)
struct ZKey {
    double dv[12];
    long long iv[6];
    bool operator==(const ZKey &o) const { return !memcmp(this, &o, sizeof *this); }
};
struct ZKeyHash {
    size_t operator()(const ZKey &k) const {
        uint64_t h = 1469598103934665603ull, w[18];
        memcpy(w, &k, sizeof w);
        for (int i = 0; i < 18; i++) {
            h = (h ^ w[i]) * 1099511628211ull;
            h ^= h >> 29;
        }
        return (size_t)h;
    }
};
struct ZgridCache {
    std::unordered_map<ZKey, std::pair<int, int>, ZKeyHash> map;   // inputs -> (offset, samples)
    std::vector<double> zq, wq;
    size_t uploaded = 0;                                         // entries already copied to the device
    void clear() {
        map.clear();
        zq.clear();
        wq.clear();
        uploaded = 0;
    }
};
int bbh_an_subs(const double *sr, int nsub, const GridDev *g, int nzq, int blo0, int blo1, int bhi0, int bhi1,
                const double *cd2i, int maps, const int64_t *widx, const double *wval, AnSub *out, ZgridCache &zc,
                const double *sr_ref = nullptr, const AnSub *out_ref = nullptr, signed char *reused = nullptr,
                const uint16_t *diff = nullptr);
// per column of the tables a and b (16 rows, nsub columns): the bit mask of the rows whose values differ (bitwise)
void bbh_column_diff(const double *a, const double *b, int nsub, uint16_t *mask);
// true if a column with the row mask m gives the same ring-map constants in bbh_an_subs (maps mode): the same
// radius, scale height, velocity gradient, inclination, position angle, centre and side weights, and the same
// dispersion where a velocity gradient makes the vertical grid depend on it (a: the column's table; the
// velocities and the density do not enter a ring map)
bool bbh_map_same(uint16_t m, const double *a, int nsub, int ir);
// (an MC column with the row mask m differs at most in the density, row 5: the same clouds, at the same pixels
// and channels, with another flux, when !(m & ~(1 << 5)))
// The second-difference prior of the deconvolved profile at the radii R (n) (bbarolo/profile.py:60-151):
// rows (n - 2) x 3 columns lc and weights lv, the order of the radii, the "near" rows, the median ring
// distance d and the norm of the relative prior
void bbh_profile_consts(const double *R, int n, int *lc, double *lv, int *ord, unsigned char *near, double *d,
                        double *norm);
// The pixels of a ring for the CLASSIC residual (bbarolo/galfit.py:62-93): inside flags and weights (bsy, bsx)
void bbh_norm_footprint(int bsy, int bsx, double x0, double y0, double phi, double inc, double r1, double r2,
                        double wpow, int side, int foot, double hmax, uint8_t *inside, double *wmap);
}
#endif
