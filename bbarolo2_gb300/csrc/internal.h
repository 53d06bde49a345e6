// Shared definitions of the bbgpu runtime: host set-up (C++) and device kernels (CUDA).
#pragma once

#include <stdint.h>
#include <stddef.h>

#define BBGPU_MAXL 4          // emission lines supported by the device path
#define BBGPU_MAXK 63         // largest beam kernel side
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

// Per (member, sub-ring) parameters of the ANALYTIC deposit.
struct SubAN {
    double xpos, ypos, spa, cpa, sinc, cinc, z0, zcyl, dvdz, vrot, vrad, vvert, vsys, sig, wrec, wapp, R0;
    double fluxsc, r_inner, cd, sd;
    int naz, K, nzz, zq_off;        // azimuths, line half-window, vertical samples (offset in the zq table)
    int zdep, active, sample_base, pad;
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
extern "C++" {
// host_setup.cpp
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
int bbh_submc(const double *sr, int nsub, const int *nc, const int *nv, const GridDev *g, SubMC *out);
// The pixels of a ring for the CLASSIC residual (bbarolo/galfit.py:62-93): inside flags and weights (bsy, bsx)
void bbh_norm_footprint(int bsy, int bsx, double x0, double y0, double phi, double inc, double r1, double r2,
                        double wpow, int side, int foot, double hmax, uint8_t *inside, double *wmap);
}
#endif
