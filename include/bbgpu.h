/*
 * bbgpu: the C ABI of the GB300 (sm_103a) model-evaluation path of BBarolo 2's 3DFIT.
 *
 * Plain C types only (pointers, sizes, doubles). Every function returns an int status (BBGPU_OK = 0, or a
 * negative code; bbgpu_last_error() gives the message of the last failure of the context) and never throws
 * or aborts. Host arrays are caller-owned and C-contiguous; device buffers are owned by the context.
 *
 * Reference interfaces replaced (paths within the reference project):
 *   bbgpu_galmod_mc           <- _galmod_mc(out, sr, ring_lo, ring_hi, seed, radsep, nv, ...)   bbarolo/galmod.py:92-95
 *   bbgpu_galmod_analytic     <- _galmod_analytic(out, sr, ring_lo, ring_hi, ...)                bbarolo/galmod.py:326-329
 *   bbgpu_ring_maps_analytic  <- _ring_maps_analytic(out, sr, widx, wval, ...)                   bbarolo/galmod.py:468-470
 *   bbgpu_convolve            <- FFTConvolver.__call__(data, workers) + the threshold and scale of
 *                                DiskModel.convolve(mod, layout, workers)                          bbarolo/smooth.py:145, bbarolo/galmod.py:1273
 *   bbgpu_conv_sparse         <- _conv_sparse(model, kern, scale)                                 bbarolo/galmod.py:974-975
 *   bbgpu_sumsq_residuals     <- _sumsq_residuals(model, data, mask, maskmode, region)            bbarolo/bayesian/likelihood.py:22-23
 *   bbgpu_residuals_fracerr   <- _residuals_fracerr(model, data, mask, maskmode, region, s2, e2)  bbarolo/bayesian/likelihood.py:48-49
 *   bbgpu_norm                <- _norm(model, data, mask, blo0, blo1, x0, y0, phi, inc, ...)      bbarolo/galfit.py:39-41
 *   bbgpu_eval_*              <- LikelihoodMixin._log_likelihood(theta) for a batch of theta:
 *                                DiskModel.array -> convolve -> _calculate_residuals             bbarolo/bayesian/likelihood.py:567-619
 *   bbgpu_galmod_wind         <- _galmod_wind(out, sr, ring_lo, ring_hi, seed, sep, nv, ...)      bbarolo/galmod.py:539-542
 *   bbgpu_galwind_spherical   <- GalWind._spherical(out): the chunks of shells and their seeds    bbarolo/galwind.py:301-331
 *   bbgpu_wind_points         <- _wind_points(cells, qn, qoff, radii, vw, vd, vr, ...)            bbarolo/windmodel.py:225-227
 *   bbgpu_wind_boxes          <- WindModel.boxes(p, lim, pts, weight): _raw_boxes, _deposit_raw,
 *                                _convolve_boxes                                                   bbarolo/windmodel.py:829-859
 *   bbgpu_wind_normal         <- Boxes.voxel_lists(wm, lim, rel) + Boxes.normal(wd, wm, lists)    bbarolo/windmodel.py:672-687
 *   bbgpu_wind_model          <- Boxes.model(amp, shape) (_scatter)                               bbarolo/windmodel.py:584-585, 657
 *
 * Layouts follow the reference: sub-ring tables sr (16, nsub) float64 in internal units (row order of
 * GalmodSetup.subrings, bbarolo/galmod.py:761-851); models (ny, nx, nz) float64 ("yxz"); cubes (nz, ny, nx).
 */
#ifndef BBGPU_H
#define BBGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    BBGPU_OK = 0,
    BBGPU_ERR_ARG = -1,       /* invalid argument (shape, size, null pointer, unsupported option) */
    BBGPU_ERR_CUDA = -2,      /* a CUDA runtime call failed */
    BBGPU_ERR_NOMEM = -3,     /* device or host allocation failed */
    BBGPU_ERR_STATE = -4,     /* call out of order (e.g. evaluation before bbgpu_set_grid) */
    BBGPU_ERR_KERNEL = -5     /* a kernel reported an inconsistency (its error flag) */
};

enum { BBGPU_MC = 0, BBGPU_ANALYTIC = 1 };

typedef struct bbgpu_ctx bbgpu_ctx;

/* The header-derived constants of a cube (GalmodSetup, bbarolo/galmod.py:613-725). */
typedef struct {
    int nx, ny, nz;           /* cube dimensions */
    int nlines;               /* number of emission lines (lfreq0, relint) */
    int axtyp, velsys;        /* spectral axis: 2 wave, 3 freq, 4 velocity; 1 radio, 2 optical, 3 relativistic */
    int ltype, cmode;         /* vertical layer (1..5), cloud-number mode (0..2) */
    double radsep, cdens, pixarea, cdelt0, cdelt1, crota2, sig_instr;
    double crval3, cdelt3, crpix3;
    double chwidth;           /* narrowest channel in velocity (GalmodSetup._chmin): ANALYTIC line windows */
    double zstep;             /* vertical sample spacing of the ANALYTIC models (pixels) */
    double scalefactor;       /* flux scale of the convolution (1 for DENSFLUX) */
} bbgpu_grid;

/* One evaluation of a batch: the model of one sub-ring table in a box, convolved, compared with the cube. */
typedef struct {
    int32_t blo0, blo1, bhi0, bhi1;   /* model box [blo, bhi) in pixels (x, y) */
    uint64_t seed;            /* MC stream seed (ISEED & 0xFFFFFFFF) */
    int32_t maskmode;         /* residual mode: 0 all voxels, 1 data*mask, 2 voxels in the mask only */
    int32_t use_region;       /* 1: skip the pixels outside the region set with bbgpu_set_cube */
    double sigma2;            /* noise variance (fracerr mode) */
    double eps2;              /* fractional model error squared; 0: plain sum of squares */
} bbgpu_eval_desc;

/* ---- context ---------------------------------------------------------------------------------------- */
int bbgpu_ctx_create(bbgpu_ctx **out, int device);
int bbgpu_ctx_destroy(bbgpu_ctx *ctx);
const char *bbgpu_last_error(const bbgpu_ctx *ctx);
int bbgpu_version(void);

/* ---- set-up (once per cube / kernel) ------------------------------------------------------------------ */
/* cd2i (nz), lfreq0 (nlines), relint (nlines), vedges (nlines, nz+1) velocity channel edges per line. */
int bbgpu_set_grid(bbgpu_ctx *ctx, const bbgpu_grid *g, const double *cd2i, const double *lfreq0,
                   const double *relint, const double *vedges);
/* Beam kernel (ky, kx) float64 (bbarolo/smooth.py:62-88); ky, kx odd, at most 511 (the reference's FFT convolver
 * takes sides below 512). The float32 convolution stages its input tile in shared memory for widths up to 31 with
 * (16 + ky - 1) (16 + width - 1) 128 bytes within 220 KB (ky up to 23 at width 31) and reads wider kernels' inputs
 * from global memory (k_conv_wide); the tensor-core variants take ky <= 32 and widths <= 33, and the f32 kernel
 * runs when they cannot. */
int bbgpu_set_kernel(bbgpu_ctx *ctx, const double *kernel, int ky, int kx);
/* Cube data (nz, ny, nx) float32, mask (nz, ny, nx) uint8 or NULL, region (ny, nx) uint8 or NULL. */
int bbgpu_set_cube(bbgpu_ctx *ctx, const float *data, const uint8_t *mask, const uint8_t *region);

/* ---- reference-kernel entry points (one model per call; host arrays in and out) ------------------------ */
/* out (bhi1-blo1, bhi0-blo0, nz) float64 is ACCUMULATED (out +=), as the reference kernels. */
int bbgpu_galmod_mc(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int ring_lo, int ring_hi,
                    uint64_t seed, const int64_t *nv, int blo0, int blo1, int bhi0, int bhi1);
/* GALWIND WTYPE 1: the clouds of spherical shells. sr (11, nsub): radius, vrot, vsph, vdisp, dens, inc, pa,
 * openang, xpos, ypos, vsys (internal units); sep: the shells' thickness (arcmin); the grid's cdens, cmode,
 * pixarea, cdelt, crota2, sig_instr, spectral axis, lines and cd2i are those of bbgpu_set_grid. out (bhi1-blo1,
 * bhi0-blo0, nz) float64 is ACCUMULATED. */
int bbgpu_galmod_wind(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int ring_lo, int ring_hi,
                      uint64_t seed, double sep, const int64_t *nv, int blo0, int blo1, int bhi0, int bhi1);
/* GalWind._spherical (bbarolo/galwind.py:301-331): the chunks [chunk_lo[c], chunk_hi[c]) of the shells, each with
 * its own stream seeds[c], their streams parsed on up to `threads` host threads, all clouds deposited in one pass;
 * out += the sum of the chunks' models (the fixed-point sums are exact: the same as adding them one by one). */
int bbgpu_galwind_spherical(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int nchunks,
                            const int *chunk_lo, const int *chunk_hi, const uint64_t *seeds, double sep,
                            const int64_t *nv, int blo0, int blo1, int bhi0, int bhi1, int threads);
int bbgpu_galmod_analytic(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int ring_lo, int ring_hi,
                          int nzq, int blo0, int blo1, int bhi0, int bhi1);
/* out (nr, bhi1-blo1, bhi0-blo0) float64 accumulated; widx (nsub, 2) int64 (-1: none), wval (nsub, 2). */
int bbgpu_ring_maps_analytic(bbgpu_ctx *ctx, double *out, int nr, const double *sr, int nsub,
                             const int64_t *widx, const double *wval, int nzq, int blo0, int blo1, int bhi0,
                             int bhi1);
/* "same" convolution of each plane of in (nz, ny, nx) float64 with the kernel; threshold != 0: values
 * below 1e-12 set to zero, then x scale (DiskModel.convolve); out (nz, ny, nx) float64. */
int bbgpu_convolve(bbgpu_ctx *ctx, const double *in, double *out, int nz, int ny, int nx, double scale,
                   int threshold);
/* model (ny, nx, nz) float64 -> out (ny, nx, nz) float64 (bbarolo/galmod.py:974-1037). */
int bbgpu_conv_sparse(bbgpu_ctx *ctx, const double *model, double *out, int ny, int nx, int nz,
                      const double *kernel, int ky, int kx, double scale);
/* model (nz, ny, nx) float64, data float32 and mask uint8 of the same shape, region (ny, nx) or NULL. */
int bbgpu_sumsq_residuals(bbgpu_ctx *ctx, const double *model, const float *data, const uint8_t *mask,
                          int maskmode, const uint8_t *region, int nz, int ny, int nx, double *out);
int bbgpu_residuals_fracerr(bbgpu_ctx *ctx, const double *model, const float *data, const uint8_t *mask,
                            int maskmode, const uint8_t *region, int nz, int ny, int nx, double sigma2,
                            double eps2, double *out2);
/* CLASSIC normalisation + residual; model (bsy, bsx, nz) float64 is multiplied by the factor in place;
 * data float32 and mask uint8 (dny, dnx, nz) ("yxz"); pre (bsy, bsx, nz) or NULL (MC support emulation);
 * ilo, ihi (ky) int64; thr (nz). Result in *out. */
int bbgpu_norm(bbgpu_ctx *ctx, double *model, int bsy, int bsx, int nz, const float *data, const uint8_t *mask,
               int dny, int dnx, int64_t blo0, int64_t blo1, double x0, double y0, double phi, double inc,
               double r1, double r2, double wpow, int side, int ftype, const double *chan_noise,
               double data_noise, double bweight, int normtype, const double *pre, const int64_t *ilo,
               const int64_t *ihi, int ky, const double *thr, int foot, double hmax, double *out);

/* ---- flux normalisation of the batched likelihood ------------------------------------------------------ */
/* The deconvolved density profile of each member, recomputed on the device at every evaluation, as
 * Bayesian3DFIT does when DENS is not fitted and the geometry is free (bbarolo/bayesian/likelihood.py:595-596,
 * bbarolo/bayesian/density.py:39-88, bbarolo/profile.py:33-138). Set once per fit: the likelihood box, the data
 * map ymap, its noise rms and the pixels to use ok (all (bhi1-blo1, bhi0-blo0)), the radii of the nr rings and of
 * the exterior annulus (nr + 1, nr + 1 <= 64), the prior (smooth, corr, floor as solve_profile) and mapscale =
 * mean(cd2i) x sum(relint) x the beam scale factor (DiskModel.ring_maps). */
int bbgpu_set_profile(bbgpu_ctx *ctx, int nr, int blo0, int blo1, int bhi0, int bhi1, const double *ymap,
                      const double *rms, const uint8_t *ok, const double *radii, double smooth, double corr,
                      double floor_, double mapscale);
/* Per MC batch, after bbgpu_eval_upload: the sub-rings of the ring maps of every member, sr_maps (nb, 16, nsm):
 * the model's sub-rings (the first nsub, as uploaded) then those of the exterior annulus; widx, wval (nsm, 2)
 * the map of each sub-ring and its weight (-1: none). eval_run then computes the maps, their convolution, the
 * normal equations and the profile, and sets the densities of the model's sub-rings before the MC model. */
int bbgpu_eval_upload_profile(bbgpu_ctx *ctx, int nsm, const double *sr_maps, const int64_t *widx,
                              const double *wval);
/* The densities of the last run: x (nb, nr + 1), status (nb; 0 = converged, or NULL). */
int bbgpu_eval_profile(bbgpu_ctx *ctx, double *x, int *status);
/* solve_profile(A, b, radii, smooth, corr, floor) on the device: A (m, n) row-major, b (m), radii (n); x (n).
 * status: 0 converged, 1 a passive block not positive definite, 2 iteration limit (or NULL).
 * (Replaces the profile constants set by bbgpu_set_profile.) */
int bbgpu_solve_profile(bbgpu_ctx *ctx, const double *A, const double *b, int m, int n, const double *radii,
                        double smooth, double corr, double floor_, double *x, int *status);

/* ---- batched likelihood path ------------------------------------------------------------------------- */
/* A batch of nb evaluations of the same sub-ring count nsub: sr (nb, 16, nsub) float64, nv (nb, nsub) int64,
 * descs (nb). The GALMOD model (galmodtype), the beam convolution (if a kernel is set), the threshold and
 * scale, and the residual over the box are computed on the device; ss (nb) receives the sum of squares
 * (fracerr: the variance-weighted sum) and lg (nb, may be NULL) the sum of log(v / sigma2).
 * bbgpu_eval_upload copies the batch to the device, bbgpu_eval_run computes it on the device (inputs
 * resident), bbgpu_eval_download copies the results; bbgpu_eval_batch does the three. */
int bbgpu_eval_upload(bbgpu_ctx *ctx, int galmodtype, int nb, int nsub, const double *sr, const int64_t *nv,
                      const bbgpu_eval_desc *descs);
int bbgpu_eval_run(bbgpu_ctx *ctx);
int bbgpu_eval_download(bbgpu_ctx *ctx, double *ss, double *lg);
int bbgpu_eval_batch(bbgpu_ctx *ctx, int galmodtype, int nb, int nsub, const double *sr, const int64_t *nv,
                     const bbgpu_eval_desc *descs, double *ss, double *lg);
/* The smoothed (or unsmoothed, smoothed = 0) model of member k of the last batch run: (by, bx, nz) float32. */
int bbgpu_eval_model(bbgpu_ctx *ctx, int k, int smoothed, float *out, int by, int bx, int nz);
/* Synchronise the context's stream. */
int bbgpu_sync(bbgpu_ctx *ctx);
/* Options: 1 keep the smoothed models of a batch (for bbgpu_eval_model), 2 time the kernels of each run,
 * 3 compute the members of a batch that differ from the first member in a few sub-rings (the steps of a
 * finite-difference gradient) as the first member's ring maps, profile and MC model plus the difference (default
 * 1; the results are the same bit for bit, 0 computes every member from all its samples and clouds);
 * 4 the beam convolution of the batch models: 0 float32 FMA, 1 bf16x3 or 2 tf32x3 on the tensor cores (split
 * products, FP32 accumulation), -1 (default) the faster of float32 and tf32x3, timed on the first batch of each
 * kernel shape and channel count and kept for the context's lifetime. float32 and tf32x3 keep every smoothed
 * voxel within 1e-5 of the float64 convolution; bf16x3 within about 2e-5 (its split), so it is never chosen
 * automatically. The ring maps of the flux normalisation always use float32;
 * 5 CUDA graphs (default 1): the second bbgpu_eval_run of an unchanged batch (nothing uploaded, set or
 * reallocated since the first) is captured into a graph, both streams included, and later runs of that batch
 * replay it; 0 launches every kernel each run. The stage timers (option 2) run without a graph. */
int bbgpu_set_option(bbgpu_ctx *ctx, int option, int value);

/* The graph of the current batch: replays so far in the context, kernels per replay (0: no graph for the current
 * state). No counterpart in the reference. */
int bbgpu_graph_stats(const bbgpu_ctx *ctx, int64_t *replays, int64_t *kernels);

/* The variant of the last batch convolution (0 float32, 1 bf16x3, 2 tf32x3) and the autotuner's timings of a batch
 * convolution in ms per variant (-1: not timed). No counterpart in the reference (its convolution is scipy's FFT). */
int bbgpu_conv_variant(const bbgpu_ctx *ctx, int *used, float *tune_ms);

/* ---- the surrogate of the log-likelihood ------------------------------------------------------------------- */
/* A multilayer perceptron d_in -> hidden -> hidden -> hidden -> 1 (GELU) trained online on the likelihood evaluations
 * of a sampler, to screen its proposals. No counterpart in the reference (its nested sampler trains neural bounds in
 * numba, bbarolo/bayesian/nautilus/mlp.py:18-118, and bounds/neural.py). BF16 weights and activations in the
 * products, FP32 accumulation, FP32 master weights and Adam (beta 0.9, 0.999, eps 1e-8). Inputs x (n, d_in) and
 * targets t (n) float32 host arrays; the loss is the mean squared error. Parameters (float32, flattened): W1
 * (hidden, d_in), b1, W2 (hidden, hidden), b2, W3, b3, w4 (hidden), b4. */
typedef struct bbgpu_mlp bbgpu_mlp;
int bbgpu_mlp_create(bbgpu_mlp **out, int device, int d_in, int hidden, uint64_t seed);
int bbgpu_mlp_destroy(bbgpu_mlp *m);
long long bbgpu_mlp_nparams(const bbgpu_mlp *m);
int bbgpu_mlp_get_params(const bbgpu_mlp *m, float *params);
int bbgpu_mlp_set_params(bbgpu_mlp *m, const float *params);      /* (also resets Adam) */
int bbgpu_mlp_predict(bbgpu_mlp *m, const float *x, int n, float *y);
int bbgpu_mlp_gradients(bbgpu_mlp *m, const float *x, const float *t, int n, float *grads, float *loss);
int bbgpu_mlp_train_step(bbgpu_mlp *m, const float *x, const float *t, int n, float lr, float *loss);
/* `steps` Adam steps on minibatches of `batch` rows drawn with replacement (a hash of seed, step and row) from the
 * training set x (n, d_in), t (n), which is copied to the device once: one call, one synchronisation. loss: the
 * mean squared error of the last minibatch (before its step). n < 2^31. */
int bbgpu_mlp_train(bbgpu_mlp *m, const float *x, const float *t, long long n, int steps, int batch, float lr,
                    uint64_t seed, float *loss);

/* ---- bi-conical wind models (WINDFIT) ------------------------------------------------------------------ */
/* The column engine of the wind models: a handle per cube (its spectral axis, lines and beam) and grid of cells
 * (bbarolo/windmodel.py:89-210, 706-803). A column is the model of one cell for unit amplitude, a dense box
 * (x0, x1, y0, y1, k0, k1) of the cube ([lo, hi), values in (channel, y, x) order from the column's offset). */
typedef struct bbgpu_wind bbgpu_wind;
typedef struct {
    int nx, ny, nz;           /* cube dimensions */
    int nlines;               /* emission lines (at most 4) */
    int axtyp, velsys;        /* spectral axis, as bbgpu_grid */
    double cdelt0, cdelt1;    /* arcsec per pixel with the sign of CDELT (WindModel.cdelt) */
    double sig_instr;         /* instrumental dispersion (m/s) */
    double chmin;             /* narrowest channel in velocity (m/s; GalmodSetup._chmin) */
    double crval3, cdelt3, crpix3;
} bbgpu_wind_grid;
/* The geometry of one wind (WindModel.points, bbarolo/windmodel.py:808-827): centre (pixels), VSYS (m/s), sin and
 * cos of INC and of PA + CROTA, the half opening angles OPENIN/2 and OPENANG/2 (radians) and CONELEN (arcsec). */
typedef struct {
    double x0, y0, vsys, sinc, cinc, spa, cpa, th_in, th_out, rmax;
} bbgpu_wind_pars;
/* lfreq0, relint (nlines); vedges (nlines, nz + 1): the velocity of the channel edges per line; kern (2hy+1,
 * 2hx+1) the beam kernel, hx = hy = 0 for the bilinear deposit alone; separable: kx (2hx+1), ky (2hy+1). */
int bbgpu_wind_create(bbgpu_wind **out, int device, const bbgpu_wind_grid *g, const double *lfreq0,
                      const double *relint, const double *vedges, const double *kern, int hy, int hx, const double *kx,
                      const double *ky, int separable);
int bbgpu_wind_destroy(bbgpu_wind *w);
const char *bbgpu_wind_last_error(const bbgpu_wind *w);
int64_t bbgpu_wind_launch_count(const bbgpu_wind *w);
/* The cells (ncell, 7: cone, r0, r1, theta0, theta1, phi0, phi1; arcsec and radians), their quadrature counts qn
 * (ncell, 3) and point offsets qoff (ncell + 1) (WindCells.cells, qn, qoff). At most 16384 cells, 2^31 - 1 points. */
int bbgpu_wind_set_cells(bbgpu_wind *w, int ncell, const double *cells, const int64_t *qn, const int64_t *qoff);
/* The quadrature points of the wind p (radii, vwind, vdisp, vrot: nrad <= 256 shells, arcsec and km/s), kept on the
 * device; the non-NULL outputs are filled (gx, gy, vel, sig, wt, r per point; vol, rbar per cell). */
int bbgpu_wind_points(bbgpu_wind *w, const bbgpu_wind_pars *p, int nrad, const double *radii, const double *vwind,
                      const double *vdisp, const double *vrot, double *gx, double *gy, double *vel, double *sig,
                      double *wt, double *r, double *vol, double *rbar);
/* Points given by the caller instead (gx, gy, vel, sig, weights; one per quadrature point). */
int bbgpu_wind_set_points(bbgpu_wind *w, const double *gx, const double *gy, const double *vel, const double *sig,
                          const double *wt);
/* The columns of the current points within lim (6: x0, x1, y0, y1, k0, k1 of the cube), the points' weights times
 * weight (one per point, or NULL); boxes (ncell, 6) and total (the number of column values) returned. */
int bbgpu_wind_boxes(bbgpu_wind *w, const int64_t *lim, const double *weight, int64_t *boxes, int64_t *total);
/* The column values (total) and their offsets (ncell + 1). */
int bbgpu_wind_columns(bbgpu_wind *w, double *buf, int64_t *offs);
/* The weights wm and the weighted data wd = wm * data (nz, ny, nx) of the normal equations, kept on the device. */
int bbgpu_wind_set_weights(bbgpu_wind *w, const double *wm, const double *wd);
/* G (ncell, ncell) = A'WA and b (ncell) = A'Wd over the voxel lists of the columns within lim (6 integers, NULL:
 * the cube; the columns must lie inside it): the values != 0, |value| >= rel x the peak of their column, wm != 0. */
int bbgpu_wind_normal(bbgpu_wind *w, const int64_t *lim, double rel, double *G, double *b);
/* out (nz, ny, nx) = sum_k amp[k] column k. */
int bbgpu_wind_model(bbgpu_wind *w, const double *amp, double *out);

/* ---- without allocation ------------------------------------------------------------------------------- */
/* bbgpu_sumsq_residuals / bbgpu_residuals_fracerr for callers that may not allocate device memory (their own
 * memory pool, a fixed footprint after warm-up). No counterpart in
 * the reference: it exists for such callers. Needs no context. model (nz, ny, nx) float64, data float32, mask
 * and region uint8 and out2 (double[2]: sum of squares or variance-weighted sum, sum of log-variances) are
 * DEVICE pointers of the current device; eps2 = 0 gives the plain sum of squares. Kernels run on stream
 * (cudaStream_t, NULL: the default stream) and out2 is written there. The partial sums use a 64 KB scratch
 * array held by every GPU that loads the library; at most 16,777,216 voxels (4096 blocks of 4096) per call,
 * BBGPU_ERR_ARG beyond (and for a negative or NaN eps2). The first call on a device looks the array's address up
 * (cudaGetSymbolAddress) and keeps it: do not reset the device
 * (cudaDeviceReset) between calls. A CUDA error pending from earlier work makes the call return BBGPU_ERR_CUDA
 * without launching. Calls whose kernels overlap on the GPU share the array and race. */
int bbgpu_sumsq_residuals_noalloc(const double *model, const float *data, const uint8_t *mask, int maskmode,
                                  const uint8_t *region, int nz, int ny, int nx, double sigma2, double eps2,
                                  double *out2, void *stream);

/* ---- host set-up ------------------------------------------------------------------------------------ */
/* The sub-ring tables of a batch of thin-disk ring sets on one radius grid (bbarolo/galmod.py:761-851, the
 * reference's float64 operations in its order; host only, no context): rows (nb, 17, nr) the model rings'
 * values (radii, xpos, ypos, vsys, vrot, vdisp, vrad, vvert, dvdz, zcyl, dens, z0, inc, phi, z0thick, fthick,
 * vdispthick), nr >= 2; the grid's nsub sub-rings: i1 (the ring after each sub-ring's segment, 1 .. nr-1), dr
 * (offset from the segment's first ring), dseg (nr - 1 ring spacings), cst (1: before the first ring, the
 * first ring's values), radii; edgew (nsub, NULL: none) the weights of the outer edge on the densities, side
 * (2, nsub) the side weights; nvtmp the velocity samples of a sub-ring with a dispersion. Writes sr (nb, 16,
 * nsub), nv (nb, nsub) and, if ms is not NULL, the same tables into the first nsub columns of ms (nb, 16,
 * nsm). Replaces GalmodSetup.subrings per ring set (the vectorised subrings_batch of the engine). */
int bbgpu_subrings_rows(const double *rows, int nb, int nr, int nsub, const int64_t *i1, const double *dr,
                        const double *dseg, const uint8_t *cst, const double *radii, const double *edgew,
                        const double *side, int64_t nvtmp, double *sr, int64_t *nv, double *ms, int nsm);

/* ---- counters --------------------------------------------------------------------------------------- */
/* Kernel launches issued by the context so far, and the device time (ms) of the last bbgpu_eval_run split
 * into its kernels: times[0..n) in the order of bbgpu_kernel_name(i). */
int64_t bbgpu_launch_count(const bbgpu_ctx *ctx);
int bbgpu_last_run_times(const bbgpu_ctx *ctx, double *times, int n);
const char *bbgpu_kernel_name(int i);
/* Bytes copied host -> device and device -> host by the last bbgpu_eval_upload / bbgpu_eval_download. */
int bbgpu_transfer_bytes(const bbgpu_ctx *ctx, int64_t *h2d, int64_t *d2h);
/* How the last batch was shared (option 3): profiles computed (rows of ring maps), MC members that deposited all
 * their clouds, MC members computed as a difference from the first member's model, MC members that replayed the
 * first member's clouds with their own flux. */
int bbgpu_shared_members(const bbgpu_ctx *ctx, int *profiles, int *mc_full, int *mc_delta, int *mc_replay);

#ifdef __cplusplus
}
#endif

#endif /* BBGPU_H */
