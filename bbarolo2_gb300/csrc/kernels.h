// Launch wrappers of the bbgpu kernels (defined in mc.cu, conv.cu, analytic.cu, resid.cu), called by api.cu.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "internal.h"

// The device copy of a parsed MC stream (LayoutHost).
struct LayoutDev {
    int ncloud, nsub;
    long long nsubcloud, nslow;
    float4 *cf;          // per cloud: R, cos az, sin az, layer deviate (float32)
    double *cd;          // per cloud: the same in float64, 4 values per cloud
    int *sub;            // per cloud: sub-ring
    int *slow_base;      // per cloud: slow normals before it
    int32_t *hz;         // per sub-cloud: the first word of its normal (exact path)
    float *nf;           // per cloud: its normal deviates in float32, sorted (ascending channel order); each
                         // cloud's run starts at a multiple of 4 floats (16 bytes): pbase[ir] + (c - cloud_base) nvp
    uint16_t *ord;       // same layout: the index in the stream of the sorted normal at that position
    long long *pbase;    // per sub-ring: first padded position
    long long npad;      // padded length
    double *slow_val;    // slow normal values
    long long *sub_base; // per sub-ring: first sub-cloud
    int *nvs;            // per sub-ring: velocity samples per cloud
    int *cloud_base;     // per sub-ring: first cloud
};

// Per member of a batch (device array).
struct MemberDev {
    int blo0, blo1, bhi0, bhi1;   // box
    int bx, by;                   // box size
    int ntx, nty;                 // tiles of the deposit
    int tile_off;                 // first tile of the member in the tile arrays
    int fix_exp;                  // fixed-point exponent e (unit 2^-e)
    int maskmode, use_region;
    float sigma2f, eps2f;
    double sigma2, eps2;
    const float *deff;            // data used by the residual, (ny, nx, nz) float32, NaN where not used
};

struct ZigDev {
    unsigned kn[128];
    float wnf[128];
    double wn[128];
};

// ---- MC (mc.cu)
// For every (member, cloud): its pixel in the member's box (or -1) and the count of clouds per tile.
// Tile lists are split by pixel (NOWN per tile, tiles of at most 64 pixels): list index = (tile_off + tile) * NOWN
// + (lp % 8) * 8 + lp / 8 for pixel lp of the tile, so that the lists of the pixels lp = w (mod 8), owned by
// warp w of the deposit, are contiguous.
#define NOWN 64
// The (member, cloud) pairs of a batch by segments of threads: segment i (threads cstart[i] .. cstart[i + 1]) is
// cseg[4i .. 4i + 4) = (member whose tiles take the clouds, member whose constants place them, first cloud, sign
// of the deposits); ntot = cstart[nseg]. A member's own clouds are one segment (k, k, 0, +1) of ncloud threads.
void launch_mc_bin(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub, int nsub,
                   const MemberDev *mem, const long long *cstart, const int *cseg, int nseg, long long ntot, int tx,
                   int ty, int *pix, int *tile_count, int *err);
// Exclusive scan of n list counts into offsets (and cursors); scratch holds (n + 1023) / 1024 ints.
void launch_scan_tiles(cudaStream_t s, const int *count, int *offset, int *cursor, int n, int *scratch);
// bucket: 32-byte entries (Entry in mc.cu), one per in-box (member, cloud)
#define ENTRY_BYTES 32
void launch_mc_scatter(cudaStream_t s, const LayoutDev &L, const SubMC *sub, int nsub, const MemberDev *mem,
                       const long long *cstart, const int *cseg, int nseg, long long ntot, int tx, int ty,
                       const int *pix, int *cursor, void *bucket, int defer_fix);
// The fixed-point flux of the entries of a scatter with defer_fix (after the sub-ring constants are final):
// ntot bounds the entries (the (member, cloud) pairs), nlist lists
void launch_entry_fix(cudaStream_t s, const SubMC *sub, const int *offset, const int *count, int nlist,
                      long long ntot, void *bucket);
// Deposits the clouds of every tile into a shared-memory fixed-point tile and writes the model
// (by, bx, nz) float32 of each member at model + k * mstride (and, if model64, float64 sums); lean: the batch
// qualifies for the fast kernels (one line, a linear channel map, at most 128 samples per cloud).
// klist (nk members; nullptr: every member) selects the members of the launch. With base64 and tsrc (the
// pixel-owned kernel only, see mc_deposit_shares): delta = 0 leaves member 0's fixed-point sums in base64 (its
// box); delta = 1 adds them to the members' lists, which hold the difference from member 0's model (same box and
// exponent; ERR_SHARE otherwise), and leaves the tiles without entries unwritten. tsrc[tile_off + t] receives
// the member whose model holds tile t of the member (itself, or 0 for a tile left unwritten).
#define ERR_SHARE 8
bool mc_deposit_shares(int lean, bool model64, int tx, int ty);
// delta = 2 (replay): the member's clouds in the sub-rings not marked in chg (nchw 64-bit words a member) are
// member 0's clouds with the member's flux: the deposit adds member 0's channel counts of them (per pixel,
// sub-ring and half, in windows of RP_W channels: launch_replay_records) times the member's fixed-point flux; its
// own lists hold the clouds of the marked sub-rings. delta = 1 with records: member 0's clouds of the marked
// sub-rings are taken out of its sums by their counts times member 0's flux (the lists hold the member's own).
#define RP_W 64
struct Replay {
    const int2 *rec;
    const uint32_t *cnt;
    const int *nrec;
    const unsigned long long *chg;
    int nchw;
    const unsigned long long *tmask;    // per tile of member 0: the sub-rings with clouds in it (nchw words)
};
// the channel counts of member 0's clouds summed per (list = pixel, sub-ring, half) (sub0: its sub-ring constants;
// its nlist0 lists come first): rec (2 ints a record: first channel, sub-ring | half << 16 | extent << 17) and
// cnt (RP_W / 2 words of two 16-bit counts a record, in the lane order of the deposit's tiles of tp pixels) at the
// places of the list's entries, nrec (per list) their number
void launch_replay_records(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub0,
                           const ZigDev *zig, const void *bucket, const int *offset, const int *count, int nlist0,
                           int tp, int *rec, uint32_t *cnt, int *nrec, unsigned long long *tmask, int nchw,
                           int *err);
void launch_mc_deposit(cudaStream_t s, const GridDev &g, const LayoutDev &L, const SubMC *sub, int nsub,
                       const MemberDev *mem, const MemberDev *mem_host, int nb, int tx, int ty,
                       const int *offset, const int *count, const void *bucket, const ZigDev *zig,
                       const float *cd2if, const double *cd2i, float *model, long long mstride, double *model64,
                       int *err, int lean, const int *klist = nullptr, int nk = 0, int delta = 0,
                       long long *base64 = nullptr, int *tsrc = nullptr, Replay rp = Replay{nullptr, nullptr, nullptr, nullptr, 0, nullptr});

// ---- convolution + residual (conv.cu)
// The taps of a beam kernel (ky, kx) as the conv kernels read them: flipped, float32, rows padded to the
// compile-time window width kxw >= kx (returned; 0 if kx is too large). taps must hold ky * kxw floats.
int conv_taps(const double *k, int ky, int kx, float *taps);
// model (by, bx, nz) float32 per member -> the "same" convolution, threshold and scale, then the residual
// against deff (ny, nx, nz) float32 (NaN: voxel not used) over the box; per-CTA partial sums (ss, lg).
// If smoothed is not NULL the convolved model is written there (same layout).
// partial: (nb, npart) pairs (ss, lg), npart = tiles of the largest box x channel blocks (returned).
int conv_resid_npart(const MemberDev *mem_host, int nb, int nz);
// the output tiles of the convolution of a (by, bx, nz) box: nct tiles, ntx a row, of 2^shx x 2^shy pixels
void conv_tile_shape(int nz, int bx, int by, int &nct, int &ntx, int &shx, int &shy);
// With a tile table (tsrc): the model of member k at a pixel is that of member tsrc[tile_off + (y >> shy) ntx +
// (x >> shx)] (the MC deposit tiles of 2^shx x 2^shy pixels; a member computed as a difference from member 0
// leaves the tiles it shares with member 0 unwritten).
// With kout (the ring maps' convolution into K): a tile whose input lies wholly in member 0's is left unwritten,
// and kout[k kstride + t] receives the member whose output holds tile t (0 there, else k).
struct TileSrc {
    const int *tsrc;
    int shx, shy;
    int *kout;
    int kstride;
};
void launch_conv_resid(cudaStream_t s, const GridDev &g, const MemberDev *mem, const MemberDev *mem_host, int nb,
                       const float *model, long long mstride, int nz, const float *taps, int ky, int kx, int kxw,
                       float *smoothed, int do_conv, int do_resid, double *partial, TileSrc ts = TileSrc{nullptr, 0, 0, nullptr, 0});
// (the tile-table variant, conv_table.cu: maxt tiles and nzb channel blocks of ZB = 16 (z16) or 32 channels)
void launch_conv_table(cudaStream_t s, const GridDev &g, const MemberDev *mem, int nb, int maxt, int nzb, bool z16,
                       const float *model, long long mstride, int nz, const float *taps, int ky, int kx, int kxw,
                       float *smoothed, int do_conv, int do_resid, double *partial, int npart, TileSrc ts);
void launch_reduce_partials(cudaStream_t s, const double *partial, int npart, int nb, double *out2);
// (conv_wide.cu: kernels wider than the templates, kxw = 0 in launch_conv_resid; the taps (ky, kx) flipped)
void conv_wide_taps(const double *k, int ky, int kx, float *taps);
void launch_conv_wide(cudaStream_t s, const GridDev &g, const MemberDev *mem, int nb, int maxt, int nzb, bool z16,
                      const float *model, long long mstride, int nz, const float *taps, int ky, int kx,
                      float *smoothed, int do_conv, int do_resid, double *partial, int npart, TileSrc ts);

// ---- convolution + residual on the tensor cores (conv_tc.cu): variant 1 bf16x3, 2 tf32x3 (split products,
// FP32 accumulation in TMEM). Kernels of at most 16 rows and 33 columns, nz a multiple of 4 (TMA rows of 16 bytes).
#define ERR_TC 16                 // a bounded wait of the tensor-core convolution expired
bool conv_tc_supported(int variant, int ky, int kx, int nz);
// the B operand image (the banded Toeplitz rows of the flipped kernel, split hi / lo) of a kernel (ky, kx)
void conv_tc_image(int variant, const double *kern, int ky, int kx, std::vector<uint8_t> &img);
// TMA descriptors: maps[k] the model (by, bx, nz) float32 of member k at model + k mstride, maps[nb + k] its data
// (the cube's deff, ny x nx x nz)
bool conv_tc_maps(const MemberDev *mem_host, int nb, const float *model, long long mstride, int nz, int nx, int ny,
                  std::vector<CUtensorMap> &maps);
// partial pairs per member (16 x 16 pixel tiles x blocks of 128 channels x 8 epilogue warps); zeroed by the caller
int conv_tc_npart(const MemberDev *mem_host, int nb, int nz);
void launch_conv_tc(cudaStream_t s, int variant, const GridDev &g, const MemberDev *mem, const MemberDev *mem_host,
                    int nb, const CUtensorMap *maps, const void *bimg, long long mstride, int nz, int ky, int kx,
                    float *smoothed, int do_conv, int do_resid, double *partial, int npart, TileSrc ts, int *err,
                    int *queue);

// ---- layouts and stand-alone residuals (resid.cu)
void launch_prep_deff(cudaStream_t s, const float *data, const uint8_t *mask, const uint8_t *region, int maskmode,
                      int nz, int ny, int nx, float *deff);
// returns the number of partial pairs written
int launch_sumsq64(cudaStream_t s, const double *model, const float *data, const uint8_t *mask, int maskmode,
                   const uint8_t *region, int nz, int ny, int nx, double sigma2, double eps2, double *partial,
                   int maxblocks);
void launch_zyx64_to_yxz32(cudaStream_t s, const double *in, float *out, int nz, int ny, int nx);
void launch_yxz32_to_zyx64(cudaStream_t s, const float *in, double *out, int nz, int ny, int nx);

// ---- CLASSIC (classic.cu)
void launch_conv_sparse(cudaStream_t s, const double *model, double *out, int ny, int nx, int nz, const double *kern,
                        int ky, int kx, double scale);
void launch_norm_sums(cudaStream_t s, const double *model, const float *data, const uint8_t *mask,
                      const uint8_t *inside, int bsy, int bsx, int nz, double *part);
void launch_norm_prefix(cudaStream_t s, const double *pre, double *P, int bsy, int bsx, int nz);
void launch_norm_pix(cudaStream_t s, double *model, const float *data, const uint8_t *mask, const uint8_t *inside,
                     const double *wmap, int bsy, int bsx, int nz, int ftype, const double *chan_noise,
                     double data_noise, int normtype, double factor_azim, const double *P, const long long *ilo,
                     const long long *ihi, int ky, const double *thr, double *part);

// ---- ANALYTIC (analytic.cu)
// dynamic shared memory of launch_an_model (the host keeps it within AN_SMEM_MAX)
#define AN_SMEM_MAX (200 * 1024)
size_t an_smem_bytes(int nz, int nlines);
// The ANALYTIC models of a batch by segments of warps (a warp a sample): segment i (warps astart[i] ..
// astart[i + 1], ntot = astart[nseg]) is aseg[4i .. 4i + 4) = (member whose model takes the deposits, member whose
// constants make them, sub-ring (-1: every sample of the table), sign of the deposits).
void launch_an_model(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase, const int *ssub,
                     const double *cs, const long long *astart, const int *aseg, int nseg, long long ntot,
                     const double *zq, const double *wq, const double *vedges, const double *cd2i, const double *ptab,
                     const MemberDev *mem, long long *out64, long long mstride, int skip_fast);
// the float32 path of the ANALYTIC model (sub-rings with anfast; launch_an_model with skip_fast does the others):
// csf, zqf, wqf float32 copies of the sample and vertical tables, csff (float4 per sample) its cos and sin in
// float-float, vef (nz + 1) float-float channel edges of line 0
// relative to g.vref, ptabf the normal CDF table in float32
size_t an_fast_smem_bytes(int nz);
void launch_an_model_fast(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase,
                          const int *ssub, const double *cs, const float *csf, const float *csff,
                          const long long *astart, const int *aseg, int nseg, long long ntot,
                          const double *zq, const float *zqf, const float *wqf, const float *vef, const float *cd2if,
                          const float *ptabf, const MemberDev *mem, long long *out64, long long mstride, int thin,
                          int thick);
void launch_an_maps(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase, const int *ssub,
                    const double *cs, long long nsamp, const double *zq, const double *wq, const long long *widx,
                    const double *wval, const MemberDev &M, long long *maps64);
// mbase (nullable): per member, the member whose fixed-point sums are added (-1: none)
void launch_fix_to_model(cudaStream_t s, const long long *in, const MemberDev *mem, int nb, long long mstride, int nz,
                         float *model, double *model64, const int *mbase = nullptr);

// ---- flux normalisation (profile.cu)
#define ERR_PROFILE_LAYOUT 4      // a deconvolved density changed the MC cloud layout of a member
// the likelihood box of the ring maps: (by, bx) pixels x nrp maps, ring fastest
struct ProfBox {
    int blo0, blo1, bhi0, bhi1, bx, by, nrp, pad;
    long long npix;
};
// the constants of solve_profile shared by a batch
struct ProfConst {
    int n, m;                     // unknowns (rings + exterior annulus), pixels used
    double bb;                    // b.b
    double smooth, corr, floor_, norm, d;
};
// The ring maps of a batch, by segments of threads: segment i (threads mstart[i] .. mstart[i+1]) is mseg[4i..4i+4)
// = (row u of maps64, member whose sub-ring constants it takes, sub-ring (-1: every sample of the table), sign)
void launch_an_maps_fast(cudaStream_t s, const GridDev &g, const AnSub *subs, int nsub, const int *sbase,
                         const int *ssub, const double *cs, const float *csf, const long long *mstart,
                         const int *mseg, int nseg, long long ntot, const double *zq, const float *zqf,
                         const float *wqf, const int *widx, const float *wvalf, const ProfBox &box,
                         const int *fix_exp, long long *maps64);
// rows u < nu of maps64 (member uidx[u]; plus row ubase[u] when >= 0) -> float32; with ptab (nu x the 8 x 8
// pixel blocks of the box, row-major): the row whose maps hold each block (the row itself, or its base row where
// their maps are equal)
void launch_maps_to_f32(cudaStream_t s, const long long *in, const int *fix_exp, const int *uidx, const int *ubase,
                        int nu, long long per_member, float scale, float *out, int *ptab, const ProfBox &box);
void launch_prof_gather(cudaStream_t s, const double *xu, const int *stu, const int *prof_of, int nb, int n, double *x,
                        int *st);
int prof_gram_tiles(int npix_used);
// The rows of K that hold each convolution tile (ktab: nct tiles of 2^shx x 2^shy pixels, ntx a row, per row;
// row 0's where a row's convolution left it unwritten), and gflag (rows x Gram tiles): 1 where a Gram tile took
// row 0's sums. ktab == nullptr: every row's own K.
// blk (nullable; the rows' 8 x 8 pixel blocks, nby x nbx a row: the row whose maps hold each) refines the test:
// a pixel whose beam neighbourhood lies in blocks of row 0's maps has row 0's K.
struct KRows {
    const int *ktab;
    int nct, ntx, shx, shy;
    int *gflag;
    const int *blk;
    int nbx, nby;
};
void launch_prof_gram(cudaStream_t s, const float *K, const ProfBox &box, const int *pix, const double *wpix,
                      const double *wy, int npix_used, const int *ent_i, const int *ent_j, int nent, int nb,
                      double *part, double *gh, KRows kr = KRows{});
// one system A (m, n) row-major (box.nrp = n, box.npix = m), b (m): packed G = A^T A, h = A^T b
void launch_prof_gram64(cudaStream_t s, const double *A, const ProfBox &box, const double *b, int m, const int *ent_i,
                        const int *ent_j, int nent, double *part, double *gh);
size_t prof_solve_smem(int n);
void launch_prof_solve(cudaStream_t s, const double *gh, const ProfConst &pc, const int *lc, const double *lv,
                       const int *ord, const unsigned char *near, const int *p0, int nb, double *x, int *pout,
                       int *status);
void launch_mc_dens(cudaStream_t s, const GridDev &g, SubMC *sub, int nsub, MemberDev *mem, int nb, const double *x,
                    int nx, const int *widx, const double *wval, const double *rap, int *err);
// the densities of the ANALYTIC model's sub-rings into its constants (fluxsc, line amplitudes, exponent);
// per = sum |relint| x max |cd2i| (the deposit bound of a sample of unit flux)
void launch_an_dens(cudaStream_t s, const GridDev &g, AnSub *sub, int nsub, MemberDev *mem, int nb, const double *x,
                    int nx, const int *widx, const double *wval, const double *rap, double per, int *err);

// The entries of a batch's per-(member, sub-ring) constants that repeat member 0's (reused = 1, left unwritten by
// the host): SubMC with the member's fixed-point deposits, or a plain copy of any 8-byte-word structure.
void launch_fill_submc(cudaStream_t s, SubMC *sub, int nsub, int nb, const signed char *reused, const MemberDev *mem,
                       int nlines);
void launch_fill_copy(cudaStream_t s, void *base, size_t elt_bytes, int nsub, int nb, const signed char *reused);

// GALWIND WTYPE 1 (galwind.cu): one thread per cloud; acc (by, bx, nz) of 64-bit fixed-point sums (units 1/scale)
void launch_wind_mc(cudaStream_t st, const WindShell *shells, const int *shell, const double *geo,
                    const long long *nbase, const long long *sbase, const int *hz, const double *slow,
                    const ZigDev *zig, long long ncloud, const GridDev &g, const double *cd2i, int blo0, int blo1,
                    int bhi0, int bhi1, double scale, unsigned long long *acc);
