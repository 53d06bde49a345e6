// The C ABI of bbgpu (include/bbgpu.h): contexts, device memory, the cache of MC stream layouts, and the
// batched likelihood pipeline.
//
// One context = one device, one CUDA stream, the constants of one cube (grid, beam kernel, data). Device
// buffers grow with the largest batch seen and are reused. Errors are returned as status codes with a
// message (bbgpu_last_error); nothing throws across the ABI.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bbgpu.h"
#include "kernels.h"

#define BBGPU_VERSION 1
#define NLAYOUT 64                          // cached MC layouts (the single-ring models of a CLASSIC stage have one each)
#define LAYOUT_BUDGET (1ll << 31)           // device bytes the cached layouts may hold (least recently used evicted)
#define NTIMER 13

// the timed stages of a batch: the flux normalisation (ring maps, their beam convolution, the normal equations,
// the solves and the sub-ring densities), then the MC model (or the ANALYTIC one), its convolution and the
// residual reduction (mc_deposit_delta: the members computed as a difference from member 0's model;
// mc_replay: the members replaying member 0's clouds, with the records of member 0's channel counts)
static const char *KNAMES[NTIMER] = {"prof_maps", "prof_conv",  "prof_gram",  "prof_solve",
                                     "mc_bin",    "scan_tiles", "mc_scatter", "mc_deposit",
                                     "mc_deposit_delta", "mc_replay", "an_model", "conv_resid",
                                     "reduce_partials"};

struct PoolBuf {
    void *p = nullptr;
    size_t cap = 0;
};

struct LayoutEntry {
    LayoutHost host;
    LayoutDev dev;
    double zspan = 0.0;           // largest spread (max - min) of one cloud's normal deviates
    long long bytes = 0;          // device bytes of the layout
    bool valid = false;
    long long last_use = 0;
};

struct bbgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // the MC clouds' lists are built on a second stream of lower priority while the flux normalisation runs
    // (joined before the deposits)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string err;
    bool grid_set = false, kernel_set = false, cube_set = false;
    GridDev g{};
    // constants
    double *d_cd2i = nullptr;
    float *d_cd2if = nullptr;
    std::vector<double> h_cd2i;
    double *d_vedges = nullptr;   // channel edges per line (nlines, nz + 1): ANALYTIC models
    double *d_ptab = nullptr;     // normal CDF table of the ANALYTIC line profiles
    float *d_ptabf = nullptr;     // (float32 copy: the model's fast path)
    float2 *d_vef = nullptr;      // channel edges of line 0 - vref, float-float (nz + 1): the model's fast path
    ZigDev *d_zig = nullptr;
    float *d_taps = nullptr;
    int ky = 0, kx = 0, kxw = 0;
    // cube
    float *d_data = nullptr;
    uint8_t *d_mask = nullptr, *d_region = nullptr;
    float *d_deff[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    // layouts
    LayoutEntry layouts[NLAYOUT];
    long long use_clock = 0;
    LayoutEntry *cur = nullptr;
    std::vector<PoolBuf> pool[8];       // the scratch buffers of the stand-alone calls (DevBufs), per call site
    // batch
    int nb = 0, nsub = 0, galmodtype = 0, tx = 8, ty = 8, ntile_total = 0, npart = 0;
    bool uploaded = false, ran = false;
    std::vector<MemberDev> mem_host;
    SubMC *h_sub = nullptr;
    size_t h_sub_cap = 0;
    MemberDev *h_mem = nullptr;
    size_t h_mem_cap = 0;
    double *h_out2 = nullptr;
    size_t h_out2_cap = 0;
    int *h_err = nullptr;
    SubMC *d_sub = nullptr;
    size_t d_sub_cap = 0;
    MemberDev *d_mem = nullptr;
    size_t d_mem_cap = 0;
    int *d_pix = nullptr;
    size_t d_pix_cap = 0;
    int4 *d_bucket = nullptr;     // (2 int4 per entry)
    size_t d_bucket_cap = 0;
    int *d_tcount = nullptr, *d_toff = nullptr, *d_tcur = nullptr;
    size_t d_tcount_cap = 0, d_toff_cap = 0, d_tcur_cap = 0;
    int *d_scan = nullptr;
    size_t d_scan_cap = 0;
    float *d_model = nullptr;
    size_t d_model_cap = 0;
    float *d_smooth = nullptr;
    size_t d_smooth_cap = 0;
    double *d_model64 = nullptr;
    size_t d_model64_cap = 0;
    double *d_partial = nullptr;
    size_t d_partial_cap = 0;
    double *d_out2 = nullptr;
    size_t d_out2_cap = 0;
    int *d_err = nullptr;
    long long mstride = 0;
    // flux normalisation (bbgpu_set_profile, bbgpu_eval_upload_profile)
    bool prof_set = false, prof_uploaded = false;
    ProfBox pbox{};
    ProfConst pc{};
    double mapscale = 1.0;
    int npix_used = 0, nent = 0, nsm = 0;
    long long pnsamp = 0;
    int *d_ppix = nullptr, *d_lc = nullptr, *d_ord = nullptr, *d_p0 = nullptr, *d_ent = nullptr;
    double *d_pw = nullptr, *d_pwy = nullptr, *d_lv = nullptr;
    unsigned char *d_near = nullptr;
    AnSub *d_psub = nullptr;
    size_t d_psub_cap = 0;
    int *d_psbase = nullptr, *d_pssub = nullptr, *d_pwidx = nullptr, *d_pfix = nullptr, *d_pp = nullptr,
        *d_pstat = nullptr;
    size_t d_psbase_cap = 0, d_pssub_cap = 0, d_pwidx_cap = 0, d_pfix_cap = 0, d_pp_cap = 0, d_pstat_cap = 0;
    float *d_pcsf = nullptr;
    size_t d_pcsf_cap = 0;
    double *d_pcs = nullptr, *d_pzq = nullptr, *d_pwval = nullptr, *d_rap = nullptr, *d_gpart = nullptr,
           *d_gh = nullptr, *d_px = nullptr, *d_ppart = nullptr;
    size_t d_pcs_cap = 0, d_pzq_cap = 0, d_pwval_cap = 0, d_rap_cap = 0, d_gpart_cap = 0, d_gh_cap = 0,
           d_px_cap = 0, d_ppart_cap = 0;
    float *d_pzqf = nullptr, *d_pwqf = nullptr, *d_pwvalf = nullptr, *d_maps32 = nullptr, *d_K = nullptr;
    size_t d_pzqf_cap = 0, d_pwqf_cap = 0, d_pwvalf_cap = 0, d_maps32_cap = 0, d_K_cap = 0;
    long long *d_maps64 = nullptr;
    size_t d_maps64_cap = 0;
    MemberDev *d_pmem = nullptr;
    size_t d_pmem_cap = 0;
    // rows of the maps (the members with a profile of their own, nu of them) and the segments of the maps
    // kernel's threads (bbgpu_eval_upload_profile); the solutions of the rows go to the members by prof_of
    int nu = 0, nseg = 0, nu_delta = 0;
    long long mtot = 0;
    // rows with a base row: the 8 x 8 pixel blocks of their maps (blk), the tiles of their convolution (ktab)
    // and the Gram tiles (gflag) that are row 0's
    int *d_blk = nullptr, *d_ktab = nullptr, *d_gflag = nullptr;
    size_t d_blk_cap = 0, d_ktab_cap = 0, d_gflag_cap = 0;
    long long *d_mstart = nullptr;
    int *d_mseg = nullptr, *d_uidx = nullptr, *d_ubase = nullptr, *d_prof_of = nullptr, *d_pstatu = nullptr;
    double *d_pxu = nullptr;
    size_t d_mstart_cap = 0, d_mseg_cap = 0, d_uidx_cap = 0, d_ubase_cap = 0, d_prof_of_cap = 0, d_pstatu_cap = 0,
           d_pxu_cap = 0;
    std::vector<int> psbase_host;      // first sample of each sub-ring in the sample table on the device
    std::vector<int> prof_of_host;     // the row of each member's profile (0: member 0's)
    // MC: the (member, cloud) segments of the bin and scatter kernels, and the members of the two deposit
    // launches (mc_n1 members with their own lists, then mc_n2 holding the difference from member 0's model,
    // whose fixed-point sums are kept in d_base64); rebuilt before a run when mc_dirty
    bool mc_dirty = true;
    int mc_nseg = 0, mc_n1 = 0, mc_n2 = 0, mc_n3 = 0;   // (mc_n3: the members replaying member 0's clouds)
    std::vector<signed char> mc_same_nd;   // per (member, sub-ring): member 0's column but for the density
    // ANALYTIC: the (member, sample) segments of the model kernels and, per member, the member whose fixed-point
    // sums it adds (-1: none); rebuilt before a run when an_dirty
    bool an_dirty = true;
    int an_nseg = 0, an_n2 = 0;
    long long an_ntot = 0;
    std::vector<long long> h_astart;
    std::vector<int> h_aseg, h_mbase, asbase_host;
    long long *d_astart = nullptr;
    int *d_aseg = nullptr, *d_mbase = nullptr;
    size_t d_astart_cap = 0, d_aseg_cap = 0, d_mbase_cap = 0;
    std::vector<unsigned long long> h_chg; // per member: the sub-rings a replaying member deposits itself
    int nchw = 0;
    int *d_rp_rec = nullptr, *d_rp_n = nullptr;   // (2 ints a record; records per list of member 0)
    uint32_t *d_rp_cnt = nullptr;
    unsigned long long *d_chg = nullptr, *d_tmask = nullptr;
    size_t d_tmask_cap = 0;
    bool mc_records = false;              // member 0's records are built (replaying or difference members use them)
    size_t d_rp_rec_cap = 0, d_rp_cnt_cap = 0, d_chg_cap = 0, d_rp_n_cap = 0;
    long long mc_ntot = 0;
    std::vector<long long> h_cstart;
    std::vector<int> h_cseg, h_klist;
    long long *d_cstart = nullptr, *d_base64 = nullptr;
    int *d_cseg = nullptr, *d_klist = nullptr, *d_tsrc = nullptr;
    size_t d_cstart_cap = 0, d_base64_cap = 0, d_cseg_cap = 0, d_klist_cap = 0, d_tsrc_cap = 0;
    std::vector<signed char> mc_isdelta;   // per member: computed as a difference (tiles shared with member 0)
    ZgridCache zcache;                 // vertical grids of the ring maps (host), mirrored in d_pzq/d_pzqf/d_pwqf
    std::string samp_key;              // the sub-ring radii of the sample table on the device
    AnSub *h_psub = nullptr;           // pinned staging of the sub-ring constants
    size_t h_psub_cap = 0;
    std::vector<MemberDev> pmem_host;
    // per (member, sub-ring): 1 where the member's constants are member 0's (filled on the device)
    signed char *h_reuse = nullptr, *d_reuse = nullptr, *h_preuse = nullptr, *d_preuse = nullptr;
    size_t h_reuse_cap = 0, d_reuse_cap = 0, h_preuse_cap = 0, d_preuse_cap = 0;
    // ANALYTIC batches: sub-ring constants per member, the sample table of the model's sub-rings, their vertical
    // grids (host cache mirrored on the device) and the fixed-point models
    AnSub *h_asub = nullptr, *d_asub = nullptr;
    int an_thin = 0, an_thick = 0, an_exact = 1;   // the ANALYTIC kernels the uploaded batch needs
    size_t h_asub_cap = 0, d_asub_cap = 0;
    int *d_asbase = nullptr, *d_assub = nullptr;
    size_t d_asbase_cap = 0, d_assub_cap = 0;
    double *d_acs = nullptr, *d_azq = nullptr, *d_awq = nullptr;
    size_t d_acs_cap = 0, d_azq_cap = 0, d_awq_cap = 0;
    float *d_acsf = nullptr, *d_azqf = nullptr, *d_awqf = nullptr;
    size_t d_acsf_cap = 0, d_azqf_cap = 0, d_awqf_cap = 0;
    float4 *d_acsff = nullptr;         // cos, sin of the model's samples in float-float
    size_t d_acsff_cap = 0;
    long long *d_model_fx = nullptr;
    size_t d_model_fx_cap = 0;
    long long ansamp = 0;
    std::string asamp_key;
    ZgridCache azcache;
    // options
    bool keep_smoothed = false, timing = false, want64 = false;
    bool share = true;            // members that differ from member 0 in a few sub-rings: computed as member 0's
                                  // result plus the difference (ring maps, MC model)
    int lean = 0;                 // the batch qualifies for the fast deposit kernels (one line, a linear channel
                                  // map, at most 128 samples per cloud)
    // the beam convolution of the batch models: 0 float32 FMA (k_conv_resid), 1 bf16x3 or 2 tf32x3 on the tensor
    // cores (k_conv_tc; the float32 kernel where a batch does not qualify)
    int conv_variant = -1;                // -1: the autotuner's choice (below)
    // the autotuner: per kernel shape and channels (ky, kx, nz), the variant it chose, timed on the first batch
    // (float32 and tf32x3, the variants within 1e-5 per voxel of the float64 convolution), and its timings (ms)
    std::vector<std::array<int, 4>> tuned;      // (ky, kx, nz, variant)
    float tune_ms[3] = {-1.f, -1.f, -1.f};
    std::vector<double> h_kernel;         // the beam kernel (ky, kx) float64
    void *d_bimg = nullptr;               // its B operand image for conv_variant
    size_t d_bimg_cap = 0;
    int bimg_variant = 0;
    CUtensorMap *d_tmaps = nullptr;       // per member: TMA descriptor of its model
    int *d_tcq = nullptr;                 // the next work item of a tensor-core convolution launch
    size_t d_tmaps_cap = 0;
    std::vector<CUtensorMap> h_tmaps;
    std::vector<long long> tmaps_key;     // (model, mstride, nz, boxes) of the descriptors on the device
    int npart_used = 0;                   // partial pairs per member of the last convolution
    // CUDA graph of a batch run (option 5): captured on the second run of an unchanged batch, replayed after.
    // gen counts the changes of what a run reads (uploads, options, reallocations, stand-alone calls).
    bool use_graphs = true;
    long long gen = 1, gen_ran = 0, graph_gen = 0, graph_fail_gen = 0, graph_launches = 0, graph_replays = 0;
    cudaGraphExec_t gexec = nullptr;
    int conv_used = 0;                    // variant of the last batch convolution
    long long launches = 0;
    long long h2d = 0, d2h = 0;
    cudaEvent_t ev[NTIMER + 1] = {};
    double times[NTIMER] = {};
};

// ------------------------------------------------------------------------------------------- helpers
static int fail(bbgpu_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                           \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) return fail(ctx, BBGPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CKL()                                                                                               \
    do {                                                                                                    \
        cudaError_t e_ = cudaGetLastError();                                                                \
        if (e_ != cudaSuccess) return fail(ctx, BBGPU_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
        ctx->launches++;                                                                                    \
    } while (0)

template <class T>
static int dgrow(bbgpu_ctx *ctx, T **p, size_t *cap, size_t n) {
    if (n <= *cap && *p) return 0;
    ctx->gen++;                       // (a captured batch run holds the old address)
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t m = n + n / 4 + 16;
    if (cudaMalloc((void **)p, m * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, BBGPU_ERR_NOMEM, "device allocation of %zu bytes failed", m * sizeof(T));
    }
    *cap = m;
    return 0;
}

template <class T>
static int hgrow(bbgpu_ctx *ctx, T **p, size_t *cap, size_t n) {
    if (n <= *cap && *p) return 0;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    size_t m = n + n / 4 + 16;
    if (cudaMallocHost((void **)p, m * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, BBGPU_ERR_NOMEM, "pinned allocation of %zu bytes failed", m * sizeof(T));
    }
    *cap = m;
    return 0;
}

static void layout_dev_free(LayoutDev &d) {
    cudaFree(d.cf); cudaFree(d.cd); cudaFree(d.sub); cudaFree(d.slow_base); cudaFree(d.hz); cudaFree(d.slow_val);
    cudaFree(d.nf); cudaFree(d.nvs); cudaFree(d.ord); cudaFree(d.pbase);
    cudaFree(d.sub_base); cudaFree(d.cloud_base);
    memset(&d, 0, sizeof d);
}

static int upload_layout(bbgpu_ctx *ctx, LayoutEntry &E) {
    LayoutHost &H = E.host;
    LayoutDev &D = E.dev;
    memset(&D, 0, sizeof D);
    D.ncloud = H.ncloud;
    D.nsub = H.nsub;
    D.nsubcloud = H.nsubcloud;
    D.nslow = H.nslow;
    size_t nc = (size_t)(H.ncloud ? H.ncloud : 1);
    std::vector<float4> cf(nc);
    std::vector<double> cd(4 * nc);
    for (int c = 0; c < H.ncloud; c++) {
        cf[c] = make_float4((float)H.R[c], (float)H.caz[c], (float)H.saz[c], (float)H.fdev[c]);
        cd[4 * c] = H.R[c];
        cd[4 * c + 1] = H.caz[c];
        cd[4 * c + 2] = H.saz[c];
        cd[4 * c + 3] = H.fdev[c];
    }
    CK(cudaMalloc(&D.cf, nc * sizeof(float4)));
    CK(cudaMalloc(&D.cd, 4 * nc * sizeof(double)));
    CK(cudaMalloc(&D.sub, nc * sizeof(int)));
    CK(cudaMalloc(&D.slow_base, nc * sizeof(int)));
    CK(cudaMalloc(&D.hz, (size_t)(H.nsubcloud ? H.nsubcloud : 1) * sizeof(int32_t)));
    CK(cudaMalloc(&D.slow_val, (size_t)(H.nslow ? H.nslow : 1) * sizeof(double)));
    CK(cudaMalloc(&D.sub_base, (size_t)(H.nsub ? H.nsub : 1) * sizeof(long long)));
    CK(cudaMalloc(&D.cloud_base, (size_t)(H.nsub ? H.nsub : 1) * sizeof(int)));
    CK(cudaMalloc(&D.nvs, (size_t)(H.nsub ? H.nsub : 1) * sizeof(int)));
    CK(cudaMemcpy(D.cf, cf.data(), nc * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.cd, cd.data(), 4 * nc * sizeof(double), cudaMemcpyHostToDevice));
    if (H.ncloud) {
        CK(cudaMemcpy(D.sub, H.sub, (size_t)H.ncloud * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(D.slow_base, H.slow_base, (size_t)H.ncloud * sizeof(int), cudaMemcpyHostToDevice));
    }
    if (H.nsubcloud) CK(cudaMemcpy(D.hz, H.hz, (size_t)H.nsubcloud * sizeof(int32_t), cudaMemcpyHostToDevice));
    {
        // the normal deviates of each cloud, sorted by value (descending when the channel decreases with the
        // velocity): the channels of a cloud's samples are then non-decreasing along the sorted order
        int64_t kn[128];
        double wn[128], fn[128];
        bbh_zig_tables(kn, wn, fn);
        const GridDev &g = ctx->g;
        const bool desc = g.axtyp == 4 ? g.cdelt3 < 0 : g.cdelt3 > 0;
        std::vector<long long> pbase(H.nsub ? H.nsub : 1);
        long long np = 0;
        for (int ir = 0; ir < H.nsub; ir++) {
            pbase[ir] = np;
            np += (long long)H.nc[ir] * ((H.nv[ir] + 3) & ~3);
        }
        size_t nsc = (size_t)(np ? np : 1);
        std::vector<float> nf(nsc, __builtin_nanf(""));       // (the padding: NaN, which no channel test passes)
        std::vector<uint16_t> ord(nsc, 0);
        std::vector<double> val;
        std::vector<int> idx;
        long long so = 0, q = 0;
        for (int c = 0; c < H.ncloud; c++) {
            const int ir = H.sub[c];
            const int nv = H.nv[ir];
            val.resize(nv);
            idx.resize(nv);
            for (int i = 0; i < nv; i++, q++) {
                int32_t h = H.hz[q];
                int iz = h & 127;
                long long ah = h < 0 ? -(long long)h : (long long)h;
                val[i] = ah < kn[iz] ? (double)h * wn[iz] : H.slow_val[so++];
                idx[i] = i;
            }
            std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return desc ? val[a] > val[b] : val[a] < val[b]; });
            if (nv > 0) E.zspan = std::max(E.zspan, fabs(val[idx[nv - 1]] - val[idx[0]]));
            long long b0 = pbase[ir] + (long long)(c - H.cloud_base[ir]) * ((nv + 3) & ~3);
            for (int i = 0; i < nv; i++) {
                nf[b0 + i] = (float)val[idx[i]];
                ord[b0 + i] = (uint16_t)idx[i];
            }
        }
        D.npad = np;
        CK(cudaMalloc(&D.pbase, pbase.size() * sizeof(long long)));
        CK(cudaMemcpy(D.pbase, pbase.data(), pbase.size() * sizeof(long long), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&D.nf, nsc * sizeof(float)));
        CK(cudaMalloc(&D.ord, nsc * sizeof(uint16_t)));
        CK(cudaMemcpy(D.nf, nf.data(), nsc * sizeof(float), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(D.ord, ord.data(), nsc * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    if (H.nslow) CK(cudaMemcpy(D.slow_val, H.slow_val, (size_t)H.nslow * sizeof(double), cudaMemcpyHostToDevice));
    if (H.nsub) {
        CK(cudaMemcpy(D.sub_base, H.sub_base, (size_t)H.nsub * sizeof(long long), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(D.cloud_base, H.cloud_base, (size_t)H.nsub * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(D.nvs, H.nv, (size_t)H.nsub * sizeof(int), cudaMemcpyHostToDevice));
    }
    return 0;
}

// The layout of (seed, ltype, nc, nv, R0): cached (NLAYOUT most recent), parsed on the host on a miss.
static int get_layout(bbgpu_ctx *ctx, uint64_t seed, int nsub, const int *nc, const int *nv, const double *R0,
                      LayoutEntry **out) {
    uint64_t key = bbh_layout_key(seed, ctx->g.ltype, nsub, nc, nv, R0, ctx->g.radsep);
    LayoutEntry *victim = &ctx->layouts[0];
    for (auto &E : ctx->layouts) {
        if (E.valid && E.host.key == key && E.host.nsub == nsub && memcmp(E.host.nc, nc, sizeof(int) * nsub) == 0 &&
            memcmp(E.host.nv, nv, sizeof(int) * nsub) == 0) {
            E.last_use = ++ctx->use_clock;
            *out = &E;
            return 0;
        }
        if (!E.valid || E.last_use < victim->last_use) victim = &E;
    }
    // room: the least recently used slot, and more while the cached layouts hold more than the budget
    auto evict = [&](LayoutEntry &E) -> int {
        CK(cudaStreamSynchronize(ctx->stream));
        layout_dev_free(E.dev);
        bbh_layout_free(&E.host);
        E.valid = false;
        E.bytes = 0;
        if (ctx->cur == &E) {          // (the uploaded MC batch used it: it must be uploaded again)
            ctx->cur = nullptr;
            ctx->uploaded = false;
            ctx->gen++;
        }
        return 0;
    };
    if (victim->valid && evict(*victim)) return BBGPU_ERR_CUDA;
    for (;;) {
        long long total = 0;
        LayoutEntry *lru = nullptr;
        for (auto &E : ctx->layouts)
            if (E.valid) {
                total += E.bytes;
                if (!lru || E.last_use < lru->last_use) lru = &E;
            }
        if (total <= LAYOUT_BUDGET || !lru) break;
        if (evict(*lru)) return BBGPU_ERR_CUDA;
    }
    if (bbh_layout_build(&victim->host, seed, ctx->g.ltype, nsub, nc, nv, R0, ctx->g.radsep) != 0)
        return fail(ctx, BBGPU_ERR_NOMEM, "MC layout: too many clouds or host allocation failed");
    int rc = upload_layout(ctx, *victim);
    if (rc) return rc;
    {
        const LayoutHost &H = victim->host;
        victim->bytes = (long long)H.ncloud * 56 + (long long)H.nsubcloud * 12 + (long long)H.nslow * 8 +
                        (long long)H.nsub * 16;
    }
    victim->valid = true;
    victim->last_use = ++ctx->use_clock;
    *out = victim;
    return 0;
}

static int ensure_deff(bbgpu_ctx *ctx, int maskmode, int use_region) {
    if (maskmode < 0 || maskmode > 2) return fail(ctx, BBGPU_ERR_ARG, "maskmode must be 0, 1 or 2");
    if (use_region && !ctx->d_region) return fail(ctx, BBGPU_ERR_ARG, "use_region without a region");
    float *&d = ctx->d_deff[maskmode][use_region ? 1 : 0];
    if (d) return 0;
    size_t n = (size_t)ctx->g.nx * ctx->g.ny * ctx->g.nz;
    CK(cudaMalloc(&d, n * sizeof(float)));
    launch_prep_deff(ctx->stream, ctx->d_data, ctx->d_mask, use_region ? ctx->d_region : nullptr, maskmode, ctx->g.nz,
                     ctx->g.ny, ctx->g.nx, d);
    CKL();
    return 0;
}

// ------------------------------------------------------------------------------------------- context
extern "C" int bbgpu_version(void) { return BBGPU_VERSION; }

extern "C" int bbgpu_ctx_create(bbgpu_ctx **out, int device) {
    bbgpu_ctx *ctx = nullptr;
    if (!out) return BBGPU_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return BBGPU_ERR_CUDA;
    }
    if (device < 0 || device >= n) return BBGPU_ERR_ARG;
    ctx = new (std::nothrow) bbgpu_ctx();
    if (!ctx) return BBGPU_ERR_NOMEM;
    ctx->device = device;
    int prio_lo = 0, prio_hi = 0;
    if (cudaSetDevice(device) != cudaSuccess || cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return BBGPU_ERR_CUDA;
    }
    if (cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        bbgpu_ctx_destroy(ctx);
        return BBGPU_ERR_CUDA;
    }
    // ziggurat tables (fast-path bound kn fits 32 bits)
    ZigDev z;
    int64_t kn[128];
    double wn[128], fn[128];
    bbh_zig_tables(kn, wn, fn);
    for (int i = 0; i < 128; i++) {
        z.kn[i] = (unsigned)kn[i];
        z.wnf[i] = (float)wn[i];
        z.wn[i] = wn[i];
    }
    if (cudaMalloc(&ctx->d_zig, sizeof z) != cudaSuccess || cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess ||
        cudaMemcpy(ctx->d_zig, &z, sizeof z, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(ctx->d_err, 0, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_err, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        bbgpu_ctx_destroy(ctx);
        return BBGPU_ERR_CUDA;
    }
    for (int i = 0; i <= NTIMER; i++) cudaEventCreate(&ctx->ev[i]);
    *out = ctx;
    return BBGPU_OK;
}

extern "C" int bbgpu_ctx_destroy(bbgpu_ctx *ctx) {
    if (!ctx) return BBGPU_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &E : ctx->layouts)
        if (E.valid) {
            layout_dev_free(E.dev);
            bbh_layout_free(&E.host);
        }
    cudaFree(ctx->d_cd2i); cudaFree(ctx->d_cd2if); cudaFree(ctx->d_zig); cudaFree(ctx->d_taps);
    cudaFree(ctx->d_vedges); cudaFree(ctx->d_ptab); cudaFree(ctx->d_ptabf); cudaFree(ctx->d_vef);
    cudaFree(ctx->d_data); cudaFree(ctx->d_mask); cudaFree(ctx->d_region);
    for (auto &a : ctx->d_deff)
        for (auto &b : a) cudaFree(b);
    cudaFree(ctx->d_sub); cudaFree(ctx->d_mem); cudaFree(ctx->d_pix); cudaFree(ctx->d_bucket);
    cudaFree(ctx->d_tcount); cudaFree(ctx->d_toff); cudaFree(ctx->d_tcur); cudaFree(ctx->d_model); cudaFree(ctx->d_scan);
    cudaFree(ctx->d_smooth); cudaFree(ctx->d_model64); cudaFree(ctx->d_partial); cudaFree(ctx->d_out2);
    cudaFree(ctx->d_bimg); cudaFree(ctx->d_tmaps); cudaFree(ctx->d_tcq);
    for (auto &v : ctx->pool)
        for (auto &b : v) cudaFree(b.p);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    cudaFree(ctx->d_err);
    for (void *q : {(void *)ctx->d_ppix, (void *)ctx->d_lc, (void *)ctx->d_ord, (void *)ctx->d_p0, (void *)ctx->d_ent,
                    (void *)ctx->d_pw, (void *)ctx->d_pwy, (void *)ctx->d_lv, (void *)ctx->d_near, (void *)ctx->d_psub,
                    (void *)ctx->d_psbase, (void *)ctx->d_pssub, (void *)ctx->d_pcsf, (void *)ctx->d_pwidx, (void *)ctx->d_pfix,
                    (void *)ctx->d_pp, (void *)ctx->d_pstat, (void *)ctx->d_pcs, (void *)ctx->d_pzq,
                    (void *)ctx->d_pwval, (void *)ctx->d_rap, (void *)ctx->d_gpart, (void *)ctx->d_gh,
                    (void *)ctx->d_px, (void *)ctx->d_ppart, (void *)ctx->d_pzqf, (void *)ctx->d_pwqf,
                    (void *)ctx->d_pwvalf, (void *)ctx->d_maps32, (void *)ctx->d_K, (void *)ctx->d_maps64,
                    (void *)ctx->d_pmem, (void *)ctx->d_mstart, (void *)ctx->d_mseg, (void *)ctx->d_uidx,
                    (void *)ctx->d_ubase, (void *)ctx->d_prof_of, (void *)ctx->d_pstatu, (void *)ctx->d_pxu,
                    (void *)ctx->d_cstart, (void *)ctx->d_base64, (void *)ctx->d_cseg, (void *)ctx->d_klist,
                    (void *)ctx->d_tsrc, (void *)ctx->d_blk, (void *)ctx->d_ktab, (void *)ctx->d_gflag,
                    (void *)ctx->d_rp_rec, (void *)ctx->d_rp_cnt, (void *)ctx->d_chg, (void *)ctx->d_rp_n,
                    (void *)ctx->d_astart, (void *)ctx->d_aseg, (void *)ctx->d_mbase, (void *)ctx->d_tmask})
        cudaFree(q);
    for (void *q : {(void *)ctx->d_asub, (void *)ctx->d_asbase, (void *)ctx->d_assub, (void *)ctx->d_acs,
                    (void *)ctx->d_azq, (void *)ctx->d_awq, (void *)ctx->d_model_fx, (void *)ctx->d_acsf,
                    (void *)ctx->d_azqf, (void *)ctx->d_awqf, (void *)ctx->d_acsff})
        cudaFree(q);
    cudaFreeHost(ctx->h_asub);
    cudaFreeHost(ctx->h_reuse);
    cudaFreeHost(ctx->h_preuse);
    cudaFree(ctx->d_reuse);
    cudaFree(ctx->d_preuse);
    cudaFreeHost(ctx->h_psub);
    cudaFreeHost(ctx->h_sub); cudaFreeHost(ctx->h_mem); cudaFreeHost(ctx->h_out2); cudaFreeHost(ctx->h_err);
    for (int i = 0; i <= NTIMER; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    cudaGetLastError();
    delete ctx;
    return BBGPU_OK;
}

extern "C" const char *bbgpu_last_error(const bbgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

extern "C" int bbgpu_sync(bbgpu_ctx *ctx) {
    if (!ctx) return BBGPU_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    return BBGPU_OK;
}

extern "C" int64_t bbgpu_launch_count(const bbgpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int bbgpu_last_run_times(const bbgpu_ctx *ctx, double *times, int n) {
    if (!ctx || !times) return BBGPU_ERR_ARG;
    for (int i = 0; i < n && i < NTIMER; i++) times[i] = ctx->times[i];
    return NTIMER;
}

extern "C" const char *bbgpu_kernel_name(int i) { return (i >= 0 && i < NTIMER) ? KNAMES[i] : ""; }

extern "C" int bbgpu_shared_members(const bbgpu_ctx *ctx, int *profiles, int *mc_full, int *mc_delta,
                                    int *mc_replay) {
    if (!ctx) return BBGPU_ERR_ARG;
    const bool mc = ctx->galmodtype == BBGPU_MC && !ctx->mc_dirty;
    const bool an = ctx->galmodtype == BBGPU_ANALYTIC && !ctx->an_dirty;
    if (profiles) *profiles = ctx->prof_uploaded ? ctx->nu : 0;
    if (mc_full) *mc_full = mc ? ctx->mc_n1 : (an ? ctx->nb - ctx->an_n2 : 0);
    if (mc_delta) *mc_delta = mc ? ctx->mc_n2 : (an ? ctx->an_n2 : 0);
    if (mc_replay) *mc_replay = mc ? ctx->mc_n3 : 0;
    return BBGPU_OK;
}

extern "C" int bbgpu_transfer_bytes(const bbgpu_ctx *ctx, int64_t *h2d, int64_t *d2h) {
    if (!ctx) return BBGPU_ERR_ARG;
    if (h2d) *h2d = ctx->h2d;
    if (d2h) *d2h = ctx->d2h;
    return BBGPU_OK;
}

extern "C" int bbgpu_set_option(bbgpu_ctx *ctx, int opt, int value) {
    if (!ctx) return BBGPU_ERR_ARG;
    ctx->gen++;
    switch (opt) {
        case 1: ctx->keep_smoothed = value != 0; break;
        case 2: ctx->timing = value != 0; break;
        case 3:
            ctx->share = value != 0;
            ctx->mc_dirty = true;
            ctx->an_dirty = true;
            break;
        case 5: ctx->use_graphs = value != 0; break;
        case 4:
            if (value < -1 || value > 2)
                return fail(ctx, BBGPU_ERR_ARG, "option 4: convolution variant -1 (autotuned), 0, 1 or 2");
            ctx->conv_variant = value;
            break;
        default: return fail(ctx, BBGPU_ERR_ARG, "unknown option %d", opt);
    }
    return BBGPU_OK;
}

extern "C" int bbgpu_conv_variant(const bbgpu_ctx *ctx, int *used, float *tune_ms) {
    if (!ctx) return BBGPU_ERR_ARG;
    if (used) *used = ctx->conv_used;
    if (tune_ms)
        for (int i = 0; i < 3; i++) tune_ms[i] = ctx->tune_ms[i];
    return BBGPU_OK;
}

// ------------------------------------------------------------------------------------------- set-up
extern "C" int bbgpu_set_grid(bbgpu_ctx *ctx, const bbgpu_grid *gr, const double *cd2i, const double *lfreq0,
                              const double *relint, const double *vedges) {
    if (ctx) ctx->gen++;
    if (!ctx || !gr || !cd2i || !lfreq0 || !relint) return fail(ctx, BBGPU_ERR_ARG, "set_grid: null argument");
    if (gr->nx <= 0 || gr->ny <= 0 || gr->nz <= 0) return fail(ctx, BBGPU_ERR_ARG, "set_grid: empty cube");
    if (gr->nlines < 1 || gr->nlines > BBGPU_MAXL)
        return fail(ctx, BBGPU_ERR_ARG, "set_grid: %d lines (1 to %d supported)", gr->nlines, BBGPU_MAXL);
    if (!(gr->cdelt3 != 0) || !(gr->pixarea > 0) || !(gr->radsep > 0))
        return fail(ctx, BBGPU_ERR_ARG, "set_grid: invalid cdelt3, pixarea or radsep");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    GridDev &g = ctx->g;
    memset(&g, 0, sizeof g);
    g.nx = gr->nx; g.ny = gr->ny; g.nz = gr->nz; g.nlines = gr->nlines;
    g.axtyp = gr->axtyp; g.velsys = gr->velsys; g.ltype = gr->ltype; g.cmode = gr->cmode;
    g.radsep = gr->radsep; g.cdens = gr->cdens; g.pixarea = gr->pixarea; g.cdelt0 = gr->cdelt0; g.cdelt1 = gr->cdelt1;
    g.crota2 = gr->crota2; g.sig_instr = gr->sig_instr; g.crval3 = gr->crval3; g.cdelt3 = gr->cdelt3;
    g.crpix3 = gr->crpix3; g.chwidth = gr->chwidth; g.zstep = gr->zstep; g.scalefactor = gr->scalefactor;
    // bbarolo/galmod.py:103-105: the linear channel map of a velocity axis
    g.ia = 1.0 / g.cdelt3;
    g.ib = -g.crval3 / g.cdelt3 + g.crpix3 - 1;
    for (int nl = 0; nl < g.nlines; nl++) {
        g.lfreq0[nl] = lfreq0[nl];
        g.relint[nl] = relint[nl];
        if (g.axtyp == 4) {
            g.lia[nl] = (float)g.ia;
            g.lib[nl] = (float)g.ib;
        } else {
            // radio velocities on a frequency axis: channel = v (-f0 / (c cdelt3)) + (f0 - crval3) / cdelt3 + crpix3 - 1
            g.lia[nl] = (float)(-lfreq0[nl] / (2.99792458e08 * g.cdelt3));
            g.lib[nl] = (float)((lfreq0[nl] - g.crval3) / g.cdelt3 + g.crpix3 - 1);
        }
    }
    g.fast_ok = (g.axtyp == 4 && g.nlines == 1) || (g.axtyp == 3 && g.velsys == 1);
    if (g.axtyp == 4) {
        g.ia0 = g.ia;
        g.ib0 = g.ib;
    } else {
        g.ia0 = -lfreq0[0] / (2.99792458e08 * g.cdelt3);
        g.ib0 = (lfreq0[0] - g.crval3) / g.cdelt3 + g.crpix3 - 1;
    }
    g.vref = g.nz > 0 && vedges ? vedges[g.nz / 2] : 0.0;    // (the middle channel edge of line 0)
    {
        auto split = [](double v, float &hi, float &lo) {
            hi = (float)v;
            lo = (float)(v - (double)hi);
        };
        split(g.ia0, g.ia0h, g.ia0l);
        split(g.ib0, g.ib0h, g.ib0l);
        split(g.vref, g.vrefh, g.vrefl);
    }
    std::vector<float> cf(g.nz);
    for (int i = 0; i < g.nz; i++) cf[i] = (float)cd2i[i];
    cudaFree(ctx->d_cd2i);
    cudaFree(ctx->d_cd2if);
    ctx->d_cd2i = nullptr;
    ctx->d_cd2if = nullptr;
    CK(cudaMalloc(&ctx->d_cd2i, g.nz * sizeof(double)));
    CK(cudaMalloc(&ctx->d_cd2if, g.nz * sizeof(float)));
    CK(cudaMemcpy(ctx->d_cd2i, cd2i, g.nz * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_cd2if, cf.data(), g.nz * sizeof(float), cudaMemcpyHostToDevice));
    ctx->h_cd2i.assign(cd2i, cd2i + g.nz);
    cudaFree(ctx->d_vedges);
    cudaFree(ctx->d_vef);
    ctx->d_vedges = nullptr;
    ctx->d_vef = nullptr;
    if (vedges) {
        const size_t ne = (size_t)g.nlines * (g.nz + 1);
        CK(cudaMalloc(&ctx->d_vedges, ne * sizeof(double)));
        CK(cudaMemcpy(ctx->d_vedges, vedges, ne * sizeof(double), cudaMemcpyHostToDevice));
        std::vector<float2> vef(g.nz + 1);
        for (int k = 0; k <= g.nz; k++) {
            const double d = vedges[k] - g.vref;
            vef[k].x = (float)d;
            vef[k].y = (float)(d - (double)vef[k].x);
        }
        CK(cudaMalloc(&ctx->d_vef, vef.size() * sizeof(float2)));
        CK(cudaMemcpy(ctx->d_vef, vef.data(), vef.size() * sizeof(float2), cudaMemcpyHostToDevice));
    }
    if (!ctx->d_ptab) {
        std::vector<double> tab(6146);
        bbh_phi_table(tab.data());
        std::vector<float> tf(tab.begin(), tab.end());
        CK(cudaMalloc(&ctx->d_ptab, tab.size() * sizeof(double)));
        CK(cudaMemcpy(ctx->d_ptab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&ctx->d_ptabf, tf.size() * sizeof(float)));
        CK(cudaMemcpy(ctx->d_ptabf, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    // deposit tile: pixels x channels of 8-byte sums within 56 KB (3 CTAs per SM with the staging buffers)
    int tp = 57344 / (8 * g.nz);
    if (tp >= 64) { ctx->tx = 8; ctx->ty = 8; }
    else if (tp >= 32) { ctx->tx = 8; ctx->ty = 4; }
    else if (tp >= 16) { ctx->tx = 4; ctx->ty = 4; }
    else if (tp >= 8) { ctx->tx = 4; ctx->ty = 2; }
    else if (tp >= 2) { ctx->tx = 2; ctx->ty = 1; }
    else { ctx->tx = 1; ctx->ty = 1; }
    for (auto &E : ctx->layouts)
        if (E.valid) {
            layout_dev_free(E.dev);
            bbh_layout_free(&E.host);
            E.valid = false;
        }
    ctx->zcache.clear();
    ctx->samp_key.clear();
    ctx->prof_set = ctx->prof_uploaded = false;
    ctx->grid_set = true;
    ctx->uploaded = ctx->ran = false;
    return BBGPU_OK;
}

extern "C" int bbgpu_set_kernel(bbgpu_ctx *ctx, const double *kernel, int ky, int kx) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!kernel || ky < 1 || kx < 1 || !(ky & 1) || !(kx & 1) || ky > BBGPU_MAXK || kx > BBGPU_MAXK)
        return fail(ctx, BBGPU_ERR_ARG, "set_kernel: kernel sides must be odd, 1 to %d", BBGPU_MAXK);
    // the shared-memory templates of k_conv_resid take widths up to 31 and tiles up to 220 KB; a wider kernel
    // (kxw = 0) keeps all its taps and runs k_conv_wide
    std::vector<float> taps((size_t)ky * std::max(kx, 31));
    int kxw = conv_taps(kernel, ky, kx, taps.data());
    if (kxw && (size_t)(16 + ky - 1) * (16 + kxw - 1) * 32 * 4 + (size_t)ky * kxw * 4 > 220 * 1024) kxw = 0;
    if (!kxw) conv_wide_taps(kernel, ky, kx, taps.data());
    const size_t ntaps = (size_t)ky * (kxw ? kxw : kx);
    CK(cudaSetDevice(ctx->device));
    cudaFree(ctx->d_taps);
    ctx->d_taps = nullptr;
    CK(cudaMalloc(&ctx->d_taps, ntaps * sizeof(float)));
    CK(cudaMemcpy(ctx->d_taps, taps.data(), ntaps * sizeof(float), cudaMemcpyHostToDevice));
    ctx->ky = ky;
    ctx->kx = kx;
    ctx->kxw = kxw;
    ctx->h_kernel.assign(kernel, kernel + (size_t)ky * kx);
    ctx->bimg_variant = 0;
    ctx->tuned.clear();
    ctx->kernel_set = true;
    return BBGPU_OK;
}

extern "C" int bbgpu_set_cube(bbgpu_ctx *ctx, const float *data, const uint8_t *mask, const uint8_t *region) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!ctx->grid_set) return fail(ctx, BBGPU_ERR_STATE, "set_cube before set_grid");
    if (!data) return fail(ctx, BBGPU_ERR_ARG, "set_cube: null data");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    size_t n = (size_t)ctx->g.nx * ctx->g.ny * ctx->g.nz;
    cudaFree(ctx->d_data); cudaFree(ctx->d_mask); cudaFree(ctx->d_region);
    ctx->d_data = nullptr; ctx->d_mask = nullptr; ctx->d_region = nullptr;
    for (auto &a : ctx->d_deff)
        for (auto &b : a) { cudaFree(b); b = nullptr; }
    CK(cudaMalloc(&ctx->d_data, n * sizeof(float)));
    CK(cudaMemcpy(ctx->d_data, data, n * sizeof(float), cudaMemcpyHostToDevice));
    if (mask) {
        CK(cudaMalloc(&ctx->d_mask, n));
        CK(cudaMemcpy(ctx->d_mask, mask, n, cudaMemcpyHostToDevice));
    }
    if (region) {
        CK(cudaMalloc(&ctx->d_region, (size_t)ctx->g.nx * ctx->g.ny));
        CK(cudaMemcpy(ctx->d_region, region, (size_t)ctx->g.nx * ctx->g.ny, cudaMemcpyHostToDevice));
    }
    ctx->cube_set = true;
    return BBGPU_OK;
}

// ------------------------------------------------------------------------------------------- batches
// The member descriptor of a batch (box, residual options, data view).
static int member_desc(bbgpu_ctx *ctx, int k, const bbgpu_eval_desc &d, int fix_exp, bool need_cube, MemberDev &M) {
    const GridDev &g = ctx->g;
    if (d.blo0 < 0 || d.blo1 < 0 || d.bhi0 > g.nx || d.bhi1 > g.ny || d.bhi0 < d.blo0 || d.bhi1 < d.blo1)
        return fail(ctx, BBGPU_ERR_ARG, "eval: member %d: box outside the cube", k);
    if (d.eps2 > 0 && !(d.sigma2 > 0)) return fail(ctx, BBGPU_ERR_ARG, "eval: member %d: eps2 > 0 needs sigma2 > 0", k);
    memset(&M, 0, sizeof M);
    M.blo0 = d.blo0; M.blo1 = d.blo1; M.bhi0 = d.bhi0; M.bhi1 = d.bhi1;
    M.bx = d.bhi0 - d.blo0; M.by = d.bhi1 - d.blo1;
    M.fix_exp = fix_exp;
    M.maskmode = d.maskmode;
    M.use_region = d.use_region;
    M.sigma2 = d.sigma2;
    M.eps2 = d.eps2;
    M.sigma2f = (float)d.sigma2;
    M.eps2f = (float)d.eps2;
    if (need_cube) {
        int rc = ensure_deff(ctx, d.maskmode, d.use_region);
        if (rc) return rc;
        M.deff = ctx->d_deff[d.maskmode][d.use_region ? 1 : 0];
    }
    return 0;
}

// An ANALYTIC batch (bbarolo/galmod.py:326-465 per member): the sub-ring constants of every member on the host
// (vertical grids shared through a cache), the azimuthal samples of the shared radii, all uploaded; the members
// may differ in every ring value but the radii.
static int batch_prepare_analytic(bbgpu_ctx *ctx, int nb, int nsub, const double *sr, const bbgpu_eval_desc *descs,
                                  bool need_cube) {
    const GridDev &g = ctx->g;
    if (!ctx->d_vedges) return fail(ctx, BBGPU_ERR_STATE, "eval: ANALYTIC batch, but set_grid was given no channel edges");
    if (an_smem_bytes(g.nz, g.nlines) > AN_SMEM_MAX)
        return fail(ctx, BBGPU_ERR_ARG, "eval: %d channels x %d lines above the ANALYTIC kernel's limit", g.nz, g.nlines);
    for (int k = 1; k < nb; k++)
        if (memcmp(sr + (size_t)k * BBGPU_NSR * nsub, sr, sizeof(double) * nsub))
            return fail(ctx, BBGPU_ERR_ARG, "eval: member %d has other radii: evaluate it in another batch", k);
    int rc;
    if ((rc = hgrow(ctx, &ctx->h_asub, &ctx->h_asub_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_mem, &ctx->h_mem_cap, (size_t)nb))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_reuse, &ctx->h_reuse_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    ctx->mem_host.resize(nb);
    ZgridCache &zc = ctx->azcache;
    if (zc.zq.size() > ((size_t)1 << 24)) zc.clear();
    int nzq0 = 1;
    for (int k = 0; k < nb; k++) {
        const bbgpu_eval_desc &d = descs[k];
        const double *s = sr + (size_t)k * BBGPU_NSR * nsub;
        int nzq = 1;                                // bbarolo/galmod.py:912: vertical samples for a thick layer
        for (int i = 0; i < nsub; i++)
            if (s[6 * (size_t)nsub + i] > 0) { nzq = 1024; break; }
        if (k == 0) nzq0 = nzq;
        // the constants of a sub-ring whose column equals member 0's are member 0's when the box and the vertical
        // sampling are the same (the vertical grid depends on the box)
        const bool reuse = k > 0 && nzq == nzq0 && d.blo0 == descs[0].blo0 && d.blo1 == descs[0].blo1 &&
                           d.bhi0 == descs[0].bhi0 && d.bhi1 == descs[0].bhi1;
        if (d.blo0 < 0 || d.blo1 < 0 || d.bhi0 > g.nx || d.bhi1 > g.ny || d.bhi0 < d.blo0 || d.bhi1 < d.blo1)
            return fail(ctx, BBGPU_ERR_ARG, "eval: member %d: box outside the cube", k);
        signed char *ru = ctx->h_reuse + (size_t)k * nsub;
        memset(ru, 0, (size_t)nsub);
        const int e = bbh_an_subs(s, nsub, &g, nzq, d.blo0, d.blo1, d.bhi0, d.bhi1, ctx->h_cd2i.data(), 0, nullptr,
                                  nullptr, ctx->h_asub + (size_t)k * nsub, zc, reuse ? sr : nullptr,
                                  reuse ? ctx->h_asub : nullptr, reuse ? ru : nullptr);
        if (e == -10000) return fail(ctx, BBGPU_ERR_ARG, "eval: member %d: the total flux is not finite", k);
        if ((rc = member_desc(ctx, k, d, e, need_cube, ctx->mem_host[k]))) return rc;
        ctx->h_mem[k] = ctx->mem_host[k];
    }
    ctx->nb = nb;
    ctx->nsub = nsub;
    ctx->galmodtype = BBGPU_ANALYTIC;
    ctx->an_dirty = true;
    ctx->lean = 0;
    ctx->ntile_total = 0;
    ctx->mstride = (long long)g.nx * g.ny * g.nz;
    ctx->npart = std::max(conv_resid_npart(ctx->mem_host.data(), nb, g.nz), conv_tc_npart(ctx->mem_host.data(), nb, g.nz));
    ctx->h2d = 0;
    // the azimuthal samples of the radii (uploaded when the radii change)
    std::string key((const char *)sr, sizeof(double) * nsub);
    key.append((const char *)&g.pixarea, sizeof(double));
    if (key != ctx->asamp_key) {
        std::vector<int> sbase, ssub;
        std::vector<double> cs;
        bbh_an_samples(sr, nsub, &g, sbase, ssub, cs);
        if ((rc = dgrow(ctx, &ctx->d_asbase, &ctx->d_asbase_cap, sbase.size()))) return rc;
        if ((rc = dgrow(ctx, &ctx->d_assub, &ctx->d_assub_cap, ssub.size() ? ssub.size() : 1))) return rc;
        if ((rc = dgrow(ctx, &ctx->d_acs, &ctx->d_acs_cap, cs.size() ? cs.size() : 1))) return rc;
        std::vector<float> csf;
        bbh_an_samples_f32(cs, csf);
        if ((rc = dgrow(ctx, &ctx->d_acsf, &ctx->d_acsf_cap, csf.size() ? csf.size() : 1))) return rc;
        if (csf.size()) CK(cudaMemcpy(ctx->d_acsf, csf.data(), sizeof(float) * csf.size(), cudaMemcpyHostToDevice));
        std::vector<float4> csff(cs.size() / 2);
        for (size_t q = 0; q < csff.size(); q++) {
            const double c = cs[2 * q], sn = cs[2 * q + 1];
            csff[q].x = (float)c;
            csff[q].y = (float)(c - (double)csff[q].x);
            csff[q].z = (float)sn;
            csff[q].w = (float)(sn - (double)csff[q].z);
        }
        if ((rc = dgrow(ctx, &ctx->d_acsff, &ctx->d_acsff_cap, csff.size() ? csff.size() : 1))) return rc;
        if (csff.size())
            CK(cudaMemcpy(ctx->d_acsff, csff.data(), sizeof(float4) * csff.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_asbase, sbase.data(), sizeof(int) * sbase.size(), cudaMemcpyHostToDevice));
        if (ssub.size()) CK(cudaMemcpy(ctx->d_assub, ssub.data(), sizeof(int) * ssub.size(), cudaMemcpyHostToDevice));
        if (cs.size()) CK(cudaMemcpy(ctx->d_acs, cs.data(), sizeof(double) * cs.size(), cudaMemcpyHostToDevice));
        ctx->ansamp = sbase[nsub];
        ctx->asbase_host = sbase;
        ctx->asamp_key = key;
        ctx->h2d += (long long)(sizeof(int) * (sbase.size() + ssub.size()) + sizeof(double) * cs.size());
    }
    // the vertical grids: the new ones appended on the device (the table grows with a copy of the whole)
    const size_t nz1 = zc.zq.size() + 1;
    if (zc.uploaded == 0 || nz1 > ctx->d_azq_cap) {
        if (nz1 > ctx->d_azq_cap) {
            for (void *q : {(void *)ctx->d_azq, (void *)ctx->d_awq, (void *)ctx->d_azqf, (void *)ctx->d_awqf}) cudaFree(q);
            ctx->d_azq = ctx->d_awq = nullptr;
            ctx->d_azqf = ctx->d_awqf = nullptr;
            ctx->d_azq_cap = ctx->d_awq_cap = ctx->d_azqf_cap = ctx->d_awqf_cap = 0;
            if ((rc = dgrow(ctx, &ctx->d_azq, &ctx->d_azq_cap, 2 * nz1))) return rc;
            if ((rc = dgrow(ctx, &ctx->d_awq, &ctx->d_awq_cap, 2 * nz1))) return rc;
            if ((rc = dgrow(ctx, &ctx->d_azqf, &ctx->d_azqf_cap, 2 * nz1))) return rc;
            if ((rc = dgrow(ctx, &ctx->d_awqf, &ctx->d_awqf_cap, 2 * nz1))) return rc;
        }
        zc.uploaded = 0;
    }
    if (zc.zq.size() > zc.uploaded) {
        const size_t a0 = zc.uploaded, m = zc.zq.size() - a0;
        std::vector<float> zf(m), wf(m);
        for (size_t i = 0; i < m; i++) {
            zf[i] = (float)zc.zq[a0 + i];
            wf[i] = (float)zc.wq[a0 + i];
        }
        CK(cudaMemcpy(ctx->d_azq + a0, zc.zq.data() + a0, sizeof(double) * m, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_awq + a0, zc.wq.data() + a0, sizeof(double) * m, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_azqf + a0, zf.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_awqf + a0, wf.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
        ctx->h2d += (long long)(24 * m);
        zc.uploaded = zc.zq.size();
    }
    if ((rc = dgrow(ctx, &ctx->d_asub, &ctx->d_asub_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_mem, &ctx->d_mem_cap, (size_t)nb))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_model, &ctx->d_model_cap, (size_t)nb * ctx->mstride))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_model_fx, &ctx->d_model_fx_cap, (size_t)nb * ctx->mstride))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_partial, &ctx->d_partial_cap, (size_t)2 * nb * (ctx->npart ? ctx->npart : 1)))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_out2, &ctx->d_out2_cap, (size_t)2 * nb))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_out2, &ctx->h_out2_cap, (size_t)2 * nb))) return rc;
    if (ctx->keep_smoothed)
        if ((rc = dgrow(ctx, &ctx->d_smooth, &ctx->d_smooth_cap, (size_t)nb * ctx->mstride))) return rc;
    if (ctx->want64)
        if ((rc = dgrow(ctx, &ctx->d_model64, &ctx->d_model64_cap, (size_t)nb * ctx->mstride))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_reuse, &ctx->d_reuse_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    // which ANALYTIC kernels the batch needs: the float32 path of thin sub-rings (one height), of thick ones, the
    // exact kernel for the others (a reused column is member 0's, whose flags count already)
    ctx->an_thin = ctx->an_thick = ctx->an_exact = 0;
    for (size_t i = 0; i < (size_t)nb * nsub; i++) {
        if (ctx->h_reuse[i]) continue;
        const AnSub &S = ctx->h_asub[i];
        if (!S.active) continue;
        if (!S.anfast) ctx->an_exact = 1;
        else if (S.nzz == 1) ctx->an_thin = 1;
        else ctx->an_thick = 1;
    }
    CK(cudaMemcpyAsync(ctx->d_asub, ctx->h_asub, sizeof(AnSub) * (size_t)nb * nsub, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_mem, ctx->h_mem, sizeof(MemberDev) * (size_t)nb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_reuse, ctx->h_reuse, (size_t)nb * nsub, cudaMemcpyHostToDevice, ctx->stream));
    launch_fill_copy(ctx->stream, ctx->d_asub, sizeof(AnSub), nsub, nb, ctx->d_reuse);
    CKL();
    ctx->h2d += (long long)((sizeof(AnSub) + 1) * (size_t)nb * nsub + sizeof(MemberDev) * (size_t)nb);
    ctx->uploaded = true;
    ctx->ran = false;
    return 0;
}

static int batch_prepare(bbgpu_ctx *ctx, int galmodtype, int nb, int nsub, const double *sr, const int64_t *nv,
                         const bbgpu_eval_desc *descs, bool need_cube) {
    ctx->prof_uploaded = false;       // (a new batch: its ring maps come with bbgpu_eval_upload_profile)
    if (!ctx->grid_set) return fail(ctx, BBGPU_ERR_STATE, "evaluation before set_grid");
    if (need_cube && !ctx->cube_set) return fail(ctx, BBGPU_ERR_STATE, "evaluation before set_cube");
    if (galmodtype != BBGPU_MC && galmodtype != BBGPU_ANALYTIC)
        return fail(ctx, BBGPU_ERR_ARG, "galmodtype %d not supported by the batch path", galmodtype);
    if (nb < 1 || nsub < 0 || !sr || !nv || !descs) return fail(ctx, BBGPU_ERR_ARG, "eval: invalid batch");
    if (galmodtype == BBGPU_ANALYTIC) return batch_prepare_analytic(ctx, nb, nsub, sr, descs, need_cube);
    const GridDev &g = ctx->g;
    std::vector<int> nc0(nsub), nv0(nsub), nc(nsub), nvv(nsub);
    std::vector<double> R0(nsub);
    for (int i = 0; i < nsub; i++) R0[i] = sr[i];
    bbh_cloud_counts(sr, nsub, nv, &g, nc0.data(), nv0.data());
    uint64_t seed = descs[0].seed;
    for (int k = 1; k < nb; k++) {
        const double *s = sr + (size_t)k * BBGPU_NSR * nsub;
        // (the counts are a function of the radii, densities and velocity samples: equal rows, equal counts)
        if (descs[k].seed == seed && !memcmp(s, sr, sizeof(double) * nsub) &&
            !memcmp(s + (size_t)5 * nsub, sr + (size_t)5 * nsub, sizeof(double) * nsub) &&
            !memcmp(nv + (size_t)k * nsub, nv, sizeof(int64_t) * nsub))
            continue;
        bbh_cloud_counts(s, nsub, nv + (size_t)k * nsub, &g, nc.data(), nvv.data());
        if (descs[k].seed != seed || memcmp(nc.data(), nc0.data(), sizeof(int) * nsub) ||
            memcmp(nvv.data(), nv0.data(), sizeof(int) * nsub) || memcmp(s, sr, sizeof(double) * nsub))
            return fail(ctx, BBGPU_ERR_ARG,
                        "eval: member %d has another cloud layout (seed, radii, cloud or velocity counts): "
                        "evaluate it in another batch", k);
    }
    for (int i = 0; i < nsub; i++)
        if (nv0[i] > 65535) return fail(ctx, BBGPU_ERR_ARG, "eval: NV above 65535 velocity samples per cloud");
    LayoutEntry *E = nullptr;
    int rc = get_layout(ctx, seed, nsub, nc0.data(), nv0.data(), R0.data(), &E);
    if (rc) return rc;
    ctx->cur = E;
    if ((rc = hgrow(ctx, &ctx->h_sub, &ctx->h_sub_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_mem, &ctx->h_mem_cap, (size_t)nb))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_reuse, &ctx->h_reuse_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    memset(ctx->h_reuse, 0, (size_t)nsub);
    ctx->mem_host.resize(nb);
    std::vector<uint16_t> dmask((size_t)nsub);
    ctx->mc_same_nd.assign((size_t)nb * nsub, 1);
    int toff = 0;
    for (int k = 0; k < nb; k++) {
        const bbgpu_eval_desc &d = descs[k];
        if (d.blo0 < 0 || d.blo1 < 0 || d.bhi0 > g.nx || d.bhi1 > g.ny || d.bhi0 < d.blo0 || d.bhi1 < d.blo1)
            return fail(ctx, BBGPU_ERR_ARG, "eval: member %d: box outside the cube", k);
        SubMC *S = ctx->h_sub + (size_t)k * nsub;
        // (the rows of each column that differ from member 0's: the constants reused, and the columns that
        // differ in the density only)
        if (k) bbh_column_diff(sr + (size_t)k * BBGPU_NSR * nsub, sr, nsub, dmask.data());
        int e = bbh_submc(sr + (size_t)k * BBGPU_NSR * nsub, nsub, nc0.data(), nv0.data(), &g, S,
                          k ? sr : nullptr, k ? ctx->h_sub : nullptr, k ? ctx->h_reuse + (size_t)k * nsub : nullptr,
                          k ? dmask.data() : nullptr);
        if (k)
            for (int ir = 0; ir < nsub; ir++)
                ctx->mc_same_nd[(size_t)k * nsub + ir] = (dmask[ir] & ~(1u << 5)) ? 0 : 1;
        MemberDev &M = ctx->mem_host[k];
        if ((rc = member_desc(ctx, k, d, e, need_cube, M))) return rc;
        M.ntx = (M.bx + ctx->tx - 1) / ctx->tx;
        M.nty = (M.by + ctx->ty - 1) / ctx->ty;
        M.tile_off = toff;
        toff += M.ntx * M.nty;
        ctx->h_mem[k] = M;
    }
    ctx->nb = nb;
    ctx->nsub = nsub;
    ctx->galmodtype = galmodtype;
    {
        int maxnv = 0;
        for (int i = 0; i < nsub; i++) maxnv = nv0[i] > maxnv ? nv0[i] : maxnv;
        ctx->lean = g.fast_ok && g.nlines == 1 && maxnv <= 128;
    }
    ctx->ntile_total = toff;
    ctx->mc_dirty = true;
    ctx->mstride = (long long)g.nx * g.ny * g.nz;
    ctx->npart = std::max(conv_resid_npart(ctx->mem_host.data(), nb, g.nz), conv_tc_npart(ctx->mem_host.data(), nb, g.nz));
    size_t ncl = (size_t)nb * (E->host.ncloud ? E->host.ncloud : 1);
    if ((rc = dgrow(ctx, &ctx->d_sub, &ctx->d_sub_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_mem, &ctx->d_mem_cap, (size_t)nb))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pix, &ctx->d_pix_cap, ncl))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_bucket, &ctx->d_bucket_cap, ncl * (ENTRY_BYTES / 16)))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_tcount, &ctx->d_tcount_cap, (size_t)toff * NOWN + 1))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_toff, &ctx->d_toff_cap, (size_t)toff * NOWN + 1))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_tcur, &ctx->d_tcur_cap, (size_t)toff * NOWN + 1))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_scan, &ctx->d_scan_cap, (size_t)toff * NOWN / 1024 + 2))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_model, &ctx->d_model_cap, (size_t)nb * ctx->mstride))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_partial, &ctx->d_partial_cap, (size_t)2 * nb * (ctx->npart ? ctx->npart : 1)))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_out2, &ctx->d_out2_cap, (size_t)2 * nb))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_out2, &ctx->h_out2_cap, (size_t)2 * nb))) return rc;
    if (ctx->keep_smoothed)
        if ((rc = dgrow(ctx, &ctx->d_smooth, &ctx->d_smooth_cap, (size_t)nb * ctx->mstride))) return rc;
    if (ctx->want64)
        if ((rc = dgrow(ctx, &ctx->d_model64, &ctx->d_model64_cap, (size_t)nb * ctx->mstride))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_reuse, &ctx->d_reuse_cap, (size_t)nb * (nsub ? nsub : 1)))) return rc;
    CK(cudaMemcpyAsync(ctx->d_sub, ctx->h_sub, sizeof(SubMC) * (size_t)nb * nsub, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_mem, ctx->h_mem, sizeof(MemberDev) * (size_t)nb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_reuse, ctx->h_reuse, (size_t)nb * nsub, cudaMemcpyHostToDevice, ctx->stream));
    launch_fill_submc(ctx->stream, ctx->d_sub, nsub, nb, ctx->d_reuse, ctx->d_mem, g.nlines);
    CKL();
    ctx->h2d = (long long)((sizeof(SubMC) + 1) * (size_t)nb * nsub + sizeof(MemberDev) * (size_t)nb);
    ctx->uploaded = true;
    ctx->ran = false;
    return 0;
}

// The flux normalisation of the batch (bbarolo/bayesian/likelihood.py:595-596): ring maps, beam convolution,
// normal equations, the profile solve and the densities of the model's sub-rings, all on the device.
static int profile_run(bbgpu_ctx *ctx, bool tm) {
    const GridDev &g = ctx->g;
    cudaStream_t s = ctx->stream;
    const ProfBox &bx = ctx->pbox;
    const int nb = ctx->nb, n = ctx->pc.n, nu = ctx->nu;
    const long long per = bx.npix * bx.nrp;
    CK(cudaMemsetAsync(ctx->d_maps64, 0, sizeof(long long) * (size_t)nu * per, s));
    launch_an_maps_fast(s, g, ctx->d_psub, ctx->nsm, ctx->d_psbase, ctx->d_pssub, ctx->d_pcs, ctx->d_pcsf,
                        ctx->d_mstart, ctx->d_mseg, ctx->nseg, ctx->mtot, ctx->d_pzq, ctx->d_pzqf, ctx->d_pwqf,
                        ctx->d_pwidx, ctx->d_pwvalf, bx, ctx->d_pfix, ctx->d_maps64);
    CKL();
    const bool shared = ctx->nu_delta > 0 && per < (1LL << 31);      // (the block table indexes in 32 bits)
    launch_maps_to_f32(s, ctx->d_maps64, ctx->d_pfix, ctx->d_uidx, ctx->d_ubase, nu, per, (float)ctx->mapscale,
                       ctx->d_maps32, shared ? ctx->d_blk : nullptr, bx);
    CKL();
    if (shared) ctx->launches++;      // (the block table's initialisation)
    int nct = 0, ntxc = 0, shx = 0, shy = 0;
    conv_tile_shape(bx.nrp, bx.bx, bx.by, nct, ntxc, shx, shy);
    if (tm) CK(cudaEventRecord(ctx->ev[1], s));
    if (ctx->kernel_set) {
        launch_conv_resid(s, g, ctx->d_pmem, ctx->pmem_host.data(), nu, ctx->d_maps32, per, bx.nrp, ctx->d_taps,
                          ctx->ky, ctx->kx, ctx->kxw, ctx->d_K, 2, 0, ctx->d_ppart,
                          shared ? TileSrc{ctx->d_blk, 3, 3, ctx->d_ktab, nct} : TileSrc{nullptr, 0, 0, nullptr, 0});
        CKL();
    }
    if (tm) CK(cudaEventRecord(ctx->ev[2], s));
    const float *K = ctx->kernel_set ? ctx->d_K : ctx->d_maps32;
    launch_prof_gram(s, K, bx, ctx->d_ppix, ctx->d_pw, ctx->d_pwy, ctx->npix_used, ctx->d_ent, ctx->d_ent + ctx->nent,
                     ctx->nent, nu, ctx->d_gpart, ctx->d_gh,
                     shared && ctx->kernel_set
                         ? KRows{ctx->d_ktab, nct, ntxc, shx, shy, ctx->d_gflag,
                                 ctx->ky / 2 <= 8 && ctx->kx / 2 <= 8 ? ctx->d_blk : nullptr, (bx.bx + 7) / 8,
                                 (bx.by + 7) / 8}
                         : KRows{});
    ctx->launches += 2;
    CKL();
    if (tm) CK(cudaEventRecord(ctx->ev[3], s));
    launch_prof_solve(s, ctx->d_gh, ctx->pc, ctx->d_lc, ctx->d_lv, ctx->d_ord, ctx->d_near, ctx->d_p0, nu,
                      ctx->d_pxu, ctx->d_pp, ctx->d_pstatu);
    CKL();
    launch_prof_gather(s, ctx->d_pxu, ctx->d_pstatu, ctx->d_prof_of, nb, n, ctx->d_px, ctx->d_pstat);
    CKL();
    if (ctx->galmodtype == BBGPU_ANALYTIC) {
        double lsum = 0.0, cmax = 0.0;
        for (int nl = 0; nl < g.nlines; nl++) lsum += fabs(g.relint[nl]);
        for (double c : ctx->h_cd2i) cmax = std::max(cmax, fabs(c));
        launch_an_dens(s, g, ctx->d_asub, ctx->nsub, ctx->d_mem, nb, ctx->d_px, n, ctx->d_pwidx, ctx->d_pwval,
                       ctx->d_rap, lsum * cmax, ctx->d_err);
    } else {
        launch_mc_dens(s, g, ctx->d_sub, ctx->nsub, ctx->d_mem, nb, ctx->d_px, n, ctx->d_pwidx, ctx->d_pwval,
                       ctx->d_rap, ctx->d_err);
    }
    CKL();
    if (tm) CK(cudaEventRecord(ctx->ev[4], s));
    (void)per;
    return 0;
}

// The (member, cloud) segments of an MC batch. A member k > 0 whose model is member 0's but for a few sub-rings
// (the columns that differ from member 0's), with member 0's box and fixed-point exponent (the host's, or with a
// flux normalisation member 0's profile: the same densities), is computed as member 0's fixed-point sums plus
// the deposits of those sub-rings' clouds with its constants, minus the same clouds with member 0's (exact: the
// sums are modulo 2^64 and equal clouds deposit equal integers). The deposit of such a member reads member 0's
// sums, so it runs in a second launch. Every other member deposits all its clouds.
static int ilog2(int v) {
    int e = 0;
    while ((1 << (e + 1)) <= v) e++;
    return e;
}

static int mc_segments(bbgpu_ctx *ctx) {
    const int nb = ctx->nb, nsub = ctx->nsub;
    const LayoutHost &L = ctx->cur->host;
    const long long ncl = L.ncloud;
    std::vector<long long> &cs = ctx->h_cstart;
    std::vector<int> &sg = ctx->h_cseg, &kl = ctx->h_klist;
    cs.clear();
    sg.clear();
    kl.clear();
    long long tot = 0;
    auto seg = [&](int k, int src, int c0, int sign, long long n) {
        if (n <= 0) return;
        cs.push_back(tot);
        sg.insert(sg.end(), {k, src, c0, sign});
        tot += n;
    };
    const bool can = ctx->share && nb > 1 && mc_deposit_shares(ctx->lean, ctx->want64, ctx->tx, ctx->ty) &&
                     (!ctx->prof_uploaded || (int)ctx->prof_of_host.size() == nb);
    const MemberDev &M0 = ctx->mem_host[0];
    std::vector<int> dl, rl;
    ctx->mc_isdelta.assign(nb, 0);
    // replay: the spread of a cloud's channels within the window (the layout's largest spread of normals times
    // member 0's channels per unit normal)
    double sgmax = 0.0;
    for (int ir = 0; ir < nsub; ir++) sgmax = std::max(sgmax, (double)fabsf(ctx->h_sub[ir].sg[0]));
    const bool rp_ok = can && ctx->cur->zspan * sgmax + 3.0 < (double)RP_W;
    ctx->nchw = (nsub + 63) / 64;
    ctx->h_chg.assign((size_t)nb * (ctx->nchw ? ctx->nchw : 1), 0ULL);
    for (int k = 0; k < nb; k++) {
        if (can && k > 0) {
            const MemberDev &M = ctx->mem_host[k];
            bool ok = M.blo0 == M0.blo0 && M.blo1 == M0.blo1 && M.bx == M0.bx && M.by == M0.by;
            if (ok) ok = ctx->prof_uploaded ? ctx->prof_of_host[k] == 0 : M.fix_exp == M0.fix_exp;
            if (ok) {
                const signed char *ru = ctx->h_reuse + (size_t)k * nsub;
                long long nch = 0;
                for (int ir = 0; ir < nsub; ir++)
                    if (!ru[ir]) nch += L.nc[ir];
                if (2 * nch < ncl) {
                    // (with member 0's records, its clouds of the changed sub-rings are taken out by their counts)
                    unsigned long long *cm = ctx->h_chg.data() + (size_t)k * ctx->nchw;
                    for (int ir = 0; ir < nsub; ir++)
                        if (!ru[ir]) {
                            seg(k, k, L.cloud_base[ir], 1, L.nc[ir]);
                            if (!rp_ok) seg(k, 0, L.cloud_base[ir], -1, L.nc[ir]);
                            cm[ir >> 6] |= 1ULL << (ir & 63);
                        }
                    dl.push_back(k);
                    ctx->mc_isdelta[k] = 1;
                    continue;
                }
            }
            const bool box = M.blo0 == M0.blo0 && M.blo1 == M0.blo1 && M.bx == M0.bx && M.by == M0.by;
            if (rp_ok && box) {
                // member 0's clouds but for the flux, except in a few sub-rings (which it deposits itself)
                const signed char *sn = ctx->mc_same_nd.data() + (size_t)k * nsub;
                long long nch = 0;
                for (int ir = 0; ir < nsub; ir++)
                    if (!sn[ir]) nch += L.nc[ir];
                if (2 * nch < ncl) {
                    unsigned long long *cm = ctx->h_chg.data() + (size_t)k * ctx->nchw;
                    for (int ir = 0; ir < nsub; ir++)
                        if (!sn[ir]) {
                            seg(k, k, L.cloud_base[ir], 1, L.nc[ir]);
                            cm[ir >> 6] |= 1ULL << (ir & 63);
                        }
                    rl.push_back(k);
                    continue;
                }
            }
        }
        seg(k, k, 0, 1, ncl);
        kl.push_back(k);
    }
    ctx->mc_n1 = (int)kl.size();
    ctx->mc_n2 = (int)dl.size();
    ctx->mc_n3 = (int)rl.size();
    kl.insert(kl.end(), dl.begin(), dl.end());
    kl.insert(kl.end(), rl.begin(), rl.end());
    cs.push_back(tot);
    ctx->mc_nseg = (int)cs.size() - 1;
    ctx->mc_ntot = tot;
    int rc;
    if ((rc = dgrow(ctx, &ctx->d_cstart, &ctx->d_cstart_cap, cs.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_cseg, &ctx->d_cseg_cap, sg.size() + 4))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_klist, &ctx->d_klist_cap, kl.size()))) return rc;
    if (ctx->mc_n2 &&
        ((rc = dgrow(ctx, &ctx->d_base64, &ctx->d_base64_cap, (size_t)M0.bx * M0.by * ctx->g.nz + 1)) ||
         (rc = dgrow(ctx, &ctx->d_tsrc, &ctx->d_tsrc_cap, (size_t)ctx->ntile_total + 1))))
        return rc;
    ctx->mc_records = rp_ok && (ctx->mc_n2 || ctx->mc_n3);
    if (ctx->mc_records) {
        if ((rc = dgrow(ctx, &ctx->d_rp_rec, &ctx->d_rp_rec_cap, 2 * (size_t)ncl + 2)) ||
            (rc = dgrow(ctx, &ctx->d_rp_cnt, &ctx->d_rp_cnt_cap, (size_t)ncl * (RP_W / 2) + 1)) ||
            (rc = dgrow(ctx, &ctx->d_rp_n, &ctx->d_rp_n_cap, (size_t)(M0.ntx * M0.nty) * NOWN + 1)) ||
            (rc = dgrow(ctx, &ctx->d_tmask, &ctx->d_tmask_cap, (size_t)(M0.ntx * M0.nty) * ctx->nchw + 1)) ||
            (rc = dgrow(ctx, &ctx->d_chg, &ctx->d_chg_cap, ctx->h_chg.size())))
            return rc;
        CK(cudaMemcpyAsync(ctx->d_chg, ctx->h_chg.data(), sizeof(unsigned long long) * ctx->h_chg.size(),
                           cudaMemcpyHostToDevice, ctx->stream));
    }
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(ctx->d_cstart, cs.data(), sizeof(long long) * cs.size(), cudaMemcpyHostToDevice, s));
    if (!sg.empty()) CK(cudaMemcpyAsync(ctx->d_cseg, sg.data(), sizeof(int) * sg.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_klist, kl.data(), sizeof(int) * kl.size(), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));     // (the host vectors change with the next batch)
    ctx->mc_dirty = false;
    return 0;
}

// The (member, sample) segments of an ANALYTIC batch. A member k > 0 whose columns differ from member 0's in a
// few sub-rings, with member 0's box and fixed-point exponent (with a flux normalisation: member 0's profile), is
// computed as member 0's fixed-point sums plus the deposits of those sub-rings' samples with its constants, minus
// the same samples with member 0's (exact: the sums are modulo 2^64, the deposits rounded symmetrically); every
// other member deposits all its samples.
static int an_segments(bbgpu_ctx *ctx) {
    const int nb = ctx->nb, nsub = ctx->nsub;
    const long long ns = ctx->ansamp;
    const std::vector<int> &sb = ctx->asbase_host;
    std::vector<long long> &cs = ctx->h_astart;
    std::vector<int> &sg = ctx->h_aseg, &mb = ctx->h_mbase;
    cs.clear();
    sg.clear();
    mb.assign(nb, -1);
    long long tot = 0;
    auto seg = [&](int k, int src, int ir, int sign, long long n) {
        if (n <= 0) return;
        cs.push_back(tot);
        sg.insert(sg.end(), {k, src, ir, sign});
        tot += n;
    };
    const bool can = ctx->share && nb > 1 && (int)sb.size() == nsub + 1 &&
                     (!ctx->prof_uploaded || (int)ctx->prof_of_host.size() == nb);
    const MemberDev &M0 = ctx->mem_host[0];
    int n2 = 0;
    for (int k = 0; k < nb; k++) {
        if (can && k > 0) {
            const MemberDev &M = ctx->mem_host[k];
            bool ok = M.blo0 == M0.blo0 && M.blo1 == M0.blo1 && M.bx == M0.bx && M.by == M0.by;
            if (ok) ok = ctx->prof_uploaded ? ctx->prof_of_host[k] == 0 : M.fix_exp == M0.fix_exp;
            if (ok) {
                const signed char *ru = ctx->h_reuse + (size_t)k * nsub;
                long long nch = 0;
                for (int ir = 0; ir < nsub; ir++)
                    if (!ru[ir]) nch += sb[ir + 1] - sb[ir];
                if (2 * nch < ns) {
                    for (int ir = 0; ir < nsub; ir++)
                        if (!ru[ir]) {
                            seg(k, k, ir, 1, sb[ir + 1] - sb[ir]);
                            seg(k, 0, ir, -1, sb[ir + 1] - sb[ir]);
                        }
                    mb[k] = 0;
                    n2++;
                    continue;
                }
            }
        }
        seg(k, k, -1, 1, ns);
    }
    cs.push_back(tot);
    ctx->an_nseg = (int)cs.size() - 1;
    ctx->an_ntot = tot;
    ctx->an_n2 = n2;
    int rc;
    if ((rc = dgrow(ctx, &ctx->d_astart, &ctx->d_astart_cap, cs.size())) ||
        (rc = dgrow(ctx, &ctx->d_aseg, &ctx->d_aseg_cap, sg.size() + 4)) ||
        (rc = dgrow(ctx, &ctx->d_mbase, &ctx->d_mbase_cap, (size_t)nb)))
        return rc;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(ctx->d_astart, cs.data(), sizeof(long long) * cs.size(), cudaMemcpyHostToDevice, s));
    if (!sg.empty()) CK(cudaMemcpyAsync(ctx->d_aseg, sg.data(), sizeof(int) * sg.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_mbase, mb.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));     // (the host vectors change with the next batch)
    ctx->an_dirty = false;
    return 0;
}

// The MC clouds' tile lists on stream s: each (member, cloud) pair binned to its pixel, the lists' offsets, the
// entries (their fixed-point fluxes left to k_entry_fix: they come from the flux normalisation, which may still
// be running), and, when members replay member 0's clouds, member 0's channel counts. None of it reads what the
// flux normalisation writes (the clouds' densities and fluxes, the members' exponents).
static int mc_lists(bbgpu_ctx *ctx, cudaStream_t s, bool tm) {
    const GridDev &g = ctx->g;
    const LayoutDev &L = ctx->cur->dev;
    CK(cudaMemsetAsync(ctx->d_tcount, 0, sizeof(int) * (size_t)(ctx->ntile_total * NOWN + 1), s));
    launch_mc_bin(s, g, L, ctx->d_sub, ctx->nsub, ctx->d_mem, ctx->d_cstart, ctx->d_cseg, ctx->mc_nseg,
                  ctx->mc_ntot, ctx->tx, ctx->ty, ctx->d_pix, ctx->d_tcount, ctx->d_err);
    CKL();
    if (tm) CK(cudaEventRecord(ctx->ev[5], s));
    launch_scan_tiles(s, ctx->d_tcount, ctx->d_toff, ctx->d_tcur, ctx->ntile_total * NOWN, ctx->d_scan);
    CKL();
    if (tm) CK(cudaEventRecord(ctx->ev[6], s));
    launch_mc_scatter(s, L, ctx->d_sub, ctx->nsub, ctx->d_mem, ctx->d_cstart, ctx->d_cseg, ctx->mc_nseg,
                      ctx->mc_ntot, ctx->tx, ctx->ty, ctx->d_pix, ctx->d_tcur, ctx->d_bucket, 1);
    CKL();
    if (ctx->mc_records) {
        const MemberDev &M0 = ctx->mem_host[0];
        launch_replay_records(s, g, L, ctx->d_sub, ctx->d_zig, ctx->d_bucket, ctx->d_toff, ctx->d_tcount,
                              (M0.tile_off + M0.ntx * M0.nty) * NOWN, ctx->tx * ctx->ty, ctx->d_rp_rec, ctx->d_rp_cnt,
                              ctx->d_rp_n, ctx->d_tmask, ctx->nchw, ctx->d_err);
        CKL();
    }
    return 0;
}

// The beam convolution and residual of the batch's models: on the tensor cores (ctx->conv_variant 1 or 2) when the
// kernel, the channels and the tile table qualify, else the float32 kernel. Sets npart_used and conv_used.
static bool conv_tc_ok(const bbgpu_ctx *ctx, int v, const TileSrc &ts) {
    return v && conv_tc_supported(v, ctx->ky, ctx->kx, ctx->g.nz) && (ctx->mstride % 4) == 0 &&
           (!ts.tsrc || ts.shx >= 3) && !ts.kout;
}

static int conv_run(bbgpu_ctx *ctx, cudaStream_t s, int v, bool conv, bool do_resid, TileSrc ts);

// The variant of the batch convolution: the option's, or (option -1) the autotuner's for this kernel and these
// channels. The autotuner runs the batch's convolution with each candidate (float32; tf32x3 where the kernel and the
// channels qualify) on the batch in hand, twice each, times the second run with events, and keeps the faster for the
// context's lifetime: every later batch with the same kernel shape and channels gets the same arithmetic.
static int conv_variant_of(bbgpu_ctx *ctx, cudaStream_t s, bool conv, bool do_resid, TileSrc ts, int &v) {
    v = ctx->conv_variant;
    if (v >= 0 || !conv) {
        v = v < 0 ? 0 : v;
        return 0;
    }
    // one choice per kernel shape and channel count, made on the first batch: a parameter vector then gets the
    // same bits in a batch of any size or composition (a sampler's points, a gradient's stencil)
    for (auto &t : ctx->tuned)
        if (t[0] == ctx->ky && t[1] == ctx->kx && t[2] == ctx->g.nz) {
            v = t[3];
            return 0;
        }
    int best = 0;
    float bms = 1e30f;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = 0;
    for (int cand : {0, 2}) {
        if (cand && !conv_tc_ok(ctx, cand, ts)) continue;
        float ms = 0.f;
        for (int rep = 0; rep < 2 && !rc; rep++) {
            cudaEventRecord(e0, s);
            rc = conv_run(ctx, s, cand, conv, do_resid, ts);
            cudaEventRecord(e1, s);
        }
        if (rc) break;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
            rc = fail(ctx, BBGPU_ERR_CUDA, "convolution autotuner: event timing failed");
            break;
        }
        ctx->tune_ms[cand] = ms;
        if (ms < bms) {
            bms = ms;
            best = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    ctx->tuned.push_back({ctx->ky, ctx->kx, ctx->g.nz, best});
    v = best;
    return 0;
}

// The beam convolution and residual of the batch's models with the variant of conv_variant_of. Sets npart_used
// and conv_used.
static int conv_batch(bbgpu_ctx *ctx, cudaStream_t s, bool conv, bool do_resid, TileSrc ts) {
    int v = 0;
    int rc = conv_variant_of(ctx, s, conv, do_resid, ts, v);
    if (rc) return rc;
    return conv_run(ctx, s, v, conv, do_resid, ts);
}

// the convolution with variant v: on the tensor cores (1 bf16x3, 2 tf32x3) when the kernel, the channels and the tile
// table qualify, else the float32 kernel
static int conv_run(bbgpu_ctx *ctx, cudaStream_t s, int v, bool conv, bool do_resid, TileSrc ts) {
    const GridDev &g = ctx->g;
    float *smoothed = ctx->keep_smoothed ? ctx->d_smooth : nullptr;
    const bool tc = conv && conv_tc_ok(ctx, v, ts);
    if (!tc) {
        launch_conv_resid(s, g, ctx->d_mem, ctx->mem_host.data(), ctx->nb, ctx->d_model, ctx->mstride, g.nz,
                          ctx->d_taps, ctx->ky, ctx->kx, ctx->kxw, smoothed, conv ? 1 : 0, do_resid ? 1 : 0,
                          ctx->d_partial, ts);
        CKL();
        ctx->npart_used = conv_resid_npart(ctx->mem_host.data(), ctx->nb, g.nz);
        ctx->conv_used = 0;
        return 0;
    }
    int rc;
    if (ctx->bimg_variant != v) {
        std::vector<uint8_t> img;
        conv_tc_image(v, ctx->h_kernel.data(), ctx->ky, ctx->kx, img);
        if ((rc = dgrow(ctx, (uint8_t **)&ctx->d_bimg, &ctx->d_bimg_cap, img.size()))) return rc;
        CK(cudaMemcpyAsync(ctx->d_bimg, img.data(), img.size(), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        ctx->bimg_variant = v;
    }
    // the members' TMA descriptors, rebuilt when the model buffer or a box changes
    std::vector<long long> key{(long long)(uintptr_t)ctx->d_model, ctx->mstride, (long long)g.nz, (long long)ctx->nb};
    for (int k = 0; k < ctx->nb; k++) {
        key.push_back(ctx->mem_host[k].bx);
        key.push_back(ctx->mem_host[k].by);
        key.push_back((long long)(uintptr_t)ctx->mem_host[k].deff);
    }
    if (key != ctx->tmaps_key) {
        if (!conv_tc_maps(ctx->mem_host.data(), ctx->nb, ctx->d_model, ctx->mstride, g.nz, g.nx, g.ny, ctx->h_tmaps))
            return fail(ctx, BBGPU_ERR_CUDA, "cuTensorMapEncodeTiled refused a model descriptor");
        if ((rc = dgrow(ctx, &ctx->d_tmaps, &ctx->d_tmaps_cap, 2 * (size_t)ctx->nb))) return rc;
        CK(cudaMemcpyAsync(ctx->d_tmaps, ctx->h_tmaps.data(), sizeof(CUtensorMap) * 2 * ctx->nb,
                           cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        ctx->tmaps_key = key;
    }
    const int npart = conv_tc_npart(ctx->mem_host.data(), ctx->nb, g.nz);
    if (!ctx->d_tcq) CK(cudaMalloc(&ctx->d_tcq, sizeof(int)));
    CK(cudaMemsetAsync(ctx->d_partial, 0, sizeof(double) * 2 * (size_t)ctx->nb * npart, s));
    launch_conv_tc(s, v, g, ctx->d_mem, ctx->mem_host.data(), ctx->nb, ctx->d_tmaps, ctx->d_bimg, ctx->mstride, g.nz,
                   ctx->ky, ctx->kx, smoothed, 1, do_resid ? 1 : 0, ctx->d_partial, npart, ts, ctx->d_err,
                   ctx->d_tcq);
    CKL();
    ctx->npart_used = npart;
    ctx->conv_used = v;
    return 0;
}

static int batch_run(bbgpu_ctx *ctx, bool do_resid) {
    if (!ctx->uploaded) return fail(ctx, BBGPU_ERR_STATE, "run before upload");
    const GridDev &g = ctx->g;
    cudaStream_t s = ctx->stream;
    const bool tm = ctx->timing;
    const bool mc = ctx->galmodtype != BBGPU_ANALYTIC;
    if (mc && ctx->mc_dirty) {
        int rc = mc_segments(ctx);
        if (rc) return rc;
    }
    // with a flux normalisation (and the stage timers off), the MC lists are built on the second stream while
    // it runs
    const bool side = mc && ctx->prof_uploaded && !tm;
    if (tm) CK(cudaEventRecord(ctx->ev[0], s));
    if (side) {
        CK(cudaEventRecord(ctx->ev_fork, s));
        CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
        int rc = mc_lists(ctx, ctx->side, false);
        cudaError_t e = cudaEventRecord(ctx->ev_join, ctx->side);
        if (rc) return rc;
        if (e != cudaSuccess) return fail(ctx, BBGPU_ERR_CUDA, "cudaEventRecord: %s", cudaGetErrorString(e));
    }
    if (ctx->prof_uploaded) {
        int rc = profile_run(ctx, tm);
        if (side) cudaStreamWaitEvent(s, ctx->ev_join, 0);
        if (rc) return rc;
    } else if (tm) {
        for (int i = 1; i <= 4; i++) CK(cudaEventRecord(ctx->ev[i], s));
    }
    if (ctx->galmodtype == BBGPU_ANALYTIC) {
        if (tm)
            for (int i = 5; i <= 10; i++) CK(cudaEventRecord(ctx->ev[i], s));
        if (ctx->an_dirty) {
            int rc = an_segments(ctx);
            if (rc) return rc;
        }
        CK(cudaMemsetAsync(ctx->d_model_fx, 0, sizeof(long long) * (size_t)ctx->nb * ctx->mstride, s));
        launch_an_model_fast(s, g, ctx->d_asub, ctx->nsub, ctx->d_asbase, ctx->d_assub, ctx->d_acs, ctx->d_acsf,
                             (const float *)ctx->d_acsff, ctx->d_astart, ctx->d_aseg, ctx->an_nseg, ctx->an_ntot,
                             ctx->d_azq, ctx->d_azqf, ctx->d_awqf, (const float *)ctx->d_vef, ctx->d_cd2if,
                             ctx->d_ptabf, ctx->d_mem, ctx->d_model_fx, ctx->mstride, ctx->an_thin, ctx->an_thick);
        CKL();
        if (ctx->an_exact) {
            launch_an_model(s, g, ctx->d_asub, ctx->nsub, ctx->d_asbase, ctx->d_assub, ctx->d_acs, ctx->d_astart,
                            ctx->d_aseg, ctx->an_nseg, ctx->an_ntot, ctx->d_azq, ctx->d_awq, ctx->d_vedges,
                            ctx->d_cd2i, ctx->d_ptab, ctx->d_mem, ctx->d_model_fx, ctx->mstride, 1);
            CKL();
        }
        launch_fix_to_model(s, ctx->d_model_fx, ctx->d_mem, ctx->nb, ctx->mstride, g.nz, ctx->d_model,
                            ctx->want64 ? ctx->d_model64 : nullptr, ctx->an_n2 ? ctx->d_mbase : nullptr);
        CKL();
        if (tm) CK(cudaEventRecord(ctx->ev[11], s));
    } else {
        const LayoutDev &L = ctx->cur->dev;
        if (!side) {
            int rc = mc_lists(ctx, s, tm);
            if (rc) return rc;
        }
        launch_entry_fix(s, ctx->d_sub, ctx->d_toff, ctx->d_tcount, ctx->ntile_total * NOWN, ctx->mc_ntot,
                         ctx->d_bucket);
        CKL();
        if (tm) CK(cudaEventRecord(ctx->ev[7], s));
        if (ctx->mc_n2 || ctx->mc_n3) {
            launch_mc_deposit(s, g, L, ctx->d_sub, ctx->nsub, ctx->d_mem, ctx->mem_host.data(), ctx->nb, ctx->tx,
                              ctx->ty, ctx->d_toff, ctx->d_tcount, ctx->d_bucket, ctx->d_zig, ctx->d_cd2if,
                              ctx->d_cd2i, ctx->d_model, ctx->mstride, nullptr, ctx->d_err, ctx->lean, ctx->d_klist,
                              ctx->mc_n1, 0, ctx->mc_n2 ? ctx->d_base64 : nullptr, ctx->mc_n2 ? ctx->d_tsrc : nullptr);
            CKL();
            if (tm) CK(cudaEventRecord(ctx->ev[8], s));
            const Replay rp = ctx->mc_records ? Replay{(const int2 *)ctx->d_rp_rec, ctx->d_rp_cnt, ctx->d_rp_n,
                                                       ctx->d_chg, ctx->nchw, ctx->d_tmask}
                                              : Replay{nullptr, nullptr, nullptr, nullptr, 0, nullptr};
            if (ctx->mc_n2) {
                launch_mc_deposit(s, g, L, ctx->d_sub, ctx->nsub, ctx->d_mem, ctx->mem_host.data(), ctx->nb,
                                  ctx->tx, ctx->ty, ctx->d_toff, ctx->d_tcount, ctx->d_bucket, ctx->d_zig,
                                  ctx->d_cd2if, ctx->d_cd2i, ctx->d_model, ctx->mstride, nullptr, ctx->d_err,
                                  ctx->lean, ctx->d_klist + ctx->mc_n1, ctx->mc_n2, 1, ctx->d_base64, ctx->d_tsrc, rp);
                CKL();
            }
            if (tm) CK(cudaEventRecord(ctx->ev[9], s));
            if (ctx->mc_n3) {
                launch_mc_deposit(s, g, L, ctx->d_sub, ctx->nsub, ctx->d_mem, ctx->mem_host.data(), ctx->nb,
                                  ctx->tx, ctx->ty, ctx->d_toff, ctx->d_tcount, ctx->d_bucket, ctx->d_zig,
                                  ctx->d_cd2if, ctx->d_cd2i, ctx->d_model, ctx->mstride, nullptr, ctx->d_err,
                                  ctx->lean, ctx->d_klist + ctx->mc_n1 + ctx->mc_n2, ctx->mc_n3, 2, nullptr,
                                  ctx->mc_n2 ? ctx->d_tsrc : nullptr, rp);
                CKL();
            }
            if (tm) CK(cudaEventRecord(ctx->ev[10], s));
        } else {
            launch_mc_deposit(s, g, L, ctx->d_sub, ctx->nsub, ctx->d_mem, ctx->mem_host.data(), ctx->nb, ctx->tx,
                              ctx->ty, ctx->d_toff, ctx->d_tcount, ctx->d_bucket, ctx->d_zig, ctx->d_cd2if,
                              ctx->d_cd2i, ctx->d_model, ctx->mstride, ctx->want64 ? ctx->d_model64 : nullptr,
                              ctx->d_err, ctx->lean);
            CKL();
            if (tm) {
                CK(cudaEventRecord(ctx->ev[8], s));
                CK(cudaEventRecord(ctx->ev[9], s));
                CK(cudaEventRecord(ctx->ev[10], s));
            }
        }
        if (tm) CK(cudaEventRecord(ctx->ev[11], s));
    }
    const bool conv = ctx->kernel_set;
    if (do_resid || ctx->keep_smoothed) {
        TileSrc ts{nullptr, 0, 0, nullptr, 0};
        if (ctx->galmodtype == BBGPU_MC && ctx->mc_n2)
            ts = TileSrc{ctx->d_tsrc, ilog2(ctx->tx), ilog2(ctx->ty), nullptr, 0};
        int rc = conv_batch(ctx, s, conv, do_resid, ts);
        if (rc) return rc;
    }
    if (tm) CK(cudaEventRecord(ctx->ev[12], s));
    if (do_resid) {
        launch_reduce_partials(s, ctx->d_partial, ctx->npart_used, ctx->nb, ctx->d_out2);
        CKL();
    }
    if (tm) {
        CK(cudaEventRecord(ctx->ev[13], s));
        CK(cudaEventSynchronize(ctx->ev[13]));
        for (int i = 0; i < NTIMER; i++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev[i], ctx->ev[i + 1]);
            ctx->times[i] = ms;
        }
    }
    ctx->ran = true;
    return 0;
}

static int check_err(bbgpu_ctx *ctx) {
    CK(cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (*ctx->h_err) {
        int e = *ctx->h_err;
        CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
        if (e & ERR_TC)
            return fail(ctx, BBGPU_ERR_KERNEL,
                        "the tensor-core convolution gave up waiting for one of its stages (bounded wait expired)");
        if (e & ERR_SHARE)
            return fail(ctx, BBGPU_ERR_KERNEL,
                        "a member computed as a difference from member 0's model has another fixed-point exponent "
                        "(disable option 3 for this batch)");
        if (e & ERR_PROFILE_LAYOUT)
            return fail(ctx, BBGPU_ERR_KERNEL,
                        "the deconvolved density profile changed the MC cloud layout of a member (a ring density "
                        "at zero, or above the 10-clouds-per-pixel floor): evaluate that member with its densities");
        return fail(ctx, BBGPU_ERR_KERNEL, "kernel error flag 0x%x (cloud layout inconsistent with the sub-rings)", e);
    }
    return 0;
}

extern "C" int bbgpu_eval_upload(bbgpu_ctx *ctx, int galmodtype, int nb, int nsub, const double *sr,
                                 const int64_t *nv, const bbgpu_eval_desc *descs) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    ctx->want64 = false;
    return batch_prepare(ctx, galmodtype, nb, nsub, sr, nv, descs, true);
}

// A batch run through a CUDA graph (option 5, on by default): the run after one that completed with the same
// state (nothing uploaded, set or reallocated since: its host-side set-up is done) is captured, both streams with
// their fork and join, and replayed by every later run of that state; the stage timers run without a graph. A
// capture that fails leaves the run to the ordinary path.
static int graph_run(bbgpu_ctx *ctx) {
    if (ctx->gexec && ctx->graph_gen == ctx->gen) {
        CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
        ctx->launches += ctx->graph_launches;
        ctx->graph_replays++;
        ctx->ran = true;
        return 0;
    }
    if (ctx->gexec) {
        cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    const long long l0 = ctx->launches, g0 = ctx->gen;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    const int rc = batch_run(ctx, true);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    const bool ok = !rc && e == cudaSuccess && graph && ctx->gen == g0 &&
                    cudaGraphInstantiate(&ctx->gexec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
        cudaGetLastError();
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
        ctx->launches = l0;
        return -1;
    }
    ctx->graph_gen = ctx->gen;
    ctx->graph_launches = ctx->launches - l0;
    CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
    ctx->ran = true;
    return 0;
}

extern "C" int bbgpu_eval_run(bbgpu_ctx *ctx) {
    if (!ctx) return BBGPU_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    if (ctx->use_graphs && !ctx->timing && ctx->uploaded && ctx->gen_ran == ctx->gen &&
        ctx->graph_fail_gen != ctx->gen) {
        const int rc = graph_run(ctx);
        if (rc >= 0) return rc;
        ctx->graph_fail_gen = ctx->gen;   // (the capture failed: this state runs without a graph)
    }
    const long long g0 = ctx->gen;
    const int rc = batch_run(ctx, true);
    if (!rc && ctx->gen == g0) ctx->gen_ran = g0;
    return rc;
}

extern "C" int bbgpu_graph_stats(const bbgpu_ctx *ctx, int64_t *replays, int64_t *kernels) {
    if (!ctx) return BBGPU_ERR_ARG;
    if (replays) *replays = ctx->graph_replays;
    if (kernels) *kernels = ctx->gexec && ctx->graph_gen == ctx->gen ? ctx->graph_launches : 0;
    return BBGPU_OK;
}

extern "C" int bbgpu_eval_download(bbgpu_ctx *ctx, double *ss, double *lg) {
    if (!ctx || !ss) return BBGPU_ERR_ARG;
    if (!ctx->ran) return fail(ctx, BBGPU_ERR_STATE, "download before run");
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(ctx->h_out2, ctx->d_out2, sizeof(double) * 2 * ctx->nb, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->d2h = (long long)(sizeof(double) * 2 * ctx->nb + sizeof(int));
    int rc = check_err(ctx);
    if (rc) return rc;
    for (int k = 0; k < ctx->nb; k++) {
        ss[k] = ctx->h_out2[2 * k];
        if (lg) lg[k] = ctx->h_out2[2 * k + 1];
    }
    return BBGPU_OK;
}

extern "C" int bbgpu_eval_batch(bbgpu_ctx *ctx, int galmodtype, int nb, int nsub, const double *sr, const int64_t *nv,
                                const bbgpu_eval_desc *descs, double *ss, double *lg) {
    if (ctx) ctx->gen++;
    int rc = bbgpu_eval_upload(ctx, galmodtype, nb, nsub, sr, nv, descs);
    if (rc) return rc;
    rc = bbgpu_eval_run(ctx);
    if (rc) return rc;
    return bbgpu_eval_download(ctx, ss, lg);
}

extern "C" int bbgpu_eval_model(bbgpu_ctx *ctx, int k, int smoothed, float *out, int by, int bx, int nz) {
    if (!ctx || !out) return BBGPU_ERR_ARG;
    if (!ctx->ran || k < 0 || k >= ctx->nb) return fail(ctx, BBGPU_ERR_STATE, "eval_model: no such member");
    const MemberDev &M = ctx->mem_host[k];
    if (by != M.by || bx != M.bx || nz != ctx->g.nz) return fail(ctx, BBGPU_ERR_ARG, "eval_model: shape mismatch");
    if (smoothed && !ctx->keep_smoothed) return fail(ctx, BBGPU_ERR_STATE, "eval_model: smoothed models not kept");
    const float *src = (smoothed ? ctx->d_smooth : ctx->d_model) + (size_t)k * ctx->mstride;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(out, src, sizeof(float) * (size_t)by * bx * nz, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!smoothed && ctx->galmodtype == BBGPU_MC && ctx->mc_n2 && k < (int)ctx->mc_isdelta.size() &&
        ctx->mc_isdelta[k]) {
        // the tiles the member shares with member 0 hold member 0's values (the same box)
        const int nt = M.ntx * M.nty;
        std::vector<int> ts(nt);
        std::vector<float> m0((size_t)by * bx * nz);
        CK(cudaMemcpy(ts.data(), ctx->d_tsrc + M.tile_off, sizeof(int) * nt, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(m0.data(), ctx->d_model, sizeof(float) * m0.size(), cudaMemcpyDeviceToHost));
        for (int y = 0; y < by; y++)
            for (int x = 0; x < bx; x++)
                if (ts[(y / ctx->ty) * M.ntx + x / ctx->tx] == 0)
                    memcpy(out + ((size_t)y * bx + x) * nz, m0.data() + ((size_t)y * bx + x) * nz, sizeof(float) * nz);
    }
    return BBGPU_OK;
}

// ------------------------------------------------------------------------------------------- reference kernels
extern "C" int bbgpu_galmod_mc(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int ring_lo, int ring_hi,
                               uint64_t seed, const int64_t *nv, int blo0, int blo1, int bhi0, int bhi1) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!out || !sr || !nv || ring_lo < 0 || ring_hi > nsub || ring_lo > ring_hi)
        return fail(ctx, BBGPU_ERR_ARG, "galmod_mc: invalid arguments");
    CK(cudaSetDevice(ctx->device));
    // sub-rings [ring_lo, ring_hi) with a stream seeded by seed: the table restricted to them
    int ns = ring_hi - ring_lo;
    std::vector<double> s2((size_t)BBGPU_NSR * (ns ? ns : 1));
    std::vector<int64_t> nv2(ns ? ns : 1);
    for (int r = 0; r < BBGPU_NSR; r++)
        for (int i = 0; i < ns; i++) s2[(size_t)r * ns + i] = sr[(size_t)r * nsub + ring_lo + i];
    for (int i = 0; i < ns; i++) nv2[i] = nv[ring_lo + i];
    int by = bhi1 - blo1, bx = bhi0 - blo0;
    if (ns == 0 || by <= 0 || bx <= 0) return BBGPU_OK;
    bbgpu_eval_desc d{};
    d.blo0 = blo0; d.blo1 = blo1; d.bhi0 = bhi0; d.bhi1 = bhi1; d.seed = seed;
    ctx->want64 = true;
    int rc = batch_prepare(ctx, BBGPU_MC, 1, ns, s2.data(), nv2.data(), &d, false);
    if (rc) return rc;
    rc = batch_run(ctx, false);
    ctx->want64 = false;
    if (rc) return rc;
    rc = check_err(ctx);
    if (rc) return rc;
    size_t n = (size_t)by * bx * ctx->g.nz;
    std::vector<double> tmp(n);
    CK(cudaMemcpy(tmp.data(), ctx->d_model64, n * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) out[i] += tmp[i];
    ctx->uploaded = ctx->ran = false;
    return BBGPU_OK;
}

extern "C" int bbgpu_convolve(bbgpu_ctx *ctx, const double *in, double *out, int nz, int ny, int nx, double scale,
                              int threshold) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!in || !out || nz < 1 || ny < 1 || nx < 1) return fail(ctx, BBGPU_ERR_ARG, "convolve: invalid arguments");
    if (!ctx->kernel_set) return fail(ctx, BBGPU_ERR_STATE, "convolve before set_kernel");
    CK(cudaSetDevice(ctx->device));
    size_t n = (size_t)nz * ny * nx;
    double *d64 = nullptr;
    float *a = nullptr, *b = nullptr;
    MemberDev *dm = nullptr;
    int rc = 0;
    GridDev g = ctx->g;
    g.scalefactor = threshold ? scale : 1.0;
    MemberDev M{};
    M.blo0 = 0; M.blo1 = 0; M.bhi0 = nx; M.bhi1 = ny; M.bx = nx; M.by = ny;
    cudaStream_t s = ctx->stream;
    if (cudaMalloc(&d64, n * sizeof(double)) != cudaSuccess || cudaMalloc(&a, n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&b, n * sizeof(float)) != cudaSuccess || cudaMalloc(&dm, sizeof M) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(ctx, BBGPU_ERR_NOMEM, "convolve: allocation failed");
    }
    int npart = conv_resid_npart(&M, 1, nz);
    double *dp = nullptr;
    if (!rc && cudaMalloc(&dp, 2 * sizeof(double) * (npart ? npart : 1)) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(ctx, BBGPU_ERR_NOMEM, "convolve: allocation failed");
    }
    if (!rc) {
        cudaMemcpyAsync(d64, in, n * sizeof(double), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dm, &M, sizeof M, cudaMemcpyHostToDevice, s);
        launch_zyx64_to_yxz32(s, d64, a, nz, ny, nx);
        launch_conv_resid(s, g, dm, &M, 1, a, (long long)n, nz, ctx->d_taps, ctx->ky, ctx->kx, ctx->kxw, b,
                          threshold ? 1 : 2, 0, dp);
        launch_yxz32_to_zyx64(s, b, d64, nz, ny, nx);
        ctx->launches += 3;
        cudaMemcpyAsync(out, d64, n * sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(ctx, BBGPU_ERR_CUDA, "convolve: %s", cudaGetErrorString(e));
    }
    cudaFree(d64); cudaFree(a); cudaFree(b); cudaFree(dm); cudaFree(dp);
    return rc;
}

static int sumsq_common(bbgpu_ctx *ctx, const double *model, const float *data, const uint8_t *mask, int maskmode,
                        const uint8_t *region, int nz, int ny, int nx, double sigma2, double eps2, double *out2) {
    if (!ctx) return BBGPU_ERR_ARG;
    if (!model || !data || !out2 || nz < 0 || ny < 0 || nx < 0) return fail(ctx, BBGPU_ERR_ARG, "residuals: invalid arguments");
    if (maskmode != 0 && !mask) return fail(ctx, BBGPU_ERR_ARG, "residuals: maskmode %d without a mask", maskmode);
    CK(cudaSetDevice(ctx->device));
    size_t n = (size_t)nz * ny * nx;
    out2[0] = out2[1] = 0.0;
    if (n == 0) return BBGPU_OK;
    double *dm = nullptr, *dp = nullptr;
    float *dd = nullptr;
    uint8_t *dk = nullptr, *dr = nullptr;
    const int maxb = 1024;
    int rc = 0;
    if (cudaMalloc(&dm, n * 8) != cudaSuccess || cudaMalloc(&dd, n * 4) != cudaSuccess ||
        cudaMalloc(&dp, 2 * 8 * maxb) != cudaSuccess || (mask && cudaMalloc(&dk, n) != cudaSuccess) ||
        (region && cudaMalloc(&dr, (size_t)ny * nx) != cudaSuccess)) {
        cudaGetLastError();
        rc = fail(ctx, BBGPU_ERR_NOMEM, "residuals: allocation failed");
    }
    if (!rc) {
        cudaStream_t s = ctx->stream;
        cudaMemcpyAsync(dm, model, n * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dd, data, n * 4, cudaMemcpyHostToDevice, s);
        if (mask) cudaMemcpyAsync(dk, mask, n, cudaMemcpyHostToDevice, s);
        if (region) cudaMemcpyAsync(dr, region, (size_t)ny * nx, cudaMemcpyHostToDevice, s);
        int nbk = launch_sumsq64(s, dm, dd, dk, maskmode, dr, nz, ny, nx, sigma2, eps2, dp, maxb);
        ctx->launches++;
        std::vector<double> hp(2 * (size_t)nbk);
        cudaMemcpyAsync(hp.data(), dp, 2 * 8 * (size_t)nbk, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(ctx, BBGPU_ERR_CUDA, "residuals: %s", cudaGetErrorString(e));
        for (int i = 0; i < nbk; i++) {
            out2[0] += hp[2 * i];
            out2[1] += hp[2 * i + 1];
        }
    }
    cudaFree(dm); cudaFree(dd); cudaFree(dp); cudaFree(dk); cudaFree(dr);
    return rc;
}

extern "C" int bbgpu_sumsq_residuals(bbgpu_ctx *ctx, const double *model, const float *data, const uint8_t *mask,
                                     int maskmode, const uint8_t *region, int nz, int ny, int nx, double *out) {
    if (ctx) ctx->gen++;
    double o2[2];
    int rc = sumsq_common(ctx, model, data, mask, maskmode, region, nz, ny, nx, 1.0, 0.0, o2);
    if (!rc && out) *out = o2[0];
    return rc;
}

extern "C" int bbgpu_residuals_fracerr(bbgpu_ctx *ctx, const double *model, const float *data, const uint8_t *mask,
                                       int maskmode, const uint8_t *region, int nz, int ny, int nx, double sigma2,
                                       double eps2, double *out2) {
    if (ctx) ctx->gen++;
    if (ctx && !(sigma2 > 0)) return fail(ctx, BBGPU_ERR_ARG, "residuals_fracerr: sigma2 must be > 0");
    if (ctx && !(eps2 > 0)) return fail(ctx, BBGPU_ERR_ARG, "residuals_fracerr: eps2 must be > 0");
    return sumsq_common(ctx, model, data, mask, maskmode, region, nz, ny, nx, sigma2, eps2, out2);
}

// A scoped set of device buffers freed at the end of a stand-alone entry point.
// Scratch buffers of a stand-alone call: the i-th buffer of call site `tag` is kept in the context and reused by
// the next call of that site (grown when too small), so that a call allocates nothing once warm (a cudaFree would
// also wait for the whole device). The calls of a context run in order on its stream, so reuse is safe.
struct DevBufs {
    bbgpu_ctx *ctx;
    int tag;
    size_t i = 0;
    DevBufs(bbgpu_ctx *c, int t) : ctx(c), tag(t) {}
    template <class T>
    bool get(T **out, size_t n) {
        std::vector<PoolBuf> &v = ctx->pool[tag];
        if (i == v.size()) v.push_back(PoolBuf{});
        PoolBuf &b = v[i++];
        const size_t need = n ? n : 1;
        if (b.cap < need) {
            if (b.p) cudaFree(b.p);
            b.p = nullptr;
            b.cap = 0;
            const size_t want = need + need / 4;
            if (cudaMalloc(&b.p, want) != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            b.cap = want;
        }
        *out = (T *)b.p;
        return true;
    }
};

// The azimuthal samples and sub-ring constants of one ANALYTIC call, on the device.
struct AnDev {
    AnSub *subs = nullptr;
    int *sbase = nullptr, *ssub = nullptr;
    double *cs = nullptr, *zq = nullptr, *wq = nullptr;
    long long nsamp = 0;
};

static int an_upload(bbgpu_ctx *ctx, DevBufs &B, const std::vector<AnSub> &subs, const double *R0, int nsub,
                     const std::vector<double> &zq, const std::vector<double> &wq, AnDev &D) {
    std::vector<int> sbase, ssub;
    std::vector<double> cs;
    bbh_an_samples(R0, nsub, &ctx->g, sbase, ssub, cs);
    D.nsamp = sbase[nsub];
    if (!B.get(&D.subs, sizeof(AnSub) * (subs.size() ? subs.size() : 1)) || !B.get(&D.sbase, sizeof(int) * sbase.size()) ||
        !B.get(&D.ssub, sizeof(int) * ssub.size()) || !B.get(&D.cs, sizeof(double) * cs.size()) ||
        !B.get(&D.zq, sizeof(double) * (zq.size() ? zq.size() : 1)) ||
        !B.get(&D.wq, sizeof(double) * (wq.size() ? wq.size() : 1)))
        return fail(ctx, BBGPU_ERR_NOMEM, "analytic: allocation failed");
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(D.subs, subs.data(), sizeof(AnSub) * subs.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(D.sbase, sbase.data(), sizeof(int) * sbase.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(D.ssub, ssub.data(), sizeof(int) * ssub.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(D.cs, cs.data(), sizeof(double) * cs.size(), cudaMemcpyHostToDevice, s));
    if (zq.size()) {
        CK(cudaMemcpyAsync(D.zq, zq.data(), sizeof(double) * zq.size(), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.wq, wq.data(), sizeof(double) * wq.size(), cudaMemcpyHostToDevice, s));
    }
    // (the host vectors are freed on return: the copies complete first)
    CK(cudaStreamSynchronize(s));
    return 0;
}

// The clouds of one or more chunks of shells (each parsed from its own stream) placed and deposited in one pass:
// the fixed-point sums are exact, so the chunks' deposits add in any order; out += the sum of the chunks.
static int wind_mc_run(bbgpu_ctx *ctx, double *out, std::vector<WindClouds> &chunks, int blo0, int blo1, int bhi0,
                       int bhi1) {
    const int by = bhi1 - blo1, bx = bhi0 - blo0;
    const size_t n = (size_t)by * bx * ctx->g.nz;
    // the chunks' arrays go to the device at their offsets (shell indices and deviate offsets shifted)
    size_t nsh = 0, ncl = 0, nhz = 0, nsl = 0;
    double total = 0.;
    for (WindClouds &c : chunks) {
        for (int &v : c.shell) v += (int)nsh;
        for (long long &v : c.nbase) v += (long long)nhz;
        for (long long &v : c.sbase) v += (long long)nsl;
        nsh += c.shells.size();
        ncl += c.shell.size();
        nhz += c.hz.size();
        nsl += c.slow.size();
        total += c.total;
    }
    if (ncl == 0) return BBGPU_OK;
    // fixed-point unit: 2^E above the total flux of the deposits
    double rs = 0., cmax = 0.;
    for (int l = 0; l < ctx->g.nlines; l++) rs += fabs(ctx->g.relint[l]);
    for (double c : ctx->h_cd2i) cmax = std::max(cmax, fabs(c));
    const double bound = total * rs * cmax;
    if (!(bound > 0) || !std::isfinite(bound)) return BBGPU_OK;
    int E = 0;
    frexp(bound * 1.0000001, &E);
    const double scale = ldexp(1.0, 62 - E), unit = ldexp(1.0, E - 62);
    WindShell *d_sh = nullptr;
    int *d_shell = nullptr, *d_hz = nullptr;
    double *d_geo = nullptr, *d_slow = nullptr;
    long long *d_nb = nullptr, *d_sb = nullptr;
    unsigned long long *d_acc = nullptr;
    auto release = [&]() {
        cudaFree(d_sh); cudaFree(d_shell); cudaFree(d_hz); cudaFree(d_geo); cudaFree(d_slow); cudaFree(d_nb);
        cudaFree(d_sb); cudaFree(d_acc);
    };
    bool ok = cudaMalloc(&d_sh, sizeof(WindShell) * nsh) == cudaSuccess &&
              cudaMalloc(&d_shell, sizeof(int) * ncl) == cudaSuccess &&
              cudaMalloc(&d_geo, sizeof(double) * 5 * ncl) == cudaSuccess &&
              cudaMalloc(&d_hz, sizeof(int) * std::max<size_t>(nhz, 1)) == cudaSuccess &&
              cudaMalloc(&d_slow, sizeof(double) * std::max<size_t>(nsl, 1)) == cudaSuccess &&
              cudaMalloc(&d_nb, sizeof(long long) * ncl) == cudaSuccess &&
              cudaMalloc(&d_sb, sizeof(long long) * ncl) == cudaSuccess &&
              cudaMalloc(&d_acc, sizeof(unsigned long long) * n) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        release();
        return fail(ctx, BBGPU_ERR_NOMEM, "galmod_wind: device allocation failed");
    }
    cudaStream_t s = ctx->stream;
    ok = cudaMemsetAsync(d_acc, 0, sizeof(unsigned long long) * n, s) == cudaSuccess;
    size_t o_sh = 0, o_cl = 0, o_hz = 0, o_sl = 0;
    for (const WindClouds &c : chunks) {
        auto up = [&](void *dst, const void *src, size_t bytes) {
            return !bytes || cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
        };
        ok = ok && up(d_sh + o_sh, c.shells.data(), sizeof(WindShell) * c.shells.size()) &&
             up(d_shell + o_cl, c.shell.data(), sizeof(int) * c.shell.size()) &&
             up(d_geo + 5 * o_cl, c.geo.data(), sizeof(double) * c.geo.size()) &&
             up(d_nb + o_cl, c.nbase.data(), sizeof(long long) * c.nbase.size()) &&
             up(d_sb + o_cl, c.sbase.data(), sizeof(long long) * c.sbase.size()) &&
             up(d_hz + o_hz, c.hz.data(), sizeof(int) * c.hz.size()) &&
             up(d_slow + o_sl, c.slow.data(), sizeof(double) * c.slow.size());
        o_sh += c.shells.size();
        o_cl += c.shell.size();
        o_hz += c.hz.size();
        o_sl += c.slow.size();
    }
    if (ok) {
        launch_wind_mc(s, d_sh, d_shell, d_geo, d_nb, d_sb, d_hz, d_slow, ctx->d_zig, (long long)ncl, ctx->g,
                       ctx->d_cd2i, blo0, blo1, bhi0, bhi1, scale, d_acc);
        ctx->launches++;
        ok = cudaGetLastError() == cudaSuccess;
    }
    std::vector<unsigned long long> acc;
    if (ok) {
        acc.resize(n);
        ok = cudaMemcpyAsync(acc.data(), d_acc, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, s) ==
                 cudaSuccess &&
             cudaStreamSynchronize(s) == cudaSuccess;
    }
    release();
    if (!ok) return fail(ctx, BBGPU_ERR_CUDA, "galmod_wind: CUDA failure");
    for (size_t i = 0; i < n; i++)
        if (acc[i]) out[i] += (double)(long long)acc[i] * unit;
    return BBGPU_OK;
}

static int wind_args(bbgpu_ctx *ctx, const double *out, const double *sr, const int64_t *nv, double sep) {
    if (!out || !sr || !nv || !(sep > 0)) return fail(ctx, BBGPU_ERR_ARG, "galmod_wind: invalid arguments");
    if (!ctx->grid_set) return fail(ctx, BBGPU_ERR_STATE, "galmod_wind: no grid (bbgpu_set_grid)");
    return BBGPU_OK;
}

extern "C" int bbgpu_galmod_wind(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int ring_lo, int ring_hi,
                                 uint64_t seed, double sep, const int64_t *nv, int blo0, int blo1, int bhi0, int bhi1) {
    if (!ctx) return BBGPU_ERR_ARG;
    int rc = wind_args(ctx, out, sr, nv, sep);
    if (rc) return rc;
    if (ring_lo < 0 || ring_hi > nsub || ring_lo > ring_hi) return fail(ctx, BBGPU_ERR_ARG, "galmod_wind: shells");
    CK(cudaSetDevice(ctx->device));
    if (bhi1 <= blo1 || bhi0 <= blo0 || ring_hi == ring_lo) return BBGPU_OK;
    std::vector<WindClouds> W(1);
    if (bbh_wind_clouds(&W[0], seed, sr, nsub, ring_lo, ring_hi, sep, nv, &ctx->g))
        return fail(ctx, BBGPU_ERR_ARG, "galmod_wind: cloud or velocity-sample counts out of range");
    return wind_mc_run(ctx, out, W, blo0, blo1, bhi0, bhi1);
}

extern "C" int bbgpu_galwind_spherical(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int nchunks,
                                       const int *chunk_lo, const int *chunk_hi, const uint64_t *seeds, double sep,
                                       const int64_t *nv, int blo0, int blo1, int bhi0, int bhi1, int threads) {
    if (!ctx) return BBGPU_ERR_ARG;
    int rc = wind_args(ctx, out, sr, nv, sep);
    if (rc) return rc;
    if (nchunks < 0 || (nchunks && (!chunk_lo || !chunk_hi || !seeds)))
        return fail(ctx, BBGPU_ERR_ARG, "galwind_spherical: chunks");
    for (int c = 0; c < nchunks; c++)
        if (chunk_lo[c] < 0 || chunk_hi[c] > nsub || chunk_lo[c] > chunk_hi[c])
            return fail(ctx, BBGPU_ERR_ARG, "galwind_spherical: a chunk outside the shells");
    CK(cudaSetDevice(ctx->device));
    if (bhi1 <= blo1 || bhi0 <= blo0 || nchunks == 0) return BBGPU_OK;
    // the chunks' streams parsed on host threads (each chunk its own stream), then one device pass
    std::vector<WindClouds> W(nchunks);
    std::vector<int> err(nchunks, 0);
    const int nt = std::max(1, std::min(threads, nchunks));
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
        pool.emplace_back([&, t]() {
            for (int c = t; c < nchunks; c += nt)
                err[c] = bbh_wind_clouds(&W[c], seeds[c], sr, nsub, chunk_lo[c], chunk_hi[c], sep, nv, &ctx->g);
        });
    for (std::thread &th : pool) th.join();
    for (int e : err)
        if (e) return fail(ctx, BBGPU_ERR_ARG, "galwind_spherical: cloud or velocity-sample counts out of range");
    return wind_mc_run(ctx, out, W, blo0, blo1, bhi0, bhi1);
}

extern "C" int bbgpu_galmod_analytic(bbgpu_ctx *ctx, double *out, const double *sr, int nsub, int ring_lo, int ring_hi,
                                     int nzq, int blo0, int blo1, int bhi0, int bhi1) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!out || !sr || ring_lo < 0 || ring_hi > nsub || ring_lo > ring_hi || blo0 > bhi0 || blo1 > bhi1)
        return fail(ctx, BBGPU_ERR_ARG, "galmod_analytic: invalid arguments");
    if (!ctx->grid_set) return fail(ctx, BBGPU_ERR_STATE, "galmod_analytic before set_grid");
    if (!ctx->d_vedges) return fail(ctx, BBGPU_ERR_STATE, "galmod_analytic: set_grid was given no channel edges");
    const GridDev &g = ctx->g;
    if (an_smem_bytes(g.nz, g.nlines) > AN_SMEM_MAX)
        return fail(ctx, BBGPU_ERR_ARG, "galmod_analytic: %d channels x %d lines above the device limit", g.nz, g.nlines);
    CK(cudaSetDevice(ctx->device));
    const int ns = ring_hi - ring_lo, by = bhi1 - blo1, bx = bhi0 - blo0;
    if (ns == 0 || by == 0 || bx == 0) return BBGPU_OK;
    std::vector<double> s2((size_t)BBGPU_NSR * ns);
    for (int r = 0; r < BBGPU_NSR; r++)
        for (int i = 0; i < ns; i++) s2[(size_t)r * ns + i] = sr[(size_t)r * nsub + ring_lo + i];
    std::vector<AnSub> subs(ns);
    ZgridCache zc;
    const int e = bbh_an_subs(s2.data(), ns, &g, nzq, blo0, blo1, bhi0, bhi1, ctx->h_cd2i.data(), 0, nullptr, nullptr,
                              subs.data(), zc);
    const std::vector<double> &zq = zc.zq, &wq = zc.wq;
    if (e == -10000) return fail(ctx, BBGPU_ERR_ARG, "galmod_analytic: the total flux is not finite");
    DevBufs B(ctx, 0);
    AnDev D;
    int rc = an_upload(ctx, B, subs, s2.data(), ns, zq, wq, D);
    if (rc) return rc;
    const size_t n = (size_t)by * bx * g.nz;
    long long *o64 = nullptr;
    MemberDev *dm = nullptr;
    if (!B.get(&o64, n * sizeof(long long)) || !B.get(&dm, sizeof(MemberDev)))
        return fail(ctx, BBGPU_ERR_NOMEM, "galmod_analytic: allocation failed");
    MemberDev M{};
    M.blo0 = blo0; M.blo1 = blo1; M.bhi0 = bhi0; M.bhi1 = bhi1; M.bx = bx; M.by = by; M.fix_exp = e;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(dm, &M, sizeof M, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(o64, 0, n * sizeof(long long), s));
    long long *ast = nullptr;
    int *asg = nullptr;
    if (!B.get(&ast, 2 * sizeof(long long)) || !B.get(&asg, 4 * sizeof(int)))
        return fail(ctx, BBGPU_ERR_NOMEM, "galmod_analytic: allocation failed");
    const long long hst[2] = {0, D.nsamp};
    const int hsg[4] = {0, 0, -1, 1};                   // (the member's own samples)
    CK(cudaMemcpyAsync(ast, hst, sizeof hst, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(asg, hsg, sizeof hsg, cudaMemcpyHostToDevice, s));
    launch_an_model(s, g, D.subs, ns, D.sbase, D.ssub, D.cs, ast, asg, 1, D.nsamp, D.zq, D.wq, ctx->d_vedges,
                    ctx->d_cd2i, ctx->d_ptab, dm, o64, (long long)n, 0);
    CKL();
    std::vector<long long> h(n);
    CK(cudaMemcpyAsync(h.data(), o64, n * sizeof(long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const double sc = ldexp(1.0, -e);
    for (size_t i = 0; i < n; i++) out[i] += (double)h[i] * sc;
    return BBGPU_OK;
}

extern "C" int bbgpu_ring_maps_analytic(bbgpu_ctx *ctx, double *out, int nr, const double *sr, int nsub,
                                        const int64_t *widx, const double *wval, int nzq, int blo0, int blo1, int bhi0,
                                        int bhi1) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!out || !sr || !widx || !wval || nr < 0 || nsub < 0 || blo0 > bhi0 || blo1 > bhi1)
        return fail(ctx, BBGPU_ERR_ARG, "ring_maps_analytic: invalid arguments");
    if (!ctx->grid_set) return fail(ctx, BBGPU_ERR_STATE, "ring_maps_analytic before set_grid");
    for (int i = 0; i < 2 * nsub; i++)
        if (widx[i] >= nr) return fail(ctx, BBGPU_ERR_ARG, "ring_maps_analytic: ring index %lld >= %d", (long long)widx[i], nr);
    CK(cudaSetDevice(ctx->device));
    const int by = bhi1 - blo1, bx = bhi0 - blo0;
    if (nsub == 0 || nr == 0 || by == 0 || bx == 0) return BBGPU_OK;
    const GridDev &g = ctx->g;
    std::vector<AnSub> subs(nsub);
    ZgridCache zc;
    const int e = bbh_an_subs(sr, nsub, &g, nzq, blo0, blo1, bhi0, bhi1, ctx->h_cd2i.data(), 1, widx, wval,
                              subs.data(), zc);
    const std::vector<double> &zq = zc.zq, &wq = zc.wq;
    if (e == -10000) return fail(ctx, BBGPU_ERR_ARG, "ring_maps_analytic: the weights are not finite");
    DevBufs B(ctx, 1);
    AnDev D;
    int rc = an_upload(ctx, B, subs, sr, nsub, zq, wq, D);
    if (rc) return rc;
    const size_t n = (size_t)nr * by * bx;
    long long *m64 = nullptr, *dwi = nullptr;
    double *dwv = nullptr;
    if (!B.get(&m64, n * sizeof(long long)) || !B.get(&dwi, sizeof(long long) * 2 * nsub) ||
        !B.get(&dwv, sizeof(double) * 2 * nsub))
        return fail(ctx, BBGPU_ERR_NOMEM, "ring_maps_analytic: allocation failed");
    MemberDev M{};
    M.blo0 = blo0; M.blo1 = blo1; M.bhi0 = bhi0; M.bhi1 = bhi1; M.bx = bx; M.by = by; M.fix_exp = e;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(dwi, widx, sizeof(long long) * 2 * nsub, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dwv, wval, sizeof(double) * 2 * nsub, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(m64, 0, n * sizeof(long long), s));
    launch_an_maps(s, g, D.subs, nsub, D.sbase, D.ssub, D.cs, D.nsamp, D.zq, D.wq, dwi, dwv, M, m64);
    CKL();
    std::vector<long long> h(n);
    CK(cudaMemcpyAsync(h.data(), m64, n * sizeof(long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const double sc = ldexp(1.0, -e);
    for (size_t i = 0; i < n; i++) out[i] += (double)h[i] * sc;
    return BBGPU_OK;
}

extern "C" int bbgpu_conv_sparse(bbgpu_ctx *ctx, const double *model, double *out, int ny, int nx, int nz,
                                 const double *kernel, int ky, int kx, double scale) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!model || !out || !kernel || ny < 0 || nx < 0 || nz < 0 || ky < 1 || kx < 1)
        return fail(ctx, BBGPU_ERR_ARG, "conv_sparse: invalid arguments");
    CK(cudaSetDevice(ctx->device));
    const size_t n = (size_t)ny * nx * nz;
    if (n == 0) return BBGPU_OK;
    DevBufs B(ctx, 2);
    double *dm = nullptr, *dout = nullptr, *dk = nullptr;
    if (!B.get(&dm, n * 8) || !B.get(&dout, n * 8) || !B.get(&dk, (size_t)ky * kx * 8))
        return fail(ctx, BBGPU_ERR_NOMEM, "conv_sparse: allocation failed");
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(dm, model, n * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dk, kernel, (size_t)ky * kx * 8, cudaMemcpyHostToDevice, s));
    launch_conv_sparse(s, dm, dout, ny, nx, nz, dk, ky, kx, scale);
    CKL();
    CK(cudaMemcpyAsync(out, dout, n * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return BBGPU_OK;
}

extern "C" int bbgpu_norm(bbgpu_ctx *ctx, double *model, int bsy, int bsx, int nz, const float *data, const uint8_t *mask,
                          int dny, int dnx, int64_t blo0, int64_t blo1, double x0, double y0, double phi, double inc,
                          double r1, double r2, double wpow, int side, int ftype, const double *chan_noise,
                          double data_noise, double bweight, int normtype, const double *pre, const int64_t *ilo,
                          const int64_t *ihi, int ky, const double *thr, int foot, double hmax, double *out) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!model || !data || !mask || !chan_noise || !out || bsy < 0 || bsx < 0 || nz < 1 || blo0 < 0 || blo1 < 0 ||
        blo1 + bsy > dny || blo0 + bsx > dnx || (pre && (!ilo || !ihi || !thr || ky < 1)))
        return fail(ctx, BBGPU_ERR_ARG, "norm: invalid arguments");
    CK(cudaSetDevice(ctx->device));
    const int np = bsy * bsx;
    const size_t n = (size_t)np * nz;
    // the ring's pixels and weights (host: the reference's float64 and C library calls)
    std::vector<uint8_t> inside(np ? np : 1);
    std::vector<double> wmap(np ? np : 1);
    bbh_norm_footprint(bsy, bsx, x0, y0, phi, inc, r1, r2, wpow, side, foot, hmax, inside.data(), wmap.data());
    // the box of the data and mask ("yxz"), contiguous
    std::vector<float> dbox(n ? n : 1);
    std::vector<uint8_t> mbox(n ? n : 1);
    for (int y = 0; y < bsy; y++)
        for (int x = 0; x < bsx; x++) {
            const size_t src = (((size_t)(y + blo1)) * dnx + (size_t)(x + blo0)) * nz;
            memcpy(&dbox[((size_t)y * bsx + x) * nz], data + src, sizeof(float) * nz);
            memcpy(&mbox[((size_t)y * bsx + x) * nz], mask + src, nz);
        }
    DevBufs B(ctx, 3);
    double *dm = nullptr, *dw = nullptr, *dcn = nullptr, *dpre = nullptr, *dthr = nullptr, *dpart = nullptr,
           *dP = nullptr;
    float *dd = nullptr;
    uint8_t *dk = nullptr, *din = nullptr;
    long long *dilo = nullptr, *dihi = nullptr;
    if (!B.get(&dm, n * 8) || !B.get(&dd, n * 4) || !B.get(&dk, n) || !B.get(&din, np) || !B.get(&dw, np * 8) ||
        !B.get(&dcn, (size_t)nz * 8) || !B.get(&dpart, (size_t)np * 4 * 8) ||
        (pre && (!B.get(&dpre, n * 8) || !B.get(&dP, (size_t)bsy * (bsx + 1) * nz * 8) ||
                 !B.get(&dthr, (size_t)nz * 8) || !B.get(&dilo, (size_t)ky * 8) ||
                 !B.get(&dihi, (size_t)ky * 8))))
        return fail(ctx, BBGPU_ERR_NOMEM, "norm: allocation failed");
    cudaStream_t s = ctx->stream;
    if (n) {
        CK(cudaMemcpyAsync(dm, model, n * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dd, dbox.data(), n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dk, mbox.data(), n, cudaMemcpyHostToDevice, s));
    }
    if (np) {
        CK(cudaMemcpyAsync(din, inside.data(), np, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dw, wmap.data(), (size_t)np * 8, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(dcn, chan_noise, (size_t)nz * 8, cudaMemcpyHostToDevice, s));
    if (pre) {
        CK(cudaMemcpyAsync(dpre, pre, n * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dthr, thr, (size_t)nz * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dilo, ilo, (size_t)ky * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dihi, ihi, (size_t)ky * 8, cudaMemcpyHostToDevice, s));
        launch_norm_prefix(s, dpre, dP, bsy, bsx, nz);
        CKL();
    }
    std::vector<double> part((size_t)np * 4 + 1);
    double factor = 1.0;
    if (normtype == 1 && np) {
        launch_norm_sums(s, dm, dd, dk, din, bsy, bsx, nz, dpart);
        CKL();
        CK(cudaMemcpyAsync(part.data(), dpart, (size_t)np * 2 * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        double ms = 0.0, os = 0.0;
        for (int p = 0; p < np; p++) {
            ms += part[2 * p];
            os += part[2 * p + 1];
        }
        factor = ms != 0 ? os / ms : 0.0;
    }
    if (np) {
        launch_norm_pix(s, dm, dd, dk, din, dw, bsy, bsx, nz, ftype, dcn, data_noise, normtype, factor, dP, dilo, dihi,
                        ky, dthr, dpart);
        CKL();
        CK(cudaMemcpyAsync(part.data(), dpart, (size_t)np * 4 * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(model, dm, n * 8, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    double minfunc = 0.0;
    long long nb = 0, nt = 0;
    for (int p = 0; p < np; p++) {
        minfunc += part[4 * p];
        nb += (long long)part[4 * p + 1];
        nt += (long long)part[4 * p + 2];
    }
    if (nt - nb == 0) *out = INFINITY;
    else *out = pow(1 + (double)nb / (double)nt, bweight) * minfunc / (double)(nt - nb);
    return BBGPU_OK;
}

// ------------------------------------------------------------------------------------------- flux normalisation
static int profile_consts(bbgpu_ctx *ctx, const double *radii, int n, double smooth, double corr, double floor_,
                          std::vector<int> &ent) {
    std::vector<int> lc(3 * (n > 2 ? n - 2 : 1)), ord(n);
    std::vector<double> lv(3 * (n > 2 ? n - 2 : 1));
    std::vector<unsigned char> nr(n > 2 ? n - 2 : 1);
    double d = 0.0, norm = 0.0;
    bbh_profile_consts(radii, n, lc.data(), lv.data(), ord.data(), nr.data(), &d, &norm);
    ctx->pc.n = n;
    ctx->pc.smooth = smooth;
    ctx->pc.corr = corr;
    ctx->pc.floor_ = floor_;
    ctx->pc.norm = norm;
    ctx->pc.d = d;
    // entries of the packed normal equations: G (i <= j), then h
    const int ng = n * (n + 1) / 2;
    ctx->nent = ng + n;
    ent.assign(2 * ctx->nent, -1);
    int e = 0;
    for (int i = 0; i < n; i++)
        for (int j = i; j < n; j++, e++) {
            ent[e] = i;
            ent[ctx->nent + e] = j;
        }
    for (int i = 0; i < n; i++, e++) ent[e] = i;
    std::vector<int> p0(n, 1);
    cudaFree(ctx->d_lc); cudaFree(ctx->d_lv); cudaFree(ctx->d_ord); cudaFree(ctx->d_near); cudaFree(ctx->d_p0);
    cudaFree(ctx->d_ent);
    ctx->d_lc = nullptr; ctx->d_lv = nullptr; ctx->d_ord = nullptr; ctx->d_near = nullptr; ctx->d_p0 = nullptr;
    ctx->d_ent = nullptr;
    CK(cudaMalloc(&ctx->d_lc, lc.size() * sizeof(int)));
    CK(cudaMalloc(&ctx->d_lv, lv.size() * sizeof(double)));
    CK(cudaMalloc(&ctx->d_ord, ord.size() * sizeof(int)));
    CK(cudaMalloc(&ctx->d_near, nr.size()));
    CK(cudaMalloc(&ctx->d_p0, n * sizeof(int)));
    CK(cudaMalloc(&ctx->d_ent, ent.size() * sizeof(int)));
    CK(cudaMemcpy(ctx->d_lc, lc.data(), lc.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_lv, lv.data(), lv.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_ord, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_near, nr.data(), nr.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_p0, p0.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_ent, ent.data(), ent.size() * sizeof(int), cudaMemcpyHostToDevice));
    return 0;
}

#define PROF_NMAX 64

extern "C" int bbgpu_set_profile(bbgpu_ctx *ctx, int nr, int blo0, int blo1, int bhi0, int bhi1, const double *ymap,
                                 const double *rms, const uint8_t *ok, const double *radii, double smooth,
                                 double corr, double floor_, double mapscale) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!ctx->grid_set) return fail(ctx, BBGPU_ERR_STATE, "set_profile before set_grid");
    const GridDev &g = ctx->g;
    const int n = nr + 1;
    if (!ymap || !rms || !ok || !radii || nr < 1 || n > PROF_NMAX || blo0 < 0 || blo1 < 0 || bhi0 > g.nx ||
        bhi1 > g.ny || bhi0 <= blo0 || bhi1 <= blo1)
        return fail(ctx, BBGPU_ERR_ARG, "set_profile: invalid arguments (1 to %d rings, a box inside the cube)",
                    PROF_NMAX - 1);
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    ProfBox &b = ctx->pbox;
    b.blo0 = blo0; b.blo1 = blo1; b.bhi0 = bhi0; b.bhi1 = bhi1;
    b.bx = bhi0 - blo0; b.by = bhi1 - blo1; b.nrp = n;
    b.npix = (long long)b.bx * b.by;
    // the pixels used (bbarolo/profile.py:76-79): in the region, rms > 0, finite data
    std::vector<int> pix;
    std::vector<double> w, wy;
    double bb = 0.0;
    for (long long p = 0; p < b.npix; p++) {
        const double sg = rms[p], y = ymap[p];
        if (!ok[p] || !(sg > 0) || !std::isfinite(y)) continue;
        pix.push_back((int)p);
        w.push_back(1.0 / (sg * sg));
        wy.push_back(y / (sg * sg));
        const double bv = y / sg;
        bb += bv * bv;
    }
    // the used pixels in blocks of 8 x 16 (the tiles of the normal equations then cover compact patches, crossed
    // by few rings); within a block in raster order
    {
        std::vector<int> order(pix.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
        const int bx16 = (b.bx + 15) / 16;
        auto key = [&](int i) {
            const int p = pix[i], py = p / b.bx, px = p - py * b.bx;
            return ((long long)(py / 8) * bx16 + px / 16) * 128 + (py % 8) * 16 + px % 16;
        };
        std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return key(a) < key(c); });
        std::vector<int> p2(pix.size());
        std::vector<double> w2(w.size()), wy2(wy.size());
        for (size_t i = 0; i < order.size(); i++) {
            p2[i] = pix[order[i]];
            w2[i] = w[order[i]];
            wy2[i] = wy[order[i]];
        }
        pix.swap(p2);
        w.swap(w2);
        wy.swap(wy2);
    }
    ctx->npix_used = (int)pix.size();
    ctx->pc.m = (int)pix.size();
    ctx->pc.bb = bb;
    ctx->mapscale = mapscale;
    cudaFree(ctx->d_ppix); cudaFree(ctx->d_pw); cudaFree(ctx->d_pwy);
    ctx->d_ppix = nullptr; ctx->d_pw = nullptr; ctx->d_pwy = nullptr;
    const size_t np1 = pix.size() ? pix.size() : 1;
    CK(cudaMalloc(&ctx->d_ppix, np1 * sizeof(int)));
    CK(cudaMalloc(&ctx->d_pw, np1 * sizeof(double)));
    CK(cudaMalloc(&ctx->d_pwy, np1 * sizeof(double)));
    if (pix.size()) {
        CK(cudaMemcpy(ctx->d_ppix, pix.data(), pix.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_pw, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_pwy, wy.data(), wy.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    std::vector<int> ent;
    int rc = profile_consts(ctx, radii, n, smooth, corr, floor_, ent);
    if (rc) return rc;
    ctx->zcache.clear();
    ctx->samp_key.clear();
    ctx->prof_set = true;
    ctx->prof_uploaded = false;
    return BBGPU_OK;
}

extern "C" int bbgpu_eval_upload_profile(bbgpu_ctx *ctx, int nsm, const double *sr_maps, const int64_t *widx,
                                         const double *wval) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!ctx->prof_set) return fail(ctx, BBGPU_ERR_STATE, "eval_upload_profile before set_profile");
    if (!ctx->uploaded) return fail(ctx, BBGPU_ERR_STATE, "eval_upload_profile before eval_upload");
    const int nb = ctx->nb, nsub = ctx->nsub, n = ctx->pc.n;
    if (!sr_maps || !widx || !wval || nsm < nsub) return fail(ctx, BBGPU_ERR_ARG, "eval_upload_profile: invalid arguments");
    for (int i = 0; i < 2 * nsm; i++)
        if (widx[i] >= n) return fail(ctx, BBGPU_ERR_ARG, "eval_upload_profile: ring index %lld >= %d", (long long)widx[i], n);
    const GridDev &g = ctx->g;
    CK(cudaSetDevice(ctx->device));
    // the sub-ring radii are shared by the batch (one table of azimuthal samples)
    for (int k = 1; k < nb; k++)
        if (memcmp(sr_maps + (size_t)k * BBGPU_NSR * nsm, sr_maps, sizeof(double) * nsm))
            return fail(ctx, BBGPU_ERR_ARG, "eval_upload_profile: member %d has other sub-ring radii", k);
    bool thick = false;
    for (int k = 0; k < nb && !thick; k++)
        for (int i = 0; i < nsm; i++)
            if (sr_maps[(size_t)k * BBGPU_NSR * nsm + 6 * (size_t)nsm + i] > 0) { thick = true; break; }
    const int nzq = thick ? 1024 : 1;
    const ProfBox &bx = ctx->pbox;
    int rc;
    if ((rc = hgrow(ctx, &ctx->h_psub, &ctx->h_psub_cap, (size_t)nb * nsm))) return rc;
    if ((rc = hgrow(ctx, &ctx->h_preuse, &ctx->h_preuse_cap, (size_t)nb * nsm))) return rc;
    memset(ctx->h_preuse, 0, (size_t)nsm);
    ZgridCache &zc = ctx->zcache;
    if (zc.zq.size() > ((size_t)1 << 24)) zc.clear();
    const size_t zold = zc.uploaded;
    std::vector<int> fix(nb);
    // the rows of each column that differ from member 0's (the constants reused, the rows of the maps)
    std::vector<uint16_t> pdiff((size_t)nb * nsm, 0);
    for (int k = 0; k < nb; k++) {
        if (k) bbh_column_diff(sr_maps + (size_t)k * BBGPU_NSR * nsm, sr_maps, nsm, pdiff.data() + (size_t)k * nsm);
        const int e = bbh_an_subs(sr_maps + (size_t)k * BBGPU_NSR * nsm, nsm, &g, nzq, bx.blo0, bx.blo1, bx.bhi0,
                                  bx.bhi1, ctx->h_cd2i.data(), 1, widx, wval, ctx->h_psub + (size_t)k * nsm, zc,
                                  k ? sr_maps : nullptr, k ? ctx->h_psub : nullptr,
                                  k ? ctx->h_preuse + (size_t)k * nsm : nullptr,
                                  k ? pdiff.data() + (size_t)k * nsm : nullptr);
        if (e == -10000) return fail(ctx, BBGPU_ERR_ARG, "eval_upload_profile: member %d: weights not finite", k);
        fix[k] = std::min(e, 100);
    }
    cudaStream_t s = ctx->stream;
    // the table of azimuthal samples (radii of the sub-rings): uploaded when the radii change
    std::string skey((const char *)sr_maps, sizeof(double) * nsm);
    skey.append((const char *)&g.pixarea, sizeof(double));
    if (skey != ctx->samp_key) {
        std::vector<int> sbase, ssub;
        std::vector<double> cs;
        bbh_an_samples(sr_maps, nsm, &g, sbase, ssub, cs);
        if ((rc = dgrow(ctx, &ctx->d_psbase, &ctx->d_psbase_cap, sbase.size()))) return rc;
        if ((rc = dgrow(ctx, &ctx->d_pssub, &ctx->d_pssub_cap, ssub.size()))) return rc;
        if ((rc = dgrow(ctx, &ctx->d_pcs, &ctx->d_pcs_cap, cs.size()))) return rc;
        std::vector<float> csf;
        bbh_an_samples_f32(cs, csf);
        if ((rc = dgrow(ctx, &ctx->d_pcsf, &ctx->d_pcsf_cap, csf.size()))) return rc;
        CK(cudaMemcpy(ctx->d_pcsf, csf.data(), sizeof(float) * csf.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_psbase, sbase.data(), sizeof(int) * sbase.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_pssub, ssub.data(), sizeof(int) * ssub.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_pcs, cs.data(), sizeof(double) * cs.size(), cudaMemcpyHostToDevice));
        ctx->pnsamp = sbase[nsm];
        ctx->psbase_host = sbase;
        ctx->samp_key = skey;
        ctx->h2d += (long long)(sizeof(int) * (sbase.size() + ssub.size()) + sizeof(double) * cs.size());
    }
    // The rows of the maps. A member whose ring-map constants are member 0's in every sub-ring (a step of a
    // velocity or the density) has member 0's maps and so its profile: it takes member 0's solution. A member
    // that differs in a few sub-rings (a step of one ring's geometry), with the same fixed-point exponent, gets
    // a row holding the difference from member 0's maps: its deposits of those sub-rings and member 0's negated,
    // summed with member 0's row when the maps are converted (exact: 64-bit fixed point, the same units).
    // Every other member gets a row of its own over every sample.
    std::vector<int> uidx, ubase, prof_of(nb), mseg;
    std::vector<long long> mstart;
    {
        const std::vector<int> &sb = ctx->psbase_host;
        long long tot = 0;
        auto seg = [&](int u, int k, int ir, int sign, long long cnt) {
            if (cnt <= 0) return;
            mstart.push_back(tot);
            mseg.insert(mseg.end(), {u, k, ir, sign});
            tot += cnt;
        };
        std::vector<int> ch;
        for (int k = 0; k < nb; k++) {
            bool delta = false;
            if (ctx->share && k > 0 && fix[k] == fix[0]) {
                const double *sk = sr_maps + (size_t)k * BBGPU_NSR * nsm;
                const uint16_t *dm = pdiff.data() + (size_t)k * nsm;
                long long nch = 0;
                ch.clear();
                for (int i = 0; i < nsm; i++)
                    if (!bbh_map_same(dm[i], sk, nsm, i)) {
                        ch.push_back(i);
                        nch += sb[i + 1] - sb[i];
                    }
                if (ch.empty()) {
                    prof_of[k] = 0;
                    continue;
                }
                delta = 2 * nch < ctx->pnsamp;
            }
            const int u = (int)uidx.size();
            prof_of[k] = u;
            uidx.push_back(k);
            ubase.push_back(delta ? 0 : -1);
            if (delta) {
                for (int i : ch) {
                    seg(u, k, i, 1, sb[i + 1] - sb[i]);
                    seg(u, 0, i, -1, sb[i + 1] - sb[i]);
                }
            } else {
                seg(u, k, -1, 1, ctx->pnsamp);
            }
        }
        ctx->mtot = tot;
        mstart.push_back(tot);
    }
    ctx->nu = (int)uidx.size();
    ctx->nseg = (int)mstart.size() - 1;
    ctx->nu_delta = 0;
    for (int b : ubase) ctx->nu_delta += b >= 0;
    ctx->prof_of_host = prof_of;
    ctx->mc_dirty = true;
    ctx->an_dirty = true;
    // the vertical grids: the new ones appended on the device (the table grows with a copy of the old part)
    const size_t nz1 = zc.zq.size() + 1;
    if (zc.uploaded == 0 || nz1 > ctx->d_pzq_cap) {
        if (nz1 > ctx->d_pzq_cap) {
            for (void *q : {(void *)ctx->d_pzq, (void *)ctx->d_pzqf, (void *)ctx->d_pwqf}) cudaFree(q);
            ctx->d_pzq = nullptr; ctx->d_pzqf = nullptr; ctx->d_pwqf = nullptr;
            ctx->d_pzq_cap = ctx->d_pzqf_cap = ctx->d_pwqf_cap = 0;
            if ((rc = dgrow(ctx, &ctx->d_pzq, &ctx->d_pzq_cap, 2 * nz1))) return rc;
            if ((rc = dgrow(ctx, &ctx->d_pzqf, &ctx->d_pzqf_cap, 2 * nz1))) return rc;
            if ((rc = dgrow(ctx, &ctx->d_pwqf, &ctx->d_pwqf_cap, 2 * nz1))) return rc;
        }
        zc.uploaded = 0;
    }
    if (zc.zq.size() > zc.uploaded) {
        const size_t a0 = zc.uploaded, m = zc.zq.size() - a0;
        std::vector<float> zf(m), wf(m);
        for (size_t i = 0; i < m; i++) {
            zf[i] = (float)zc.zq[a0 + i];
            wf[i] = (float)zc.wq[a0 + i];
        }
        CK(cudaMemcpy(ctx->d_pzq + a0, zc.zq.data() + a0, sizeof(double) * m, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_pzqf + a0, zf.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->d_pwqf + a0, wf.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
        ctx->h2d += (long long)(16 * m);
        zc.uploaded = zc.zq.size();
    }
    (void)zold;
    std::vector<float> wvalf(2 * (size_t)nsm);
    std::vector<int> wi(2 * (size_t)nsm);
    for (int i = 0; i < 2 * nsm; i++) { wvalf[i] = (float)wval[i]; wi[i] = (int)widx[i]; }
    // ring area of each model sub-ring (bbarolo/galmod.py:107), for the densities of the MC model
    std::vector<double> rap(nsub ? nsub : 1);
    for (int i = 0; i < nsub; i++) rap[i] = 2 * M_PI * sr_maps[i] * g.radsep / g.pixarea;
    const long long per = bx.npix * bx.nrp;
    if ((rc = dgrow(ctx, &ctx->d_psub, &ctx->d_psub_cap, (size_t)nb * nsm))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pwidx, &ctx->d_pwidx_cap, wi.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pwvalf, &ctx->d_pwvalf_cap, wvalf.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pwval, &ctx->d_pwval_cap, 2 * (size_t)nsm))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_rap, &ctx->d_rap_cap, rap.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pfix, &ctx->d_pfix_cap, (size_t)nb))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_maps64, &ctx->d_maps64_cap, (size_t)nb * per))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_maps32, &ctx->d_maps32_cap, (size_t)nb * per))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_K, &ctx->d_K_cap, (size_t)nb * per))) return rc;
    const int nt = prof_gram_tiles(ctx->npix_used);
    if ((rc = dgrow(ctx, &ctx->d_gpart, &ctx->d_gpart_cap, (size_t)nb * (nt ? nt : 1) * ctx->nent))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_gh, &ctx->d_gh_cap, (size_t)nb * ctx->nent))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_px, &ctx->d_px_cap, (size_t)nb * n))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pp, &ctx->d_pp_cap, (size_t)nb * n))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pstat, &ctx->d_pstat_cap, (size_t)nb))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pxu, &ctx->d_pxu_cap, (size_t)nb * n))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_pstatu, &ctx->d_pstatu_cap, (size_t)nb))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_mstart, &ctx->d_mstart_cap, mstart.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_mseg, &ctx->d_mseg_cap, mseg.size() + 4))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_uidx, &ctx->d_uidx_cap, uidx.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_ubase, &ctx->d_ubase_cap, ubase.size()))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_prof_of, &ctx->d_prof_of_cap, prof_of.size()))) return rc;
    // the maps' convolution: one member descriptor per row, the likelihood box (and the row's 8 x 8 pixel blocks
    // in the block table)
    const int nbx8 = (bx.bx + 7) / 8, nblk8 = nbx8 * ((bx.by + 7) / 8);
    ctx->pmem_host.assign(nb, MemberDev{});
    for (int u = 0; u < nb; u++) {
        MemberDev &M = ctx->pmem_host[u];
        M.blo0 = bx.blo0; M.blo1 = bx.blo1; M.bhi0 = bx.bhi0; M.bhi1 = bx.bhi1; M.bx = bx.bx; M.by = bx.by;
        M.tile_off = u * nblk8;
        M.ntx = nbx8;
        M.nty = (bx.by + 7) / 8;
    }
    if (ctx->nu_delta) {
        int nct, ntxc, shx, shy;
        conv_tile_shape(bx.nrp, bx.bx, bx.by, nct, ntxc, shx, shy);
        if ((rc = dgrow(ctx, &ctx->d_blk, &ctx->d_blk_cap, (size_t)ctx->nu * nblk8 + 1)) ||
            (rc = dgrow(ctx, &ctx->d_ktab, &ctx->d_ktab_cap, (size_t)ctx->nu * nct + 1)) ||
            (rc = dgrow(ctx, &ctx->d_gflag, &ctx->d_gflag_cap, (size_t)ctx->nu * (nt ? nt : 1) + 1)))
            return rc;
    }
    const int npart = conv_resid_npart(ctx->pmem_host.data(), nb, bx.nrp);
    if ((rc = dgrow(ctx, &ctx->d_pmem, &ctx->d_pmem_cap, (size_t)nb))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_ppart, &ctx->d_ppart_cap, (size_t)2 * nb * (npart ? npart : 1)))) return rc;
    if ((rc = dgrow(ctx, &ctx->d_preuse, &ctx->d_preuse_cap, (size_t)nb * nsm))) return rc;
    CK(cudaMemcpyAsync(ctx->d_psub, ctx->h_psub, sizeof(AnSub) * (size_t)nb * nsm, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_preuse, ctx->h_preuse, (size_t)nb * nsm, cudaMemcpyHostToDevice, s));
    launch_fill_copy(s, ctx->d_psub, sizeof(AnSub), nsm, nb, ctx->d_preuse);
    CKL();
    CK(cudaMemcpyAsync(ctx->d_pwidx, wi.data(), sizeof(int) * wi.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_pwvalf, wvalf.data(), sizeof(float) * wvalf.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_pwval, wval, sizeof(double) * 2 * (size_t)nsm, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_rap, rap.data(), sizeof(double) * rap.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_pfix, fix.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_pmem, ctx->pmem_host.data(), sizeof(MemberDev) * nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_mstart, mstart.data(), sizeof(long long) * mstart.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_mseg, mseg.data(), sizeof(int) * mseg.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_uidx, uidx.data(), sizeof(int) * uidx.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_ubase, ubase.data(), sizeof(int) * ubase.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->d_prof_of, prof_of.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
    ctx->h2d += (long long)(sizeof(AnSub) * (size_t)nb * nsm + sizeof(int) * nb + sizeof(long long) * mstart.size() +
                            sizeof(int) * (mseg.size() + uidx.size() + ubase.size() + nb));
    // (the host vectors go out of scope: finish the copies first)
    CK(cudaStreamSynchronize(s));
    ctx->nsm = nsm;
    ctx->prof_uploaded = true;
    ctx->ran = false;
    return BBGPU_OK;
}

extern "C" int bbgpu_eval_profile(bbgpu_ctx *ctx, double *x, int *status) {
    if (!ctx || !x) return BBGPU_ERR_ARG;
    if (!ctx->ran || !ctx->prof_uploaded) return fail(ctx, BBGPU_ERR_STATE, "eval_profile: no profile computed");
    CK(cudaSetDevice(ctx->device));
    const int nb = ctx->nb, n = ctx->pc.n;
    CK(cudaMemcpyAsync(x, ctx->d_px, sizeof(double) * (size_t)nb * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (status) CK(cudaMemcpyAsync(status, ctx->d_pstat, sizeof(int) * nb, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return BBGPU_OK;
}

extern "C" int bbgpu_solve_profile(bbgpu_ctx *ctx, const double *A, const double *b, int m, int n, const double *radii,
                                   double smooth, double corr, double floor_, double *x, int *status) {
    if (ctx) ctx->gen++;
    if (!ctx) return BBGPU_ERR_ARG;
    if (!A || !b || !radii || !x || m < 1 || n < 1 || n > PROF_NMAX)
        return fail(ctx, BBGPU_ERR_ARG, "solve_profile: invalid arguments (1 to %d unknowns)", PROF_NMAX);
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    // (the profile constants of the batch path are replaced)
    ctx->prof_set = false;
    ctx->prof_uploaded = false;
    std::vector<int> ent;
    int rc = profile_consts(ctx, radii, n, smooth, corr, floor_, ent);
    if (rc) return rc;
    double bb = 0.0;
    for (int i = 0; i < m; i++) bb += b[i] * b[i];
    ctx->pc.m = m;
    ctx->pc.bb = bb;
    ProfBox bx{};
    bx.nrp = n;
    bx.npix = m;
    DevBufs B(ctx, 4);
    double *dA = nullptr, *db = nullptr, *dpart = nullptr, *dgh = nullptr, *dx = nullptr;
    int *dpp = nullptr, *dst = nullptr;
    const int nt = prof_gram_tiles(m);
    if (!B.get(&dA, sizeof(double) * (size_t)m * n) || !B.get(&db, sizeof(double) * m) ||
        !B.get(&dpart, sizeof(double) * (size_t)nt * ctx->nent) || !B.get(&dgh, sizeof(double) * ctx->nent) ||
        !B.get(&dx, sizeof(double) * n) || !B.get(&dpp, sizeof(int) * n) || !B.get(&dst, sizeof(int)))
        return fail(ctx, BBGPU_ERR_NOMEM, "solve_profile: allocation failed");
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(dA, A, sizeof(double) * (size_t)m * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(db, b, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    launch_prof_gram64(s, dA, bx, db, m, ctx->d_ent, ctx->d_ent + ctx->nent, ctx->nent, dpart, dgh);
    ctx->launches += 2;
    CKL();
    launch_prof_solve(s, dgh, ctx->pc, ctx->d_lc, ctx->d_lv, ctx->d_ord, ctx->d_near, ctx->d_p0, 1, dx, dpp, dst);
    CKL();
    int st = 0;
    CK(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&st, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (status) *status = st;
    return BBGPU_OK;
}
