// The beam convolution + residual on the tensor cores: tcgen05 MMAs with TMEM accumulators, the model staged by
// TMA (bbarolo/smooth.py:145-165 FFTConvolver.__call__, bbarolo/galmod.py:1273-1283 DiskModel.convolve,
// bbarolo/bayesian/likelihood.py:22-77 _sumsq_residuals / _residuals_fracerr). Same inputs, outputs and partial
// sums as k_conv_resid (conv_kernel.cuh); the float32 FMA kernel stays the default for the ring maps (41
// channels) and for kernels wider than these templates.
//
// Formulation: the "same" convolution of a channel plane is out[y, x] = sum_{a, b} kf[a, b] in[y - hy + a,
// x - hx + b] (kf the flipped beam kernel). A CTA owns a strip of 16 output columns of one member's box for
// 128 channels (the MMA's M: the channels are the rows of A, each channel a row of the model's channel-fastest
// layout), walking down the rows of the strip. For one input row yy, the row's KP input pixels x0 - hx + kk
// (kk < KP) form A (128 channels x KP pixels); B is the banded Toeplitz matrix of the kernel rows stacked along N:
// B[(j, ox), kk] = kf[ky - 1 - j, kk - ox] (zero outside the band). One MMA of N = 16 n adds the row's
// contribution to the n output rows it feeds (oy = yy + hy - a, a = 0 .. ky-1), whose accumulators are
// consecutive 16-column blocks of a TMEM ring of 32 output rows (512 columns). Output row oy is complete after
// input row oy - hy + ky - 1; the epilogue warps read it (tcgen05.ld), zero its columns for the row that reuses
// them, and apply the reference's threshold and scale and the masked residual.
//
// Precision: split products. BF16X3: a = ah + al (bf16 each, ah = rn(a), al = rn(a - ah)), likewise the taps;
// ah bh + ah bl + al bh in FP32 accumulation (dropped al bl and the splits' remainders: ~2^-17 relative per
// product). TF32X3: the same with tf32 halves (~2^-21). Both are compared per voxel with the float64 oracle.
//
// Pipeline (persistent CTAs, one per SM, 19 warps; each CTA takes work items, a strip or a run of its tiles, from a
// counter of the launch as it finishes the previous ones, so that the CTAs end together):
// warp 0 issues TMA loads of each input row (8-pixel boxes of 128 channels, zero fill outside the box; with a tile
// table each box from the member whose model holds that deposit tile) into float32 staging stages; warps 2-9 split
// the staged row into the hi/lo operand stage (K-major canonical layout, no swizzle; two warps per 32 channels, a
// half row each) and flag rows that are all zero; warp 1 (one lane) issues the MMAs and commits their completion
// to the stage's barrier and to the completed output row's barrier; warp 18 stages the data rows of the residual by
// TMA; warps 10-17 are the epilogue (warp w reads TMEM lanes 32 (w mod 4) .. 32 (w mod 4) + 31, half of a row's
// columns each). A role's time per row is its instruction count times the latency of its warps on each scheduler:
// the split and the epilogue, the longest, have two warps per lane quarter.
// Every wait on an mbarrier is bounded (about one second): on expiry the kernel sets ERR_TC in the error flag, waits
// (bounded) for its copies and MMAs in flight, frees its TMEM and returns.

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "kernels.h"

namespace {

constexpr int TC_X = 16;           // output columns of a strip
constexpr int TC_RING = 32;        // output rows held in TMEM (16 columns each)
constexpr int TC_COLS = TC_X * TC_RING;
constexpr int TC_M = 128;          // channels of a CTA
constexpr int NFS = 4;             // float32 staging stages of model rows
constexpr int NAS = 2;             // operand stages
constexpr int NDS = 4;             // float32 stages of data rows
constexpr int TC_THREADS = 608;
constexpr int EPW = 8;             // epilogue warps: two per TMEM lane quarter, 8 columns of a row each
constexpr int EPC = TC_X / 2;
constexpr int TC_MAX_TILES = 16;   // 16-row tiles of a work item
constexpr int BOX_PX = 8;          // pixels of a TMA box of the model
constexpr int BOX_BYTES = BOX_PX * TC_M * 4;
constexpr int DBOX_BYTES = TC_X * TC_M * 4;   // a data row of the strip
constexpr int ITQ = 8;             // slots of the ring that passes the CTA's work items to its warps

struct TcArgs {
    GridDev g;
    const MemberDev *mem;
    const CUtensorMap *maps;       // per member: its model (nz, bx, by) float32
    const CUtensorMap *dmaps;      // per member: the data it is compared with (nz, nx, ny) float32
    const uint4 *bimg;             // B (hi, then lo) in the shared-memory layout
    int bbytes;
    int ky, kx, hy, hx, wused, dx, nbox;
    int nz, nzb;
    int tpi, nsy, ntxg;            // tiles of a work item, work items of a strip, strips of the grid
    int nitems, nks;               // work items; K steps (32 bytes) of the MMAs
    int do_conv, do_resid;
    float *smoothed;
    long long mstride;
    double *partial;
    int npart;
    TileSrc ts;
    int *err;
    int *queue;                    // the launch's next work item (zeroed before the launch)
    unsigned fstage, astage, aop, bop, sbo_a, sbo_b;   // layout (bytes)
};

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }


__device__ __forceinline__ void mbar_init(uint64_t *b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait on the phase of parity `parity`: false (and ERR_TC) after 2^31 SM cycles (about one second at the
// GB300's clocks) or when another role gave up first. (The SM's cycle counter: reading the global timer costs
// far more, and a wait runs for every row of the pipeline.)
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile int *abort, int *err) {
    if (mbar_test(b, parity)) return true;
    const long long t0 = clock64();
    for (unsigned it = 0;; it++) {
        if (mbar_test(b, parity)) return true;
        if (it >= 8) __nanosleep(32);               // (a waiting warp leaves the issue slots to the others)
        if ((it & 63) == 63) {
            if (*abort) return false;
            if (clock64() - t0 > (1LL << 31)) {
                *abort = 1;
                atomicOr(err, ERR_TC);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// shared-memory matrix descriptor: canonical K-major layout without swizzle (core matrices of 8 rows x 16 bytes,
// lbo: next core matrix along K, sbo: next 8 rows)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
    d |= (uint64_t)1 << 46;                     // descriptor version of tcgen05
    return d;                                   // base offset 0, swizzle none
}

template <int V>
__device__ __forceinline__ void mma(uint32_t dtm, uint64_t a, uint64_t b, uint32_t idesc) {
    if (V == 0)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, 1, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtm),
            "l"(a), "l"(b), "r"(idesc)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, 1, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtm),
            "l"(a), "l"(b), "r"(idesc)
            : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(b))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_zero8(uint32_t taddr) {
    const uint32_t z = 0;
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr), "r"(z)
                 : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
            dst),
        "l"((uint64_t)map), "r"(saddr(bar)), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}

__device__ __forceinline__ float tf32_rna(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

// the work item idx (member, channel block, run of tiles, strip): strips of 16 columns of a member's box, split
// vertically in runs of tpi 16-row tiles
struct Item {
    int k, zb, sx, t0, nt, ntx;
    bool valid;
};
__device__ __forceinline__ Item item_of(const TcArgs &a, int idx) {
    Item it;
    it.sx = idx % a.ntxg;
    int rest = idx / a.ntxg;
    const int sg = rest % a.nsy;
    rest /= a.nsy;
    it.zb = rest % a.nzb;
    it.k = rest / a.nzb;
    const MemberDev &M = a.mem[it.k];
    it.ntx = (M.bx + TC_X - 1) / TC_X;
    const int nty = (M.by + TC_X - 1) / TC_X;
    it.t0 = sg * a.tpi;
    it.nt = min(a.tpi, nty - it.t0);
    it.valid = it.sx < it.ntx && it.nt > 0;
    return it;
}

// (warp-wide) bit i set: tile t0 + i of the item takes member 0's sums (a member computed as a difference from
// member 0 whose tile's input lies wholly in member 0's deposit tiles); with eg >= 0 the lane also writes the
// reduction's sentinel (-1) into that epilogue warp's partial pair of the tile
__device__ __forceinline__ unsigned skip_mask(const TcArgs &a, const Item &it, int lane, int eg) {
    bool sk = false;
    if (a.ts.tsrc && it.k != 0 && !a.smoothed && lane < it.nt) {
        const MemberDev &M = a.mem[it.k];
        const int ty = it.t0 + lane, x0 = it.sx * TC_X;
        const int ya = max(ty * TC_X - a.hy, 0), yb = min(ty * TC_X - a.hy + TC_X + a.ky - 1, M.by) - 1;
        const int xa = max(x0 - a.hx, 0), xb = min(x0 - a.hx + a.wused, M.bx) - 1;
        sk = yb >= ya && xb >= xa;
        for (int yt = ya >> a.ts.shy; yt <= (yb >> a.ts.shy) && sk; yt++)
            for (int xt = xa >> a.ts.shx; xt <= (xb >> a.ts.shx); xt++)
                if (__ldg(&a.ts.tsrc[M.tile_off + yt * M.ntx + xt]) != 0) { sk = false; break; }
        if (sk && eg >= 0 && a.do_resid) {
            double *p = a.partial +
                        2 * ((size_t)it.k * a.npart + ((size_t)(ty * it.ntx + it.sx) * a.nzb + it.zb) * EPW + eg);
            p[0] = -1.0;
            p[1] = 0.0;
        }
    }
    return __ballot_sync(0xffffffffu, sk);
}

// the runs of computed tiles [ta, tb) of an item (skip: bit i = tile i taken from member 0)
__device__ __forceinline__ bool next_run(unsigned skip, int nt, int &i, int &ta, int &tb) {
    while (i < nt && ((skip >> i) & 1)) i++;
    if (i >= nt) return false;
    ta = i;
    while (i < nt && !((skip >> i) & 1)) i++;
    tb = i;
    return true;
}

template <int V, int KP>
__global__ void __launch_bounds__(TC_THREADS, 1) k_conv_tc(const __grid_constant__ TcArgs a) {
    extern __shared__ uint8_t smraw[];
    // (aligned by an offset on the shared pointer itself: a pointer rebuilt from an integer would lose its address
    // space, and every access through it would be a generic load or store)
    uint8_t *sm = smraw + ((1024u - (saddr(smraw) & 1023u)) & 1023u);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *fst = sm;                                       // NFS x fstage: input rows, float32 [px][128]
    uint8_t *ast = fst + NFS * a.fstage;                     // NAS x (hi, lo) operand stages
    uint8_t *bsm = ast + NAS * a.astage;                     // B hi, B lo
    uint8_t *dst_ = bsm + ((a.bbytes + 127) & ~127);         // NDS x data rows, float32 [16 px][128]
    uint64_t *bars = (uint64_t *)(dst_ + NDS * DBOX_BYTES);
    uint64_t *full_f = bars, *empty_f = full_f + NFS, *full_a = empty_f + NFS, *empty_a = full_a + NAS;
    uint64_t *full_d = empty_a + NAS, *empty_d = full_d + NDS;
    uint64_t *ready = empty_d + NDS, *freeb = ready + TC_RING, *fin = freeb + TC_RING;
    uint64_t *itq_full = fin + 1, *itq_empty = itq_full + ITQ;
    int *misc = (int *)(itq_empty + ITQ);
    volatile int *abort_flag = misc;                         // [0]
    volatile uint32_t *tmem_hold = (volatile uint32_t *)(misc + 1);
    volatile uint8_t *rowflag = (volatile uint8_t *)(misc + 2);   // NAS x 8 bytes (per splitting warp)
    volatile int *itq = misc + 8;                                 // ITQ work items

    if (threadIdx.x == 0) {
        for (int i = 0; i < NFS; i++) { mbar_init(&full_f[i], 1); mbar_init(&empty_f[i], 8); }
        for (int i = 0; i < NAS; i++) { mbar_init(&full_a[i], 8); mbar_init(&empty_a[i], 1); }
        for (int i = 0; i < NDS; i++) { mbar_init(&full_d[i], 1); mbar_init(&empty_d[i], EPW); }
        for (int i = 0; i < TC_RING; i++) { mbar_init(&ready[i], 1); mbar_init(&freeb[i], EPW); }
        mbar_init(fin, 1);
        for (int i = 0; i < ITQ; i++) { mbar_init(&itq_full[i], 1); mbar_init(&itq_empty[i], TC_THREADS / 32 - 1); }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // B (hi, lo) into shared memory
    for (int i = threadIdx.x; i < a.bbytes / 16; i += TC_THREADS) ((uint4 *)bsm)[i] = __ldg(&a.bimg[i]);
    fence_async_smem();
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         saddr((const void *)tmem_hold)),
                     "r"(TC_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tmem_hold;
    if (warp >= 10 && warp < 10 + EPW) {
        // zero accumulators: every MMA accumulates
        const uint32_t tl = tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(((warp - 10) >> 2) * EPC);
        for (int c = 0; c < TC_COLS; c += TC_X) tmem_zero8(tl + c);
        tmem_wait_st();
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();

    int *err = a.err;
    const int ky = a.ky, hy = a.hy;
    const int nitems = a.nitems;
    // The CTA's work items, taken one at a time from the launch's counter (the CTAs that finish early take more:
    // the items' costs differ, e.g. the tiles a member shares with member 0 are skipped): warp 0 takes item q and
    // puts it in slot q mod ITQ of a ring, the other 18 warps read the slots in order (item -1: no more). Warp-uniform.
    auto next_item = [&](uint32_t q, bool &ok) -> int {
        int idx = -1;
        if (lane == 0 && ok) {
            const int sl = (int)(q % ITQ);
            if (warp == 0) {
                if (q >= ITQ) ok = mbar_wait(&itq_empty[sl], ((q / ITQ) - 1) & 1, abort_flag, err);
                if (ok) {
                    const int v = atomicAdd(a.queue, 1);
                    idx = v < nitems ? v : -1;
                    itq[sl] = idx;
                    mbar_arrive(&itq_full[sl]);
                }
            } else {
                ok = mbar_wait(&itq_full[sl], (q / ITQ) & 1, abort_flag, err);
                if (ok) {
                    idx = itq[sl];
                    mbar_arrive(&itq_empty[sl]);
                }
            }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        return ok ? idx : -1;
    };
    if (warp == 0) {
        // ---------------------------------------------------------------- TMA: input rows of the model
        uint32_t gf = 0;
        bool ok = true;
        for (uint32_t q = 0; ok; q++) {
            const int idx = next_item(q, ok);
            if (idx < 0) break;
            const Item it = item_of(a, idx);
            if (!it.valid) continue;
            const unsigned skip = skip_mask(a, it, lane, -1);
            if (lane == 0) {
                const MemberDev &M = a.mem[it.k];
                const bool TS = a.ts.tsrc != nullptr;
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"((uint64_t)&a.maps[it.k])
                             : "memory");
                if (TS)
                    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"((uint64_t)&a.maps[0])
                                 : "memory");
                const int xs = it.sx * TC_X - a.hx - a.dx;
                int i = 0, ta, tb;
                while (ok && next_run(skip, it.nt, i, ta, tb)) {
                    const int ylo = (it.t0 + ta) * TC_X;
                    const int nout = min((it.t0 + tb) * TC_X, M.by) - ylo;
                    const int nin = nout + ky - 1;
                    for (int r = 0; r < nin; r++, gf++) {
                        const int s = gf % NFS;
                        if (gf >= NFS && !(ok = mbar_wait(&empty_f[s], ((gf / NFS) - 1) & 1, abort_flag, err))) break;
                        const int yy = ylo - hy + r;
                        mbar_expect(&full_f[s], a.nbox * BOX_BYTES);
                        const uint32_t dst = saddr(fst + s * a.fstage);
                        for (int b = 0; b < a.nbox; b++) {
                            const int xx = xs + BOX_PX * b;
                            int src = it.k;
                            if (TS && yy >= 0 && yy < M.by && xx >= 0 && xx < M.bx)
                                src = __ldg(&a.ts.tsrc[M.tile_off + (yy >> a.ts.shy) * M.ntx + (xx >> a.ts.shx)]);
                            tma_load3(dst + b * BOX_BYTES, &a.maps[src], it.zb * TC_M, xx, yy, &full_f[s]);
                        }
                    }
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
        }
        // copies in flight (only after an early stop): the last stages issued, bounded waits
        if (lane == 0)
            for (uint32_t j = 0; j < NFS && j < gf; j++) {
                const uint32_t q = gf - 1 - j;
                mbar_wait(&full_f[q % NFS], (q / NFS) & 1, abort_flag, err);
            }
    } else if (warp == 10 + EPW) {
        // ---------------------------------------------------------------- TMA: data rows of the residual
        uint32_t gd = 0;
        bool ok = true;
        for (uint32_t q = 0; ok; q++) {
            const int idx = next_item(q, ok);
            if (idx < 0) break;
            const Item it = item_of(a, idx);
            if (!it.valid) continue;
            const unsigned skip = skip_mask(a, it, lane, -1);
            if (lane == 0 && a.do_resid) {
                const MemberDev &M = a.mem[it.k];
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                                 (uint64_t)&a.dmaps[it.k])
                             : "memory");
                int i = 0, ta, tb;
                while (ok && next_run(skip, it.nt, i, ta, tb)) {
                    const int ylo = (it.t0 + ta) * TC_X;
                    const int nout = min((it.t0 + tb) * TC_X, M.by) - ylo;
                    for (int oy = 0; oy < nout; oy++, gd++) {
                        const int s = gd % NDS;
                        if (gd >= NDS && !(ok = mbar_wait(&empty_d[s], ((gd / NDS) - 1) & 1, abort_flag, err))) break;
                        mbar_expect(&full_d[s], DBOX_BYTES);
                        tma_load3(saddr(dst_ + s * DBOX_BYTES), &a.dmaps[it.k], it.zb * TC_M, it.sx * TC_X + M.blo0,
                                  ylo + oy + M.blo1, &full_d[s]);
                    }
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
        }
        if (lane == 0)
            for (uint32_t j = 0; j < NDS && j < gd; j++) {
                const uint32_t q = gd - 1 - j;
                mbar_wait(&full_d[q % NDS], (q / NDS) & 1, abort_flag, err);
            }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer
        const uint32_t idesc0 = (1u << 4) | ((V == 0 ? 1u : 2u) << 7) | ((V == 0 ? 1u : 2u) << 10) |
                                ((uint32_t)(TC_M >> 4) << 24);
        const int nks = a.nks;                               // K steps of 32 bytes
        constexpr int KSMAX = V == 0 ? KP / 16 : KP / 8;
        uint32_t ga = 0, vbase = 0;
        bool ok = true;
        // the descriptors of the first operand stage and of B, advanced by adding address offsets (the descriptor's
        // low field is the shared-memory address / 16; every address stays below 256 KB, so nothing carries out)
        const uint64_t dA0 = sdesc(saddr(ast), 128, a.sbo_a), dB0 = sdesc(saddr(bsm), 128, a.sbo_b);
        const uint64_t astg16 = a.astage >> 4, aop16 = a.aop >> 4, bop16 = a.bop >> 4, sbob16 = a.sbo_b >> 4;
        for (uint32_t q = 0; ok; q++) {
            const int idx = next_item(q, ok);
            if (idx < 0) break;
            const Item it = item_of(a, idx);
            if (!it.valid) continue;
            const unsigned skip = skip_mask(a, it, lane, -1);
            if (lane == 0) {
                const int mby = a.mem[it.k].by;
                int i = 0, ta, tb;
                while (ok && next_run(skip, it.nt, i, ta, tb)) {
                    const int ylo = (it.t0 + ta) * TC_X;
                    const int nout = min((it.t0 + tb) * TC_X, mby) - ylo;
                    const int nin = nout + ky - 1;
                    for (int r = 0; r < nin; r++, ga++) {
                        const int sa = ga % NAS;
                        if (!(ok = mbar_wait(&full_a[sa], (ga / NAS) & 1, abort_flag, err))) break;
                        tc_fence_after();
                        if (r < nout) {
                            const uint32_t v = vbase + r;
                            if (v >= TC_RING) {
                                if (!(ok = mbar_wait(&freeb[v % TC_RING], ((v / TC_RING) - 1) & 1, abort_flag, err)))
                                    break;
                                tc_fence_after();
                            }
                        }
                        const int lo = max(0, r - ky + 1), hi = min(r, nout - 1);
                        const bool nzr = *(volatile const uint64_t *)(rowflag + sa * 8) != 0;
                        if (nzr && lo <= hi) {
                            const uint64_t dA = dA0 + (uint64_t)sa * astg16;
                            for (int o = lo; o <= hi;) {
                                const int slot = (int)((vbase + o) % TC_RING);
                                const int n = min(min(hi - o + 1, TC_RING - slot), 256 / TC_X);
                                const int jb = ky - 1 - (r - o);
                                const uint32_t idesc = idesc0 | ((uint32_t)((TC_X * n) >> 3) << 17);
                                const uint32_t dtm = tbase + (uint32_t)(slot * TC_X);
                                const uint64_t dB = dB0 + (uint64_t)(jb * 2) * sbob16;
#pragma unroll
                                for (int p = 0; p < 3; p++) {
                                    const uint64_t da = dA + (p == 2 ? aop16 : 0), db = dB + (p == 1 ? bop16 : 0);
#pragma unroll
                                    for (int ks = 0; ks < KSMAX; ks++)
                                        if (ks < nks) mma<V>(dtm, da + 16 * ks, db + 16 * ks, idesc);
                                }
                                o += n;
                            }
                        }
                        mma_commit(&empty_a[sa]);
                        const int done = r - ky + 1;
                        if (done >= 0 && done < nout) mma_commit(&ready[(vbase + done) % TC_RING]);
                    }
                    vbase += nout;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
        }
        if (lane == 0) {
            // every MMA issued has completed before the accumulators are freed
            mma_commit(fin);
            mbar_wait(fin, 0, abort_flag, err);
        }
    } else if (warp < 10) {
        // ---------------------------------------------------------------- operand split (warps 2-9)
        // two warps per group of 32 channels, each splitting half of the row's pixels
        const int sw = warp - 2, cg = sw & 3, half = sw >> 2, ch = cg * 32 + lane;
        uint32_t gf = 0, ga = 0;
        bool ok = true;
        for (uint32_t q = 0; ok; q++) {
            const int idx = next_item(q, ok);
            if (idx < 0) break;
            const Item it = item_of(a, idx);
            if (!it.valid) continue;
            const unsigned skip = skip_mask(a, it, lane, -1);
            const int mby = a.mem[it.k].by;
            const bool zin = it.zb * TC_M + ch < a.nz;
            const int wused = zin ? a.wused : 0;
            int i = 0, ta, tb;
            while (ok && next_run(skip, it.nt, i, ta, tb)) {
                const int ylo = (it.t0 + ta) * TC_X;
                const int nout = min((it.t0 + tb) * TC_X, mby) - ylo;
                const int nin = nout + ky - 1;
                for (int r = 0; r < nin; r++, gf++, ga++) {
                    const int sf = gf % NFS, sa = ga % NAS;
                    ok = mbar_wait(&full_f[sf], (gf / NFS) & 1, abort_flag, err);
                    if (ok && ga >= NAS) ok = mbar_wait(&empty_a[sa], ((ga / NAS) - 1) & 1, abort_flag, err);
                    if (!(ok = __all_sync(0xffffffffu, ok))) break;
                    const float *F = (const float *)(fst + sf * a.fstage) + (size_t)a.dx * TC_M + ch;
                    uint8_t *Ah = ast + sa * a.astage + (ch >> 3) * a.sbo_a + (ch & 7) * 16;
                    uint8_t *Al = Ah + a.aop;
                    uint32_t bits = 0;
                    if (V == 0) {
                        constexpr int NC = KP / 16;                  // 8-pixel chunks of this warp's half
#pragma unroll
                        for (int c = 0; c < NC; c++) {
                            const int kc = half * NC + c;
                            float v[8];
#pragma unroll
                            for (int e = 0; e < 8; e++) {
                                const int kk = kc * 8 + e;
                                v[e] = kk < wused ? F[kk * TC_M] : 0.0f;
                                bits |= __float_as_uint(v[e]);
                            }
                            uint32_t h[4], l[4];
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                const __nv_bfloat162 hb = __float22bfloat162_rn(make_float2(v[2 * e], v[2 * e + 1]));
                                const float2 hf = __bfloat1622float2(hb);
                                const __nv_bfloat162 lb =
                                    __float22bfloat162_rn(make_float2(v[2 * e] - hf.x, v[2 * e + 1] - hf.y));
                                h[e] = *(const uint32_t *)&hb;
                                l[e] = *(const uint32_t *)&lb;
                            }
                            *(uint4 *)(Ah + kc * 128) = make_uint4(h[0], h[1], h[2], h[3]);
                            *(uint4 *)(Al + kc * 128) = make_uint4(l[0], l[1], l[2], l[3]);
                        }
                    } else {
                        constexpr int NC = KP / 8;                   // 4-pixel chunks of this warp's half
#pragma unroll
                        for (int c = 0; c < NC; c++) {
                            const int kc = half * NC + c;
                            if (kc * 4 >= a.nks * 8) break;          // (beyond the MMAs' K: never read)
                            float v[4];
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                const int kk = kc * 4 + e;
                                v[e] = kk < wused ? F[kk * TC_M] : 0.0f;
                                bits |= __float_as_uint(v[e]);
                            }
                            float4 h, l;
                            h.x = tf32_rna(v[0]); h.y = tf32_rna(v[1]); h.z = tf32_rna(v[2]); h.w = tf32_rna(v[3]);
                            l.x = v[0] - h.x; l.y = v[1] - h.y; l.z = v[2] - h.z; l.w = v[3] - h.w;
                            *(float4 *)(Ah + kc * 128) = h;
                            *(float4 *)(Al + kc * 128) = l;
                        }
                    }
                    fence_async_smem();
                    const unsigned bal = __ballot_sync(0xffffffffu, (bits << 1) != 0);   // (any value but +-0)
                    if (lane == 0) {
                        rowflag[sa * 8 + sw] = bal != 0;
                        mbar_arrive(&full_a[sa]);
                        mbar_arrive(&empty_f[sf]);
                    }
                    __syncwarp();
                }
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue (warps 10-17)
        // warp w: TMEM lanes (channels) 32 (w mod 4) + lane, columns ex0 .. ex0 + 7 of each output row
        const int ep = warp - 10, eg = warp & 3, ch = eg * 32 + lane, ex0 = (ep >> 2) * EPC;
        const uint32_t tl = tbase + ((uint32_t)(eg * 32) << 16) + (uint32_t)ex0;
        const float scale = (float)a.g.scalefactor;
        uint32_t vbase = 0, gd = 0;
        bool ok = true;
        for (uint32_t q = 0; ok; q++) {
            const int idx = next_item(q, ok);
            if (idx < 0) break;
            const Item it = item_of(a, idx);
            if (!it.valid) continue;
            const unsigned skip = skip_mask(a, it, lane, ep);
            const MemberDev &Mg = a.mem[it.k];
            const int mbx = Mg.bx, mby = Mg.by;
            const float sig2 = Mg.sigma2f, eps2 = Mg.eps2f;
            const bool fr = Mg.eps2 > 0.0;
            const int z = it.zb * TC_M + ch;
            const bool zok = z < a.nz;
            const int x0 = it.sx * TC_X + ex0;
            float ss = 0.0f, lg = 0.0f;
            int i = 0, ta, tb;
            while (ok && next_run(skip, it.nt, i, ta, tb)) {
                const int ylo = (it.t0 + ta) * TC_X;
                const int nout = min((it.t0 + tb) * TC_X, mby) - ylo;
                for (int oy = 0; oy < nout; oy++) {
                    const int y = ylo + oy;
                    const uint32_t v = vbase + oy;
                    ok = mbar_wait(&ready[v % TC_RING], (v / TC_RING) & 1, abort_flag, err);
                    if (ok && a.do_resid) ok = mbar_wait(&full_d[gd % NDS], (gd / NDS) & 1, abort_flag, err);
                    if (!(ok = __all_sync(0xffffffffu, ok))) break;
                    tc_fence_after();
                    float acc[EPC];
                    const uint32_t col = (v % TC_RING) * TC_X;
                    tmem_ld8(tl + col, acc);
                    tmem_zero8(tl + col);
                    tmem_wait_st();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&freeb[v % TC_RING]);
                    const float *D = (const float *)(dst_ + (gd % NDS) * DBOX_BYTES) + ex0 * TC_M + ch;
                    if (zok && !a.smoothed && a.do_resid && a.do_conv == 1 && !fr) {
                        // the likelihood's case: threshold, scale and the sum of squares only
                        const int nxv = min(EPC, mbx - x0);
                        float s2 = 0.0f;
#pragma unroll
                        for (int x = 0; x < EPC; x++) {
                            float m = acc[x];
                            m = m < 1.0e-12f ? 0.0f : m * scale;
                            const float d = D[x * TC_M];
                            const float rr = d - m;
                            s2 += (x < nxv && d == d) ? rr * rr : 0.0f;
                        }
                        ss += s2;
                    } else if (zok) {
#pragma unroll
                        for (int x = 0; x < EPC; x++) {
                            const int xx = x0 + x;
                            if (xx >= mbx) continue;
                            float m = acc[x];
                            if (a.do_conv == 1) m = m < 1.0e-12f ? 0.0f : m * scale;
                            if (a.smoothed)
                                a.smoothed[(size_t)it.k * a.mstride + ((size_t)y * mbx + xx) * a.nz + z] = m;
                            if (a.do_resid) {
                                const float d = D[x * TC_M];
                                if (d == d) {
                                    const float rr = d - m;
                                    if (fr && m != 0.0f) {
                                        const float var = sig2 + eps2 * m * m;
                                        ss += rr * rr / var;
                                        lg += logf(var / sig2);
                                    } else if (fr) {
                                        ss += rr * rr / sig2;
                                    } else {
                                        ss += rr * rr;
                                    }
                                }
                            }
                        }
                    }
                    if (a.do_resid) {
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&empty_d[gd % NDS]);
                        gd++;
                    }
                    if (((y & (TC_X - 1)) == TC_X - 1) || oy == nout - 1) {
                        // the tile's sums of this warp's 32 channels, float64 in a fixed order (one partial pair
                        // per tile, channel block and epilogue warp: the reduction adds them in index order)
                        double ds = (double)ss, dl = (double)lg;
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            ds += __shfl_down_sync(0xffffffffu, ds, o);
                            dl += __shfl_down_sync(0xffffffffu, dl, o);
                        }
                        if (lane == 0 && a.do_resid) {
                            double *p = a.partial + 2 * ((size_t)it.k * a.npart +
                                                         ((size_t)((y >> 4) * it.ntx + it.sx) * a.nzb + it.zb) * EPW +
                                                         ep);
                            p[0] = ds;
                            p[1] = dl;
                        }
                        ss = 0.0f;
                        lg = 0.0f;
                    }
                }
                vbase += nout;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TC_COLS) : "memory");
    }
}

// ---------------------------------------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    }
    return fn;
}

uint16_t bf16_bits(double x) {
    // round to nearest even of the float32 value (x is first rounded to float32)
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);
    const uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(r >> 16);
}
double bf16_value(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
uint32_t tf32_bits(double x) {
    // round to nearest (ties away) to a 10-bit mantissa, as cvt.rna.tf32.f32
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return u & 0xffffe000u;
    return (u + 0x1000u) & 0xffffe000u;
}
double tf32_value(uint32_t b) {
    float f;
    memcpy(&f, &b, 4);
    return f;
}

int kp_of(int kx) { return (TC_X + kx - 1) <= 32 ? 32 : ((TC_X + kx - 1) <= 48 ? 48 : 0); }

struct TcLayout {
    int kp, nbox, dx, wused, nks;
    unsigned fstage, astage, aop, bop, sbo_a, sbo_b, bbytes;
    size_t smem;
};

TcLayout tc_layout(int variant, int ky, int kx) {
    TcLayout L{};
    const int hx = kx / 2;
    L.kp = kp_of(kx);
    L.wused = TC_X + kx - 1;
    L.dx = ((-hx) % BOX_PX + BOX_PX) % BOX_PX;
    L.nbox = (L.dx + L.wused + BOX_PX - 1) / BOX_PX;
    const int es = variant == 1 ? 2 : 4;          // bf16 or tf32 bytes
    const int chunk = 16 / es;                    // elements of a core-matrix row
    L.sbo_a = (unsigned)(L.kp / chunk) * 128;     // 8 channels: KP elements of each
    L.aop = (unsigned)TC_M * L.kp * es;           // hi -> lo
    L.astage = 2 * L.aop;
    L.sbo_b = L.sbo_a;
    L.bop = (unsigned)(TC_X * ky) * L.kp * es;
    L.bbytes = 2 * L.bop;
    L.fstage = (unsigned)L.nbox * BOX_BYTES;
    // K steps of 32 bytes that cover the used pixels (16 bf16 or 8 tf32 each)
    L.nks = variant == 1 ? (L.wused + 15) / 16 : (L.wused + 7) / 8;
    const size_t bars = (2 * NFS + 2 * NAS + 2 * NDS + 2 * TC_RING + 1 + 2 * ITQ) * 8;
    L.smem = 1024 + NFS * (size_t)L.fstage + NAS * (size_t)L.astage + ((L.bbytes + 127) & ~127u) +
             NDS * (size_t)DBOX_BYTES + bars + 32 * 4;
    return L;
}

}  // namespace

// variant 1 (bf16x3) or 2 (tf32x3): whether the tensor-core kernel takes a kernel of ky x kx taps on nz channels
bool conv_tc_supported(int variant, int ky, int kx, int nz) {
    if (variant != 1 && variant != 2) return false;
    if (ky < 1 || ky > TC_RING || !kp_of(kx) || (nz & 3)) return false;
    return tc_layout(variant, ky, kx).smem <= 227 * 1024 && encode_fn() != nullptr;
}

// B (hi, then lo) of the kernel k (ky, kx) in the operand layout of conv_tc
void conv_tc_image(int variant, const double *kern, int ky, int kx, std::vector<uint8_t> &img) {
    const TcLayout L = tc_layout(variant, ky, kx);
    img.assign(L.bbytes, 0);
    const int es = variant == 1 ? 2 : 4, chunk = 16 / es;
    const int N = TC_X * ky;
    for (int n = 0; n < N; n++) {
        const int j = n / TC_X, ox = n % TC_X;
        const int ar = ky - 1 - j;                       // kernel row of the flipped kernel
        for (int kk = 0; kk < L.kp; kk++) {
            const int b = kk - ox;
            double t = 0.0;
            if (b >= 0 && b < kx) t = kern[(ky - 1 - ar) * kx + (kx - 1 - b)];   // kf[ar][b]
            const size_t off = (size_t)(n / 8) * L.sbo_b + (size_t)(kk / chunk) * 128 + (size_t)(n % 8) * 16 +
                               (size_t)(kk % chunk) * es;
            if (variant == 1) {
                const uint16_t h = bf16_bits(t), l = bf16_bits(t - bf16_value(h));
                memcpy(&img[off], &h, 2);
                memcpy(&img[L.bop + off], &l, 2);
            } else {
                const uint32_t h = tf32_bits(t);
                const float l = (float)(t - tf32_value(h));
                memcpy(&img[off], &h, 4);
                memcpy(&img[L.bop + off], &l, 4);
            }
        }
    }
}

// two tensor maps per member: maps[k] its model (by, bx, nz) float32 at model + k mstride (boxes of 128 channels x
// 8 pixels x 1 row), maps[nb + k] the data it is compared with, deff (ny, nx, nz) float32 (boxes of 128 channels x 16
// pixels x 1 row); false if the driver refuses one
bool conv_tc_maps(const MemberDev *mem_host, int nb, const float *model, long long mstride, int nz, int nx, int ny,
                  std::vector<CUtensorMap> &maps) {
    auto fn = encode_fn();
    if (!fn) return false;
    maps.resize(2 * (size_t)nb);
    cuuint32_t es[3] = {1, 1, 1};
    for (int k = 0; k < nb; k++) {
        const MemberDev &M = mem_host[k];
        const cuuint64_t bx = M.bx > 0 ? M.bx : 1, by = M.by > 0 ? M.by : 1;
        cuuint64_t dims[3] = {(cuuint64_t)nz, bx, by};
        cuuint64_t strides[2] = {(cuuint64_t)nz * 4, (cuuint64_t)nz * 4 * bx};
        cuuint32_t box[3] = {TC_M, BOX_PX, 1};
        CUresult r = fn(&maps[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)(model + (size_t)k * mstride), dims,
                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
        cuuint64_t ddims[3] = {(cuuint64_t)nz, (cuuint64_t)nx, (cuuint64_t)ny};
        cuuint64_t dstr[2] = {(cuuint64_t)nz * 4, (cuuint64_t)nz * 4 * nx};
        cuuint32_t dbox[3] = {TC_M, TC_X, 1};
        if (!M.deff) {
            maps[nb + k] = maps[k];
            continue;
        }
        r = fn(&maps[nb + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)M.deff, ddims, dstr, dbox, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
    }
    return true;
}

int conv_tc_npart(const MemberDev *mem_host, int nb, int nz) {
    int maxt = 0;
    for (int k = 0; k < nb; k++)
        maxt = max(maxt, ((mem_host[k].bx + TC_X - 1) / TC_X) * ((mem_host[k].by + TC_X - 1) / TC_X));
    return maxt * ((nz + TC_M - 1) / TC_M) * EPW;
}

// the convolution + residual of a batch on the tensor cores (partial sums as launch_conv_resid, npart =
// conv_tc_npart; the caller zeroes them first). maps: device copies of conv_tc_maps; bimg: conv_tc_image.
void launch_conv_tc(cudaStream_t s, int variant, const GridDev &g, const MemberDev *mem, const MemberDev *mem_host,
                    int nb, const CUtensorMap *maps, const void *bimg, long long mstride, int nz, int ky, int kx,
                    float *smoothed, int do_conv, int do_resid, double *partial, int npart, TileSrc ts, int *err,
                    int *queue) {
    const TcLayout L = tc_layout(variant, ky, kx);
    int ntxg = 0, ntyg = 0;
    for (int k = 0; k < nb; k++) {
        ntxg = max(ntxg, (mem_host[k].bx + TC_X - 1) / TC_X);
        ntyg = max(ntyg, (mem_host[k].by + TC_X - 1) / TC_X);
    }
    if (nb == 0 || ntxg == 0 || ntyg == 0) return;
    // persistent CTAs, one per SM; work items: strips split in runs of at most TC_MAX_TILES tiles, at least four
    // items per CTA where the batch allows
    int nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
    const int nzb = (nz + TC_M - 1) / TC_M;
    int nsy = 1;
    while (nsy < ntyg && (long long)nb * nzb * ntxg * nsy < 4LL * nsm) nsy++;
    int tpi = (ntyg + nsy - 1) / nsy;
    if (tpi > TC_MAX_TILES) tpi = TC_MAX_TILES;
    nsy = (ntyg + tpi - 1) / tpi;
    TcArgs a;
    a.g = g;
    a.mem = mem;
    a.maps = maps;
    a.dmaps = maps + nb;
    a.bimg = (const uint4 *)bimg;
    a.bbytes = (int)L.bbytes;
    a.ky = ky; a.kx = kx; a.hy = ky / 2; a.hx = kx / 2;
    a.wused = L.wused; a.dx = L.dx; a.nbox = L.nbox;
    a.nz = nz; a.nzb = nzb;
    a.tpi = tpi; a.nsy = nsy; a.ntxg = ntxg;
    a.nitems = nb * nzb * nsy * ntxg;
    a.nks = L.nks;
    a.do_conv = do_conv; a.do_resid = do_resid;
    a.smoothed = smoothed;
    a.mstride = mstride;
    a.partial = partial;
    a.npart = npart;
    a.ts = ts;
    a.err = err;
    a.queue = queue;
    a.fstage = L.fstage; a.astage = L.astage; a.aop = L.aop; a.bop = L.bop; a.sbo_a = L.sbo_a; a.sbo_b = L.sbo_b;
    dim3 grid(std::min(a.nitems, nsm));
    cudaMemsetAsync(queue, 0, sizeof(int), s);
#define TC_CASE(V, KP)                                                                                           \
    {                                                                                                            \
        static size_t configured = 0;                                                                            \
        if (L.smem > configured) {                                                                               \
            cudaFuncSetAttribute(k_conv_tc<V, KP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);    \
            configured = L.smem;                                                                                 \
        }                                                                                                        \
        k_conv_tc<V, KP><<<grid, TC_THREADS, L.smem, s>>>(a);                                                    \
    }
    if (variant == 1) {
        if (L.kp == 32) TC_CASE(0, 32) else TC_CASE(0, 48)
    } else {
        if (L.kp == 32) TC_CASE(1, 32) else TC_CASE(1, 48)
    }
#undef TC_CASE
}
