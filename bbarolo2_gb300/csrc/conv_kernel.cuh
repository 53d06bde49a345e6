// The beam convolution + residual kernel (k_conv_resid) and its launch, shared by conv.cu (models without a
// tile table) and conv_table.cu (MC models with tiles shared with member 0): two translation units, compiled
// in parallel.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace {


constexpr int TO = 16;        // output tile width (pixels); tile height 16 (ZB = 32) or 32 (ZB = 16)
constexpr int NW = 8;         // warps per CTA: two output rows of each half-warp group

// cp.async of 16 (or 4) bytes into shared memory; src_size 0 fills the destination with zeros (the halo
// outside the box), without reading the source.
__device__ __forceinline__ void cp_async_zfill16(float *dst, const float *src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_zfill4(float *dst, const float *src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 4 : 0) : "memory");
}

// TS: the model of a pixel is looked up in a tile table (TileSrc): the table entries of the CTA's input region
// are staged in shared memory, and when they all name one member the tile is read from that member's model.
#define TS_MAX 256
template <int KXW, int ZB, bool TS>
__global__ void __launch_bounds__(256, 2) k_conv_resid(GridDev g, const MemberDev *__restrict__ mem,
                                                       const float *__restrict__ model, long long mstride, int nz,
                                                       const float *__restrict__ taps, int ky, int kx,
                                                       float *__restrict__ smoothed, int do_conv, int do_resid,
                                                       double *__restrict__ partial, int npart, TileSrc ts) {
    extern __shared__ float sm[];
    constexpr int W = TO + KXW - 1;
    constexpr int TOY = TO * (32 / ZB);     // tile rows: 32 / ZB groups of lanes, 16 rows each
    const int k = blockIdx.x;
    const MemberDev &M = mem[k];
    const int ntx = (M.bx + TO - 1) / TO, nty = (M.by + TOY - 1) / TOY;
    const int t = blockIdx.y, zb = blockIdx.z;
    const int nzb = gridDim.z;
    double *pout = partial + 2 * ((size_t)k * npart + (size_t)t * nzb + zb);
    if (t >= ntx * nty) {
        if (threadIdx.x == 0) { pout[0] = 0.0; pout[1] = 0.0; }
        return;
    }
    const int ky_eff = do_conv ? ky : 1, kx_eff = do_conv ? kx : 1;
    const int hy = ky_eff / 2, hx = kx_eff / 2;
    const int H = TOY + ky_eff - 1, ncol = TO + kx_eff - 1;
    float *S = sm;                          // H x W x ZB
    float *sk = sm + (size_t)H * W * ZB;    // ky x KXW taps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ch = lane % ZB, grp = lane / ZB;
    const int y0 = (t / ntx) * TOY, x0 = (t % ntx) * TO;
    const int z = zb * ZB + ch;
    const bool zok = z < nz;
    if (do_conv)
        for (int i = threadIdx.x; i < ky * KXW; i += blockDim.x) sk[i] = taps[i];
    const float *mk = model + (size_t)k * mstride;
    // the model of the pixel (yy, xx): the member's own, or, with a tile table, that of the member whose model
    // holds the pixel's deposit tile (member 0's for the tiles a member shares with it)
    __shared__ int tsm[TS ? TS_MAX : 1];
    int ty0r = 0, tx0r = 0, tnx = 1;
    bool uni = true;
    if (TS) {
        const int ya = max(y0 - hy, 0), yb = min(y0 - hy + H, M.by) - 1;
        const int xa = max(x0 - hx, 0), xb = min(x0 - hx + ncol, M.bx) - 1;
        ty0r = ya >> ts.shy;
        tx0r = xa >> ts.shx;
        const int tny = yb >= ya ? (yb >> ts.shy) - ty0r + 1 : 0;
        tnx = xb >= xa ? (xb >> ts.shx) - tx0r + 1 : 1;
        const int nt = min(tny * tnx, TS_MAX);
        int first = k;
        if (nt > 0) first = __ldg(&ts.tsrc[M.tile_off + ty0r * M.ntx + tx0r]);
        int diff = 0;
        for (int i = threadIdx.x; i < nt; i += blockDim.x) {
            const int v = __ldg(&ts.tsrc[M.tile_off + (ty0r + i / tnx) * M.ntx + tx0r + i % tnx]);
            tsm[i] = v;
            diff |= v != first;
        }
        uni = !__syncthreads_or(diff) && tny * tnx <= TS_MAX;
        if (uni) mk = model + (size_t)first * mstride;
        // the whole input region is member 0's model (a member computed as a difference from it, away from the
        // sub-rings that differ): the tile's sums are member 0's, taken by the reduction (sentinel -1: a sum of
        // squares is never negative)
        if (ts.kout) {
            // (the ring maps: such a tile keeps member 0's output, which the normal equations read there)
            const bool skip = uni && first == 0 && k != 0;
            if (zb == 0 && threadIdx.x == 0) ts.kout[(size_t)k * ts.kstride + t] = skip ? 0 : k;
            if (skip) {
                if (threadIdx.x == 0) { pout[0] = 0.0; pout[1] = 0.0; }
                return;
            }
        } else if (uni && first == 0 && k != 0 && !smoothed) {
            if (threadIdx.x == 0) { pout[0] = -1.0; pout[1] = 0.0; }
            return;
        }
    }
    auto src = [&](int yy, int xx) -> const float * {
        if (!TS || uni) return mk;
        const int i = ((yy >> ts.shy) - ty0r) * tnx + (xx >> ts.shx) - tx0r;
        return model + (size_t)(i < TS_MAX ? tsm[i] : __ldg(&ts.tsrc[M.tile_off + (yy >> ts.shy) * M.ntx +
                                                                       (xx >> ts.shx)])) * mstride;
    };
    // the input tile with its halo, asynchronously: 16-byte copies of 4 channels when the rows of channels are
    // 16-byte aligned (nz a multiple of 4), else 4-byte copies; zeros outside the box and past nz
    const bool vec = (nz & 3) == 0 && (((uintptr_t)mk) & 15) == 0;
    if (vec) {
        for (int c = threadIdx.x; c < H * W * (ZB / 4); c += blockDim.x) {
            const int q = c & (ZB / 4 - 1), rc = c / (ZB / 4);
            const int r = rc / W, col = rc - r * W;
            const int yy = y0 - hy + r, xx = x0 - hx + col, zz = zb * ZB + 4 * q;
            const bool ok = col < ncol && yy >= 0 && yy < M.by && xx >= 0 && xx < M.bx && zz < nz;
            cp_async_zfill16(S + (size_t)rc * ZB + 4 * q, ok ? src(yy, xx) + ((size_t)yy * M.bx + xx) * nz + zz : mk,
                             ok);
        }
    } else {
        for (int c = threadIdx.x; c < H * W * ZB; c += blockDim.x) {
            const int l = c & (ZB - 1), rc = c / ZB;
            const int r = rc / W, col = rc - r * W;
            const int yy = y0 - hy + r, xx = x0 - hx + col, zz = zb * ZB + l;
            const bool ok = col < ncol && yy >= 0 && yy < M.by && xx >= 0 && xx < M.bx && zz < nz;
            cp_async_zfill4(S + c, ok ? src(yy, xx) + ((size_t)yy * M.bx + xx) * nz + zz : mk, ok);
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    // the data of this thread's output voxels, loaded while the tile arrives
    const int ty0 = grp * 16 + warp * 2;
    float dv[2][TO];
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
        const int y = y0 + ty0 + rr;
#pragma unroll
        for (int x = 0; x < TO; x++) {
            const int xx = x0 + x;
            dv[rr][x] = (do_resid && zok && y < M.by && xx < M.bx)
                            ? __ldg(&M.deff[((size_t)(y + M.blo1) * g.nx + (xx + M.blo0)) * g.nz + z])
                            : 0.0f;
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    // all-zero input (empty channels, corners of the box): no convolution
    unsigned any = 0;
    if (vec) {
        for (int c = threadIdx.x; c < H * W * (ZB / 4); c += blockDim.x) {
            const uint4 v = *(const uint4 *)(S + (size_t)c * 4);
            any |= (v.x | v.y | v.z | v.w) << 1;
        }
    } else {
        for (int c = threadIdx.x; c < H * W * ZB; c += blockDim.x) any |= __float_as_uint(S[c]) << 1;
    }
    const int nonempty = __syncthreads_or(any != 0);
    float acc[2][TO];
#pragma unroll
    for (int rr = 0; rr < 2; rr++)
#pragma unroll
        for (int x = 0; x < TO; x++) acc[rr][x] = 0.0f;
    if (nonempty) {
        if (do_conv) {
            // input row ty0 + i feeds output row ty0 with kernel row i and output row ty0 + 1 with kernel row
            // i - 1: each input row is read from shared memory once (the sums run over the kernel rows in order)
            for (int i = 0; i <= ky; i++) {
                const float *row = S + (size_t)((ty0 + i) * W) * ZB + ch;
                float win[W];
#pragma unroll
                for (int j = 0; j < W; j++) win[j] = row[j * ZB];
                if (i < ky) {
#pragma unroll
                    for (int b = 0; b < KXW; b++) {
                        const float kv = sk[i * KXW + b];
#pragma unroll
                        for (int x = 0; x < TO; x++) acc[0][x] = fmaf(kv, win[x + b], acc[0][x]);
                    }
                }
                if (i > 0) {
#pragma unroll
                    for (int b = 0; b < KXW; b++) {
                        const float kv = sk[(i - 1) * KXW + b];
#pragma unroll
                        for (int x = 0; x < TO; x++) acc[1][x] = fmaf(kv, win[x + b], acc[1][x]);
                    }
                }
            }
        } else {
#pragma unroll
            for (int rr = 0; rr < 2; rr++) {
                const int ty = ty0 + rr;
#pragma unroll
                for (int x = 0; x < TO; x++) acc[rr][x] = S[(size_t)(ty * W + x) * ZB + ch];
            }
        }
    }
    // epilogue: threshold + scale (smoothed models only), residual
    const float scale = (float)g.scalefactor;
    float ss = 0.0f, lg = 0.0f;
    const bool fr = M.eps2 > 0.0;
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
        const int y = y0 + ty0 + rr;
        if (y >= M.by || !zok) continue;
#pragma unroll
        for (int x = 0; x < TO; x++) {
            const int xx = x0 + x;
            if (xx >= M.bx) continue;
            float m = acc[rr][x];
            if (do_conv == 1) m = m < 1.0e-12f ? 0.0f : m * scale;
            if (smoothed) smoothed[(size_t)k * mstride + ((size_t)y * M.bx + xx) * nz + z] = m;
            if (do_resid) {
                const float d = dv[rr][x];
                if (d == d) {
                    const float r = d - m;
                    if (fr && m != 0.0f) {
                        const float v = M.sigma2f + M.eps2f * m * m;
                        ss += r * r / v;
                        lg += logf(v / M.sigma2f);
                    } else if (fr) {
                        ss += r * r / M.sigma2f;
                    } else {
                        ss += r * r;
                    }
                }
            }
        }
    }
    // float64 reduction of the CTA's sums
    double ds = (double)ss, dl = (double)lg;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ds += __shfl_down_sync(0xffffffffu, ds, o);
        dl += __shfl_down_sync(0xffffffffu, dl, o);
    }
    __shared__ double red[2][NW];
    if (lane == 0) { red[0][warp] = ds; red[1][warp] = dl; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < NW; w++) { a += red[0][w]; b += red[1][w]; }
        pout[0] = a;
        pout[1] = b;
    }
}

template <int KXW, int ZB, bool TS>
void launch_t(cudaStream_t s, const GridDev &g, const MemberDev *mem, int nb, int maxt, int nzb, const float *model,
              long long mstride, int nz, const float *taps, int ky, int kx, float *smoothed, int do_conv,
              int do_resid, double *partial, int npart, TileSrc ts) {
    const int kye = do_conv ? ky : 1;
    constexpr int TOY = TO * (32 / ZB);
    size_t smem = (size_t)(TOY + kye - 1) * (TO + KXW - 1) * ZB * sizeof(float) + (size_t)ky * KXW * sizeof(float);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_conv_resid<KXW, ZB, TS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    dim3 grid(nb, maxt, nzb);
    k_conv_resid<KXW, ZB, TS><<<grid, 256, smem, s>>>(g, mem, model, mstride, nz, taps, ky, kx, smoothed, do_conv,
                                                 do_resid, partial, npart, ts);
}

}  // namespace
