// The beam convolution + residual for kernels wider than the shared-memory templates of k_conv_resid (widths
// above 31, or tiles above 220 KB): the "same" convolution of each channel plane of a member's box
// (bbarolo/smooth.py:145-165 FFTConvolver.__call__, any kernel size the reference accepts: sides below 512),
// the threshold and scale of bbarolo/galmod.py:1273-1283, and the masked residual of
// bbarolo/bayesian/likelihood.py:22-77. Same tiles, partial sums, tile-source table and outputs as k_conv_resid, so
// the reduction and every caller are shared; the input is read from global memory (L1/L2) instead of a staged
// tile, so any kernel fits.
//
// A CTA takes one conv tile (16 columns x TOY rows) of one member and one block of ZB channels; a thread one channel
// and two output rows of the tile, 16 columns each, in registers. For each kernel row a and each input column of
// the window, one load (the lanes of a warp read consecutive channels: 64 or 128 bytes) is multiplied into the
// outputs it feeds (b = column - output, 0 <= b < kx).

#include <cuda_runtime.h>

#include "kernels.h"

namespace {

constexpr int WTO = 16;     // tile columns (as k_conv_resid)

template <int ZB>
__global__ void __launch_bounds__(256) k_conv_wide(GridDev g, const MemberDev *__restrict__ mem,
                                                   const float *__restrict__ model, long long mstride, int nz,
                                                   const float *__restrict__ taps, int ky, int kx,
                                                   float *__restrict__ smoothed, int do_conv, int do_resid,
                                                   double *__restrict__ partial, int npart, TileSrc ts) {
    constexpr int TOY = WTO * (32 / ZB);
    const int k = blockIdx.x;
    const MemberDev &M = mem[k];
    const int ntx = (M.bx + WTO - 1) / WTO, nty = (M.by + TOY - 1) / TOY;
    const int t = blockIdx.y, zb = blockIdx.z;
    const int nzb = gridDim.z;
    double *pout = partial + 2 * ((size_t)k * npart + (size_t)t * nzb + zb);
    if (t >= ntx * nty) {
        if (threadIdx.x == 0) { pout[0] = 0.0; pout[1] = 0.0; }
        return;
    }
    // every tile of this member is computed from its own inputs (no tile takes member 0's sums)
    if (ts.kout && zb == 0 && threadIdx.x == 0) ts.kout[(size_t)k * ts.kstride + t] = k;
    const int hy = ky / 2, hx = kx / 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ch = lane % ZB, grp = lane / ZB;
    const int y0 = (t / ntx) * TOY, x0 = (t % ntx) * WTO;
    const int z = zb * ZB + ch;
    const bool zok = z < nz;
    const int ty0 = grp * 16 + warp * 2;
    const float *own = model + (size_t)k * mstride;
    float acc[2][WTO];
#pragma unroll
    for (int rr = 0; rr < 2; rr++)
#pragma unroll
        for (int j = 0; j < WTO; j++) acc[rr][j] = 0.0f;
    if (zok) {
        for (int rr = 0; rr < 2; rr++) {
            const int y = y0 + ty0 + rr;
            if (y >= M.by) break;
            for (int a = 0; a < ky; a++) {
                const int yy = y - hy + a;
                if (yy < 0 || yy >= M.by) continue;
                const float *kr = taps + (size_t)a * kx;
                for (int c = 0; c < WTO + kx - 1; c++) {
                    const int xx = x0 - hx + c;
                    if (xx < 0 || xx >= M.bx) continue;
                    const float *src = own;
                    if (ts.tsrc)
                        src = model + (size_t)__ldg(&ts.tsrc[M.tile_off + (yy >> ts.shy) * M.ntx + (xx >> ts.shx)]) *
                                          mstride;
                    const float v = __ldg(&src[((size_t)yy * M.bx + xx) * nz + z]);
                    if (v == 0.0f) continue;
#pragma unroll
                    for (int j = 0; j < WTO; j++) {
                        const int b = c - j;
                        if (b >= 0 && b < kx) acc[rr][j] = fmaf(__ldg(&kr[b]), v, acc[rr][j]);
                    }
                }
            }
        }
    }
    const float scale = (float)g.scalefactor;
    float ss = 0.0f, lg = 0.0f;
    const bool fr = M.eps2 > 0.0;
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
        const int y = y0 + ty0 + rr;
        if (y >= M.by || !zok) continue;
#pragma unroll
        for (int j = 0; j < WTO; j++) {
            const int xx = x0 + j;
            if (xx >= M.bx) continue;
            float m = acc[rr][j];
            if (do_conv == 1) m = m < 1.0e-12f ? 0.0f : m * scale;
            if (smoothed) smoothed[(size_t)k * mstride + ((size_t)y * M.bx + xx) * nz + z] = m;
            if (do_resid) {
                const float d = __ldg(&M.deff[((size_t)(y + M.blo1) * g.nx + (xx + M.blo0)) * g.nz + z]);
                if (d == d) {
                    const float r = d - m;
                    if (fr && m != 0.0f) {
                        const float var = M.sigma2f + M.eps2f * m * m;
                        ss += r * r / var;
                        lg += logf(var / M.sigma2f);
                    } else if (fr) {
                        ss += r * r / M.sigma2f;
                    } else {
                        ss += r * r;
                    }
                }
            }
        }
    }
    double ds = (double)ss, dl = (double)lg;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ds += __shfl_down_sync(0xffffffffu, ds, o);
        dl += __shfl_down_sync(0xffffffffu, dl, o);
    }
    __shared__ double red[2][8];
    if (lane == 0) { red[0][warp] = ds; red[1][warp] = dl; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; w++) { a += red[0][w]; b += red[1][w]; }
        pout[0] = a;
        pout[1] = b;
    }
}

}  // namespace

void conv_wide_taps(const double *k, int ky, int kx, float *taps) {
    // flipped, as conv_taps: out[y, x] = sum_{a, b} kf[a, b] in[y - hy + a, x - hx + b], kf[a, b] = k[ky-1-a, kx-1-b]
    for (int a = 0; a < ky; a++)
        for (int b = 0; b < kx; b++) taps[a * kx + b] = (float)k[(ky - 1 - a) * kx + (kx - 1 - b)];
}

void launch_conv_wide(cudaStream_t s, const GridDev &g, const MemberDev *mem, int nb, int maxt, int nzb, bool z16,
                      const float *model, long long mstride, int nz, const float *taps, int ky, int kx,
                      float *smoothed, int do_conv, int do_resid, double *partial, int npart, TileSrc ts) {
    const dim3 grid(nb, maxt, nzb);
    if (z16)
        k_conv_wide<16><<<grid, 256, 0, s>>>(g, mem, model, mstride, nz, taps, ky, kx, smoothed, do_conv, do_resid,
                                             partial, npart, ts);
    else
        k_conv_wide<32><<<grid, 256, 0, s>>>(g, mem, model, mstride, nz, taps, ky, kx, smoothed, do_conv, do_resid,
                                             partial, npart, ts);
}
