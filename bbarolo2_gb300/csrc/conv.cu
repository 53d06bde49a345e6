// Beam convolution of the model and the masked residual, fused (bbarolo/smooth.py:145-165,
// bbarolo/galmod.py:1273-1283, bbarolo/bayesian/likelihood.py:22-77).
//
// The model of a member is (by, bx, nz) float32: channels fastest, so that a warp holds 32 channels of one
// pixel and every load and store is a 128-byte line. One CTA computes a 16 x 16 pixel tile of 32 channels (or,
// when 16-channel blocks pad the channels less, as the 41 ring maps of the flux normalisation, a 16 x 32 tile of
// 16 channels, the two half-warps on the two halves of the rows):
// the input tile with its halo (zero outside the box: the reference convolves the box with zero padding) is
// staged in shared memory, each thread accumulates two output rows of 16 pixels for its channel over the
// kernel rows, from a register window of the input row (float32 FMAs; the taps are broadcast from shared
// memory). The epilogue applies the reference's threshold (values below 1e-12 set to zero) and flux scale,
// and, instead of writing the smoothed cube, compares it with the data: each CTA leaves the sum of squared
// residuals of its voxels (and the sum of log-variances for a fractional model error), reduced in float64.
// Tiles whose input is all zero skip the convolution (empty channels and the corners of the box).
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

template <int KXW, int ZB>
__global__ void __launch_bounds__(256, 2) k_conv_resid(GridDev g, const MemberDev *__restrict__ mem,
                                                       const float *__restrict__ model, long long mstride, int nz,
                                                       const float *__restrict__ taps, int ky, int kx,
                                                       float *__restrict__ smoothed, int do_conv, int do_resid,
                                                       double *__restrict__ partial, int npart) {
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
    // the input tile with its halo, asynchronously: 16-byte copies of 4 channels when the rows of channels are
    // 16-byte aligned (nz a multiple of 4), else 4-byte copies; zeros outside the box and past nz
    const bool vec = (nz & 3) == 0 && (((uintptr_t)mk) & 15) == 0;
    if (vec) {
        for (int c = threadIdx.x; c < H * W * (ZB / 4); c += blockDim.x) {
            const int q = c & (ZB / 4 - 1), rc = c / (ZB / 4);
            const int r = rc / W, col = rc - r * W;
            const int yy = y0 - hy + r, xx = x0 - hx + col, zz = zb * ZB + 4 * q;
            const bool ok = col < ncol && yy >= 0 && yy < M.by && xx >= 0 && xx < M.bx && zz < nz;
            cp_async_zfill16(S + (size_t)rc * ZB + 4 * q, ok ? mk + ((size_t)yy * M.bx + xx) * nz + zz : mk, ok);
        }
    } else {
        for (int c = threadIdx.x; c < H * W * ZB; c += blockDim.x) {
            const int l = c & (ZB - 1), rc = c / ZB;
            const int r = rc / W, col = rc - r * W;
            const int yy = y0 - hy + r, xx = x0 - hx + col, zz = zb * ZB + l;
            const bool ok = col < ncol && yy >= 0 && yy < M.by && xx >= 0 && xx < M.bx && zz < nz;
            cp_async_zfill4(S + c, ok ? mk + ((size_t)yy * M.bx + xx) * nz + zz : mk, ok);
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

__global__ void k_reduce_partials(const double *__restrict__ partial, int npart, double *__restrict__ out2) {
    // one CTA per member; fixed summation order (deterministic)
    __shared__ double sa[256], sb[256];
    const int k = blockIdx.x;
    const double *p = partial + 2 * (size_t)k * npart;
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < npart; i += 256) { a += p[2 * i]; b += p[2 * i + 1]; }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int d = 128; d > 0; d >>= 1) {
        if (threadIdx.x < d) { sa[threadIdx.x] += sa[threadIdx.x + d]; sb[threadIdx.x] += sb[threadIdx.x + d]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out2[2 * k] = sa[0]; out2[2 * k + 1] = sb[0]; }
}

// the channel block of a cube: 16 lanes when it pads the channels less than 32 (e.g. 41 ring maps: 48 against
// 64), else 32
int conv_zb(int nz) { return ((nz + 15) / 16) * 16 < ((nz + 31) / 32) * 32 ? 16 : 32; }

template <int KXW, int ZB>
void launch_t(cudaStream_t s, const GridDev &g, const MemberDev *mem, int nb, int maxt, int nzb, const float *model,
              long long mstride, int nz, const float *taps, int ky, int kx, float *smoothed, int do_conv,
              int do_resid, double *partial, int npart) {
    const int kye = do_conv ? ky : 1;
    constexpr int TOY = TO * (32 / ZB);
    size_t smem = (size_t)(TOY + kye - 1) * (TO + KXW - 1) * ZB * sizeof(float) + (size_t)ky * KXW * sizeof(float);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_conv_resid<KXW, ZB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    dim3 grid(nb, maxt, nzb);
    k_conv_resid<KXW, ZB><<<grid, 256, smem, s>>>(g, mem, model, mstride, nz, taps, ky, kx, smoothed, do_conv,
                                                 do_resid, partial, npart);
}

}  // namespace

static const int KXWS[] = {1, 3, 5, 7, 9, 11, 13, 15, 17, 21, 25, 31};

int conv_taps(const double *k, int ky, int kx, float *taps) {
    int kxw = 0;
    for (int w : KXWS)
        if (w >= kx) { kxw = w; break; }
    if (!kxw) return 0;
    // flipped: out[y, x] = sum_{a, b} kf[a, b] in[y - hy + a, x - hx + b], kf[a, b] = k[ky-1-a, kx-1-b]
    for (int a = 0; a < ky; a++)
        for (int b = 0; b < kxw; b++)
            taps[a * kxw + b] = b < kx ? (float)k[(ky - 1 - a) * kx + (kx - 1 - b)] : 0.0f;
    return kxw;
}

// tiles of the largest member box (TO x TOY pixels) and channel blocks of a cube
static void conv_grid(const MemberDev *mem_host, int nb, int nz, int &maxt, int &nzb) {
    const int zbw = conv_zb(nz), toy = TO * (32 / zbw);
    maxt = 0;
    for (int k = 0; k < nb; k++)
        maxt = max(maxt, ((mem_host[k].bx + TO - 1) / TO) * ((mem_host[k].by + toy - 1) / toy));
    nzb = (nz + zbw - 1) / zbw;
}

int conv_resid_npart(const MemberDev *mem_host, int nb, int nz) {
    int maxt, nzb;
    conv_grid(mem_host, nb, nz, maxt, nzb);
    return maxt * nzb;
}

void launch_conv_resid(cudaStream_t s, const GridDev &g, const MemberDev *mem, const MemberDev *mem_host, int nb,
                       const float *model, long long mstride, int nz, const float *taps, int ky, int kx, int kxw,
                       float *smoothed, int do_conv, int do_resid, double *partial) {
    int maxt, nzb;
    conv_grid(mem_host, nb, nz, maxt, nzb);
    if (nb == 0 || maxt == 0) return;
    const int npart = maxt * nzb;
    if (!do_conv) kxw = 1;
    const bool z16 = conv_zb(nz) == 16;
#define CASE(W)                                                                                                    \
    case W:                                                                                                        \
        if (z16)                                                                                                   \
            launch_t<W, 16>(s, g, mem, nb, maxt, nzb, model, mstride, nz, taps, ky, kx, smoothed, do_conv, do_resid, \
                            partial, npart);                                                                       \
        else                                                                                                       \
            launch_t<W, 32>(s, g, mem, nb, maxt, nzb, model, mstride, nz, taps, ky, kx, smoothed, do_conv, do_resid, \
                            partial, npart);                                                                       \
        break;
    switch (kxw) {
        CASE(1) CASE(3) CASE(5) CASE(7) CASE(9) CASE(11) CASE(13) CASE(15) CASE(17) CASE(21) CASE(25) CASE(31)
        default: break;
    }
#undef CASE
}

void launch_reduce_partials(cudaStream_t s, const double *partial, int npart, int nb, double *out2) {
    if (nb == 0) return;
    k_reduce_partials<<<nb, 256, 0, s>>>(partial, npart, out2);
}
