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

#include "conv_kernel.cuh"

namespace {

__global__ void k_reduce_partials(const double *__restrict__ partial, int npart, double *__restrict__ out2) {
    // one CTA per member; fixed summation order (deterministic)
    __shared__ double sa[256], sb[256];
    const int k = blockIdx.x;
    const double *p = partial + 2 * (size_t)k * npart;
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < npart; i += 256) {
        // (-1: the tile's sums are member 0's, see the tile table of k_conv_resid)
        const bool m0 = p[2 * i] == -1.0;
        a += m0 ? partial[2 * i] : p[2 * i];
        b += m0 ? partial[2 * i + 1] : p[2 * i + 1];
    }
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

void conv_tile_shape(int nz, int bx, int by, int &nct, int &ntx, int &shx, int &shy) {
    const int toy = TO * (32 / conv_zb(nz));
    ntx = (bx + TO - 1) / TO;
    nct = ntx * ((by + toy - 1) / toy);
    shx = 4;                               // (TO = 16)
    shy = toy == 32 ? 5 : 4;
}

int conv_resid_npart(const MemberDev *mem_host, int nb, int nz) {
    int maxt, nzb;
    conv_grid(mem_host, nb, nz, maxt, nzb);
    return maxt * nzb;
}

void launch_conv_resid(cudaStream_t s, const GridDev &g, const MemberDev *mem, const MemberDev *mem_host, int nb,
                       const float *model, long long mstride, int nz, const float *taps, int ky, int kx, int kxw,
                       float *smoothed, int do_conv, int do_resid, double *partial, TileSrc ts) {
    int maxt, nzb;
    conv_grid(mem_host, nb, nz, maxt, nzb);
    if (nb == 0 || maxt == 0) return;
    const int npart = maxt * nzb;
    if (!do_conv) kxw = 1;
    const bool z16 = conv_zb(nz) == 16;
    if (kxw == 0) {            // a kernel wider than the templates: taps (ky, kx) in global memory
        launch_conv_wide(s, g, mem, nb, maxt, nzb, z16, model, mstride, nz, taps, ky, kx, smoothed, do_conv, do_resid,
                         partial, npart, ts);
        return;
    }
    if (ts.tsrc) {
        launch_conv_table(s, g, mem, nb, maxt, nzb, z16, model, mstride, nz, taps, ky, kx, kxw, smoothed, do_conv,
                          do_resid, partial, npart, ts);
        return;
    }
#define CASE(W)                                                                                                    \
    case W:                                                                                                        \
        if (z16)                                                                                                   \
            launch_t<W, 16, false>(s, g, mem, nb, maxt, nzb, model, mstride, nz, taps, ky, kx, smoothed, do_conv,  \
                                   do_resid, partial, npart, ts);                                                  \
        else                                                                                                       \
            launch_t<W, 32, false>(s, g, mem, nb, maxt, nzb, model, mstride, nz, taps, ky, kx, smoothed, do_conv,  \
                                   do_resid, partial, npart, ts);                                                  \
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
