// The beam convolution + residual of MC models whose members share deposit tiles with member 0 (the kernel of
// conv_kernel.cuh with its tile table; a translation unit of its own so that the two variants compile in
// parallel).
#include "conv_kernel.cuh"

void launch_conv_table(cudaStream_t s, const GridDev &g, const MemberDev *mem, int nb, int maxt, int nzb, bool z16,
                       const float *model, long long mstride, int nz, const float *taps, int ky, int kx, int kxw,
                       float *smoothed, int do_conv, int do_resid, double *partial, int npart, TileSrc ts) {
#define CASE(W)                                                                                                    \
    case W:                                                                                                        \
        if (z16)                                                                                                   \
            launch_t<W, 16, true>(s, g, mem, nb, maxt, nzb, model, mstride, nz, taps, ky, kx, smoothed, do_conv,   \
                                  do_resid, partial, npart, ts);                                                   \
        else                                                                                                       \
            launch_t<W, 32, true>(s, g, mem, nb, maxt, nzb, model, mstride, nz, taps, ky, kx, smoothed, do_conv,   \
                                  do_resid, partial, npart, ts);                                                   \
        break;
    switch (kxw) {
        CASE(1) CASE(3) CASE(5) CASE(7) CASE(9) CASE(11) CASE(13) CASE(15) CASE(17) CASE(21) CASE(25) CASE(31)
        default: break;
    }
#undef CASE
}
