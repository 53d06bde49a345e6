// GALWIND WTYPE 1 on the device: the Monte-Carlo clouds of spherical shells of a bi-cone (the reference's
// _galmod_wind, bbarolo/galmod.py:539-590).
//
// The host parses the reference's stream into the clouds (radius, azimuth, polar angle, the first word of each
// velocity deviate and the values of the rare deviates off the ziggurat's one-word path) and the
// shells' constants (bbh_wind_clouds); one thread per cloud then places it (its pixel with the reference's float64
// operations in its order, no contraction, so the pixel is the reference's) and deposits each of its velocity
// samples in the channel of each line, in 64-bit fixed point (units 2^(E-62), 2^E above the total flux of the
// clouds: exact sums, independent of their order).
#include <cuda_runtime.h>
#include <stdint.h>

#include "devmath.cuh"
#include "kernels.h"

namespace {

__global__ void __launch_bounds__(256) k_wind_mc(const WindShell *__restrict__ shells, const int *__restrict__ shell,
                                                 const double *__restrict__ geo, const long long *__restrict__ nbase,
                                                 const long long *__restrict__ sbase, const int *__restrict__ hz,
                                                 const double *__restrict__ slow, const ZigDev *__restrict__ zig,
                                                 long long ncloud, GridDev g,
                                                 const double *__restrict__ cd2i, int blo0, int blo1, int bhi0,
                                                 int bhi1, double scale, unsigned long long *__restrict__ acc) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncloud) return;
    const WindShell s = shells[shell[i]];
    const double *c = geo + 5 * (size_t)i;
    const double rad = c[0], caz = c[1], saz = c[2], sphi = c[3], cphi = c[4];
    // bbarolo/galmod.py:568-575
    const double R = __dmul_rn(rad, sphi), z = __dmul_rn(rad, cphi);
    const double x = __dmul_rn(R, caz);
    const double y = __dsub_rn(__dmul_rn(__dmul_rn(R, saz), s.cinc), __dmul_rn(z, s.sinc));
    const long long g0 =
        lround_ref(__dadd_rn(s.xpos, __ddiv_rn(__dsub_rn(__dmul_rn(x, s.spa), __dmul_rn(y, s.cpa)), g.cdelt0)));
    const long long g1 =
        lround_ref(__dadd_rn(s.ypos, __ddiv_rn(__dadd_rn(__dmul_rn(x, s.cpa), __dmul_rn(y, s.spa)), g.cdelt1)));
    if (g0 < blo0 || g0 >= bhi0 || g1 < blo1 || g1 >= bhi1) return;
    // bbarolo/galmod.py:581-589
    const double geom = __dadd_rn(__dmul_rn(cphi, s.cinc), __dmul_rn(__dmul_rn(sphi, saz), s.sinc));
    const double vs = __dadd_rn(__dadd_rn(s.vsys, __dmul_rn(s.vsph, geom)), __dmul_rn(__dmul_rn(s.vrot, caz), s.sinc));
    unsigned long long *o = acc + ((size_t)(g1 - blo1) * (bhi0 - blo0) + (size_t)(g0 - blo0)) * g.nz;
    const int *h = hz + nbase[i];
    long long js = sbase[i];
    for (int iv = 0; iv < s.nvr; iv++) {
        // the deviate: from its first word on the ziggurat's one-word path (the reference's product), else recorded
        const int hv = h[iv];
        const unsigned ah = hv < 0 ? 0u - (unsigned)hv : (unsigned)hv;
        const double n = ah < zig->kn[hv & 127] ? __dmul_rn((double)hv, zig->wn[hv & 127]) : slow[js++];
        const double v = __dadd_rn(vs, __dmul_rn(n, s.vdisp));
        for (int nl = 0; nl < g.nlines; nl++) {
            const long long k = lround_ref(velgrid_exact(v, g, nl));
            if (k < 0 || k >= g.nz) continue;
            const double val = __dmul_rn(__dmul_rn(g.relint[nl], s.fluxsc), cd2i[k]);
            atomicAdd(o + k, (unsigned long long)__double2ll_rn(val * scale));
        }
    }
}

}  // namespace

void launch_wind_mc(cudaStream_t st, const WindShell *shells, const int *shell, const double *geo,
                    const long long *nbase, const long long *sbase, const int *hz, const double *slow,
                    const ZigDev *zig, long long ncloud, const GridDev &g, const double *cd2i, int blo0, int blo1,
                    int bhi0, int bhi1, double scale, unsigned long long *acc) {
    if (ncloud <= 0) return;
    k_wind_mc<<<(unsigned)((ncloud + 255) / 256), 256, 0, st>>>(shells, shell, geo, nbase, sbase, hz, slow, zig, ncloud,
                                                                 g, cd2i, blo0, blo1, bhi0, bhi1, scale, acc);
}
