// The CLASSIC 3DFIT kernels on the device: the sparse convolution of single-ring models
// (_conv_sparse, bbarolo/galmod.py:974-1037) and the normalisation + residual (_norm, bbarolo/galfit.py:39-188).
//
// Both work on the small boxes of single-ring models in float64 (the reference's arithmetic, without
// contraction); the ring footprint of _norm (inside / weight of each pixel: atan2, sin, cos, pow) is computed on
// the host with the C library, as the reference, so that the pixels used are the same.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace {

// out (ny, nx, nz) = the "same" convolution of model (ny, nx, nz) with the kernel, values < 1e-12 set to zero,
// then x scale (the reference adds each source's non-zero channel range and thresholds the union of the
// ranges: the same values, since model channels outside a source's range are zero). The reference scatters
// the sources in (y, x) order, so an output voxel receives its terms with the kernel row and column
// descending: the same order here, one rounding per term, bit-exact.
__global__ void k_conv_sparse(const double *__restrict__ model, double *__restrict__ out, int ny, int nx, int nz,
                              const double *__restrict__ kern, int ky, int kx, double scale) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)ny * nx * nz;
    if (i >= n) return;
    const int z = (int)(i % nz);
    const long long p = i / nz;
    const int x = (int)(p % nx), y = (int)(p / nx);
    const int hy = ky / 2, hx = kx / 2;
    double s = 0.0;
    for (int j = ky - 1; j >= 0; j--) {
        const int yy = y - j + hy;
        if (yy < 0 || yy >= ny) continue;
        for (int q = kx - 1; q >= 0; q--) {
            const double kv = kern[j * kx + q];
            if (kv == 0.0) continue;
            const int xx = x - q + hx;
            if (xx < 0 || xx >= nx) continue;
            s = __dadd_rn(s, __dmul_rn(kv, model[((size_t)yy * nx + xx) * nz + z]));
        }
    }
    out[i] = s < 1.E-12 ? 0.0 : (scale != 1.0 ? __dmul_rn(s, scale) : s);
}

// The running sums of pre along x of every row: P (bsy, bsx + 1, nz), P[y, 0] = 0, P[y, x + 1] = P[y, x] +
// pre[y, x] (the reference's buffer of cumulative sums, same order).
__global__ void k_norm_prefix(const double *__restrict__ pre, double *__restrict__ P, int bsy, int bsx, int nz) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)bsy * nz) return;
    const int z = (int)(i % nz), y = (int)(i / nz);
    double a = 0.0;
    P[((size_t)y * (bsx + 1)) * nz + z] = 0.0;
    for (int x = 0; x < bsx; x++) {
        a = __dadd_rn(a, pre[((size_t)y * bsx + x) * nz + z]);
        P[((size_t)y * (bsx + 1) + x + 1) * nz + z] = a;
    }
}

// _norm, pass 1 (NORM AZIM): sums of the model and of the data in the mask over the pixels of the ring.
__global__ void k_norm_sums(const double *__restrict__ model, const float *__restrict__ data,
                            const uint8_t *__restrict__ mask, const uint8_t *__restrict__ inside, int bsy, int bsx,
                            int nz, double *__restrict__ part) {
    __shared__ double sm[256], so[256];
    const int p = blockIdx.x;           // pixel
    double a = 0.0, b = 0.0;
    if (inside[p])
        for (int z = threadIdx.x; z < nz; z += blockDim.x) {
            const size_t q = (size_t)p * nz + z;
            a += model[q];
            if (mask[q]) b += data[q];
        }
    sm[threadIdx.x] = a;
    so[threadIdx.x] = b;
    __syncthreads();
    for (int d = blockDim.x / 2; d > 0; d >>= 1) {
        if (threadIdx.x < d) {
            sm[threadIdx.x] += sm[threadIdx.x + d];
            so[threadIdx.x] += so[threadIdx.x + d];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * p] = sm[0];
        part[2 * p + 1] = so[0];
    }
}

// _norm, pass 2: per pixel of the ring, the factor (LOCAL: its own; AZIM: given), the model scaled in place,
// the blanks and the residual. One CTA per pixel, threads over the channels. P/ilo/ihi/thr: the support
// emulation of ANALYTIC models (lam = sum of pre over the kernel footprint around the pixel, from the running
// sums P of k_norm_prefix). The pixel's residual sum and counts go to part[4p..4p+3] = (sum, blanks, voxels,
// factor); the sum over channels is a fixed tree (the reference's running sum over all voxels differs from it
// by rounding only).
__global__ void k_norm_pix(double *__restrict__ model, const float *__restrict__ data, const uint8_t *__restrict__ mask,
                           const uint8_t *__restrict__ inside, const double *__restrict__ wmap, int bsy, int bsx, int nz,
                           int ftype, const double *__restrict__ chan_noise, double data_noise, int normtype,
                           double factor_azim, const double *__restrict__ P, const long long *__restrict__ ilo,
                           const long long *__restrict__ ihi, int ky, const double *__restrict__ thr,
                           double *__restrict__ part) {
    __shared__ double sa[256];
    __shared__ int sc[256], sd[256];
    __shared__ int s_ca, s_cb;
    const int p = blockIdx.x;
    const int y = p / bsx, x = p - y * bsx;
    if (!inside[p]) {
        if (threadIdx.x == 0) { part[4 * p] = 0.0; part[4 * p + 1] = 0.0; part[4 * p + 2] = 0.0; part[4 * p + 3] = 0.0; }
        return;
    }
    __shared__ double s_factor;
    // NORM LOCAL: the factor of this spectrum, summed over the channels in order (as the reference)
    if (threadIdx.x == 0) {
        double f = factor_azim;
        if (normtype == 0) {
            double a = 0.0, b = 0.0;
            for (int z = 0; z < nz; z++) {
                const size_t q = (size_t)p * nz + z;
                a = __dadd_rn(a, model[q]);
                const double o = data[q];
                if (o > 0 && mask[q]) b = __dadd_rn(b, o);
            }
            f = a != 0 ? __ddiv_rn(b, a) : 0.0;
        }
        s_factor = f;
    }
    __syncthreads();
    const double factor = s_factor;
    const bool trunc = P != nullptr;
    // the channel range [ca, cb] of model voxels outside the mask (the voxels whose support is tested)
    if (threadIdx.x == 0) { s_ca = nz; s_cb = -1; }
    __syncthreads();
    if (trunc)
        for (int z = threadIdx.x; z < nz; z += blockDim.x) {
            const size_t q = (size_t)p * nz + z;
            if (model[q] != 0 && !mask[q]) { atomicMin(&s_ca, z); atomicMax(&s_cb, z); }
        }
    __syncthreads();
    const int ca = s_ca, cb = s_cb;
    const int hy = ky / 2;
    const double wi = wmap[p];
    double mf = 0.0;
    int nb = 0, nt = 0;
    for (int z = threadIdx.x; z < nz; z += blockDim.x) {
        const size_t q = (size_t)p * nz + z;
        if (normtype != 2) model[q] = __dmul_rn(model[q], factor);
        const double o = data[q];
        const double obs = o > 0 ? o : data_noise;
        const double mod = model[q];
        if (!mask[q]) {
            if (mod == 0) continue;
            if (trunc) {
                // lam: the rows' sums of pre over the kernel footprint, from the running sums (reference order)
                double lam = 0.0;
                if (z >= ca && z <= cb)
                    for (int j = 0; j < ky; j++) {
                        const int yy = y + hy - j;
                        if (yy < 0 || yy >= bsy) continue;
                        long long xa = x + ilo[j], xb = x + ihi[j] + 1;
                        if (xa < 0) xa = 0;
                        if (xb > bsx) xb = bsx;
                        if (xb <= xa) continue;
                        const double p1 = P[((size_t)yy * (bsx + 1) + xb) * nz + z];
                        const double p0 = P[((size_t)yy * (bsx + 1) + xa) * nz + z];
                        lam = __dadd_rn(lam, __dsub_rn(p1, p0));
                    }
                if (lam < thr[z]) continue;
            }
            nb++;
        }
        nt++;
        const double nw = chan_noise[z];
        const double dmo = __dsub_rn(mod, obs);
        if (ftype == 1) mf = __dadd_rn(mf, __ddiv_rn(__ddiv_rn(__dmul_rn(wi, __dmul_rn(dmo, dmo)), sqrt(obs)), nw));
        else if (ftype == 2) mf = __dadd_rn(mf, __ddiv_rn(__dmul_rn(wi, fabs(dmo)), nw));
        else if (ftype == 3) mf = __dadd_rn(mf, __ddiv_rn(__ddiv_rn(__dmul_rn(wi, fabs(dmo)), __dadd_rn(mod, obs)), nw));
        else if (ftype == 4) mf = __dadd_rn(mf, __ddiv_rn(__dmul_rn(wi, __dmul_rn(dmo, dmo)), nw));
    }
    sa[threadIdx.x] = mf;
    sc[threadIdx.x] = nb;
    sd[threadIdx.x] = nt;
    __syncthreads();
    for (int d = blockDim.x / 2; d > 0; d >>= 1) {
        if (threadIdx.x < d) {
            sa[threadIdx.x] += sa[threadIdx.x + d];
            sc[threadIdx.x] += sc[threadIdx.x + d];
            sd[threadIdx.x] += sd[threadIdx.x + d];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[4 * p] = sa[0];
        part[4 * p + 1] = (double)sc[0];
        part[4 * p + 2] = (double)sd[0];
        part[4 * p + 3] = factor;
    }
}

}  // namespace

void launch_conv_sparse(cudaStream_t s, const double *model, double *out, int ny, int nx, int nz, const double *kern,
                        int ky, int kx, double scale) {
    const long long n = (long long)ny * nx * nz;
    if (n == 0) return;
    k_conv_sparse<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(model, out, ny, nx, nz, kern, ky, kx, scale);
}

void launch_norm_sums(cudaStream_t s, const double *model, const float *data, const uint8_t *mask,
                      const uint8_t *inside, int bsy, int bsx, int nz, double *part) {
    if (bsy * bsx == 0) return;
    k_norm_sums<<<bsy * bsx, 128, 0, s>>>(model, data, mask, inside, bsy, bsx, nz, part);
}

void launch_norm_prefix(cudaStream_t s, const double *pre, double *P, int bsy, int bsx, int nz) {
    const long long n = (long long)bsy * nz;
    if (n == 0) return;
    k_norm_prefix<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(pre, P, bsy, bsx, nz);
}

void launch_norm_pix(cudaStream_t s, double *model, const float *data, const uint8_t *mask, const uint8_t *inside,
                     const double *wmap, int bsy, int bsx, int nz, int ftype, const double *chan_noise,
                     double data_noise, int normtype, double factor_azim, const double *P, const long long *ilo,
                     const long long *ihi, int ky, const double *thr, double *part) {
    if (bsy * bsx == 0) return;
    k_norm_pix<<<bsy * bsx, 128, 0, s>>>(model, data, mask, inside, wmap, bsy, bsx, nz, ftype, chan_noise, data_noise,
                                        normtype, factor_azim, P, ilo, ihi, ky, thr, part);
}
