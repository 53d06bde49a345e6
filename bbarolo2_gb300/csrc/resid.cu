// Layout changes and the stand-alone residual kernels (the reference's float64 entry points).
//
// k_prep_deff turns the cube into what the residual of a likelihood reads: (ny, nx, nz) float32, channels
// fastest like the models, NaN where a voxel is not used (bbarolo/bayesian/likelihood.py:22-45: blanks
// are NaN or 0 data; outside the region; outside the mask with maskmode 2) and 0 outside the mask with
// maskmode 1 (data * mask). It runs once per cube and mode.
//
// k_sumsq64 is _sumsq_residuals / _residuals_fracerr on a float64 model (nz, ny, nx): the stand-alone entry
// points keep the reference's float64 arithmetic per voxel; per-CTA partial sums are reduced in a fixed order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace {

__global__ void k_prep_deff(const float *__restrict__ data, const uint8_t *__restrict__ mask,
                            const uint8_t *__restrict__ region, int maskmode, int nz, int ny, int nx,
                            float *__restrict__ deff) {
    // thread per output voxel (y, x, z); reads are strided (once per cube)
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)nz * ny * nx;
    if (i >= n) return;
    int z = (int)(i % nz);
    long long p = i / nz;
    int x = (int)(p % nx), y = (int)(p / nx);
    size_t q = ((size_t)z * ny + y) * nx + x;
    float d = data[q];
    float out;
    if (region && !region[(size_t)y * nx + x]) out = __int_as_float(0x7fc00000);
    else if (d != d || d == 0.0f) out = __int_as_float(0x7fc00000);
    else if (maskmode != 0 && !(mask && mask[q])) out = maskmode == 2 ? __int_as_float(0x7fc00000) : 0.0f;
    else out = d;
    deff[i] = out;
}

__global__ void k_sumsq64(const double *__restrict__ model, const float *__restrict__ data,
                          const uint8_t *__restrict__ mask, int maskmode, const uint8_t *__restrict__ region,
                          int nz, int ny, int nx, double sigma2, double eps2, double *__restrict__ partial) {
    __shared__ double sa[256], sb[256];
    long long n = (long long)nz * ny * nx;
    double s = 0.0, lg = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        long long yx = q % ((long long)ny * nx);
        if (region && !region[yx]) continue;
        double d = data[q];
        if (d != d || d == 0.0) continue;
        if (maskmode != 0 && !mask[q]) {
            if (maskmode == 2) continue;
            d = 0.0;
        }
        double m = model[q];
        double r = __dsub_rn(d, m);
        if (eps2 > 0.0) {
            if (m != 0.0) {
                double v = __dadd_rn(sigma2, __dmul_rn(__dmul_rn(eps2, m), m));
                s = __dadd_rn(s, __ddiv_rn(__dmul_rn(r, r), v));
                lg += log(v / sigma2);
            } else {
                s = __dadd_rn(s, __ddiv_rn(__dmul_rn(r, r), sigma2));
            }
        } else {
            s = __dadd_rn(s, __dmul_rn(r, r));
        }
    }
    sa[threadIdx.x] = s;
    sb[threadIdx.x] = lg;
    __syncthreads();
    for (int d = 128; d > 0; d >>= 1) {
        if (threadIdx.x < d) { sa[threadIdx.x] += sa[threadIdx.x + d]; sb[threadIdx.x] += sb[threadIdx.x + d]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = sa[0]; partial[2 * blockIdx.x + 1] = sb[0]; }
}

// (nz, ny, nx) float64 -> (ny, nx, nz) float32 and back
__global__ void k_zyx64_to_yxz32(const double *__restrict__ in, float *__restrict__ out, int nz, int ny, int nx) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)nz * ny * nx;
    if (i >= n) return;
    int z = (int)(i % nz);
    long long p = i / nz;
    out[i] = (float)in[(size_t)z * ny * nx + p];
}

__global__ void k_yxz32_to_zyx64(const float *__restrict__ in, double *__restrict__ out, int nz, int ny, int nx) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)nz * ny * nx;
    if (i >= n) return;
    long long p = i % ((long long)ny * nx);
    int z = (int)(i / ((long long)ny * nx));
    out[i] = (double)in[p * nz + z];
}

}  // namespace

void launch_prep_deff(cudaStream_t s, const float *data, const uint8_t *mask, const uint8_t *region, int maskmode,
                      int nz, int ny, int nx, float *deff) {
    long long n = (long long)nz * ny * nx;
    k_prep_deff<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data, mask, region, maskmode, nz, ny, nx, deff);
}

int launch_sumsq64(cudaStream_t s, const double *model, const float *data, const uint8_t *mask, int maskmode,
                   const uint8_t *region, int nz, int ny, int nx, double sigma2, double eps2, double *partial,
                   int maxblocks) {
    long long n = (long long)nz * ny * nx;
    int nbk = (int)((n + 255) / 256);
    if (nbk > maxblocks) nbk = maxblocks;
    if (nbk < 1) nbk = 1;
    k_sumsq64<<<nbk, 256, 0, s>>>(model, data, mask, maskmode, region, nz, ny, nx, sigma2, eps2, partial);
    return nbk;
}

void launch_zyx64_to_yxz32(cudaStream_t s, const double *in, float *out, int nz, int ny, int nx) {
    long long n = (long long)nz * ny * nx;
    k_zyx64_to_yxz32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, nz, ny, nx);
}

void launch_yxz32_to_zyx64(cudaStream_t s, const float *in, double *out, int nz, int ny, int nx) {
    long long n = (long long)nz * ny * nx;
    k_yxz32_to_zyx64<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, nz, ny, nx);
}
