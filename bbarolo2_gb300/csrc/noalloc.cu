// bbgpu_sumsq_residuals_noalloc: the float64 residual reduction without any device allocation.
//
// Who needs it: code that may not call cudaMalloc while it evaluates a likelihood -- a host application that
// hands out all device memory from its own pool (a framework allocator, a fixed arena sized at start-up), code
// running while a CUDA graph is being captured (an allocation would break the capture), or a long-running
// service that must not grow its memory footprint after warm-up. Such callers already hold the model, the
// data and the output on the device; this entry point only launches kernels on their stream.
//
// Scratch: the per-block partial sums live in one file-scope device array (NOALLOC_MAX_BLOCKS blocks of
// NOALLOC_VOXELS_PER_BLOCK voxels, 64 KB), which every GPU that loads the library keeps until the process
// exits. Host code cannot use the array's name as a device address, so its address is looked up with
// cudaGetSymbolAddress once per device, with that device current, on the first call made on it: make that
// first call before capturing a stream into a graph. All calls share the array: each call overwrites the
// partial sums of its own blocks before reading them (nothing is carried over), but two calls whose kernels
// overlap on the GPU (on different streams, or from different host threads) race on it.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "../../include/bbgpu.h"

#define NOALLOC_THREADS 256
#define NOALLOC_VOXELS_PER_BLOCK 4096
#define NOALLOC_MAX_BLOCKS 4096
#define NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[2 * NOALLOC_MAX_BLOCKS];

namespace {

// One block sums its NOALLOC_VOXELS_PER_BLOCK consecutive voxels (the rules of _sumsq_residuals /
// _residuals_fracerr, bbarolo/bayesian/likelihood.py:22-77, in float64 without contraction) in a fixed order.
__global__ void __launch_bounds__(NOALLOC_THREADS) k_sumsq_blocks(const double *__restrict__ model,
                                                                  const float *__restrict__ data,
                                                                  const uint8_t *__restrict__ mask, int maskmode,
                                                                  const uint8_t *__restrict__ region, long long n,
                                                                  long long nyx, double sigma2, double eps2,
                                                                  double *__restrict__ partial) {
    __shared__ double sa[NOALLOC_THREADS], sb[NOALLOC_THREADS];
    const long long b0 = (long long)blockIdx.x * NOALLOC_VOXELS_PER_BLOCK;
    double s = 0.0, lg = 0.0;
    for (int j = threadIdx.x; j < NOALLOC_VOXELS_PER_BLOCK; j += NOALLOC_THREADS) {
        const long long q = b0 + j;
        if (q >= n) break;
        if (region && !region[q % nyx]) continue;
        double d = data[q];
        if (d != d || d == 0.0) continue;
        if (maskmode != 0 && !mask[q]) {
            if (maskmode == 2) continue;
            d = 0.0;
        }
        const double m = model[q];
        const double r = __dsub_rn(d, m);
        if (eps2 > 0.0) {
            if (m != 0.0) {
                const double v = __dadd_rn(sigma2, __dmul_rn(__dmul_rn(eps2, m), m));
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
    for (int d = NOALLOC_THREADS / 2; d > 0; d >>= 1) {
        if (threadIdx.x < d) {
            sa[threadIdx.x] += sa[threadIdx.x + d];
            sb[threadIdx.x] += sb[threadIdx.x + d];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = sa[0];
        partial[2 * blockIdx.x + 1] = sb[0];
    }
}

// The partial sums of the nb blocks of this call (written by k_sumsq_blocks just before), in a fixed order.
__global__ void __launch_bounds__(NOALLOC_THREADS) k_sumsq_final(const double *__restrict__ partial, int nb,
                                                                 double *__restrict__ out2) {
    __shared__ double sa[NOALLOC_THREADS], sb[NOALLOC_THREADS];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nb; i += NOALLOC_THREADS) {
        a += partial[2 * i];
        b += partial[2 * i + 1];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int d = NOALLOC_THREADS / 2; d > 0; d >>= 1) {
        if (threadIdx.x < d) {
            sa[threadIdx.x] += sa[threadIdx.x + d];
            sb[threadIdx.x] += sb[threadIdx.x + d];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out2[0] = sa[0];
        out2[1] = sb[0];
    }
}

std::mutex g_mu;
double *g_scratch[NOALLOC_MAX_DEVICES] = {};

// The device address of the scratch array on the current device, looked up once per device.
int scratch_address(double **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return BBGPU_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return BBGPU_ERR_CUDA;
        }
        g_scratch[dev] = (double *)p;
    }
    *out = g_scratch[dev];
    return BBGPU_OK;
}

}  // namespace

extern "C" int bbgpu_sumsq_residuals_noalloc(const double *model, const float *data, const uint8_t *mask,
                                             int maskmode, const uint8_t *region, int nz, int ny, int nx,
                                             double sigma2, double eps2, double *out2, void *stream) {
    if (!model || !data || !out2 || nz < 0 || ny < 0 || nx < 0) return BBGPU_ERR_ARG;
    if (maskmode < 0 || maskmode > 2 || (maskmode != 0 && !mask)) return BBGPU_ERR_ARG;
    if (!(eps2 >= 0) || (eps2 > 0 && !(sigma2 > 0))) return BBGPU_ERR_ARG;   // (a NaN eps2 fails the first test)
    const long long n = (long long)nz * ny * nx;
    const long long nblocks = (n + NOALLOC_VOXELS_PER_BLOCK - 1) / NOALLOC_VOXELS_PER_BLOCK;
    if (nblocks > NOALLOC_MAX_BLOCKS) return BBGPU_ERR_ARG;   // more voxels than the scratch holds sums for
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != BBGPU_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // an error left by earlier CUDA work of the caller is not this call's: report it without launching, and leave
    // it for the caller to read
    if (cudaPeekAtLastError() != cudaSuccess) return BBGPU_ERR_CUDA;
    if (nblocks > 0) {
        k_sumsq_blocks<<<(unsigned)nblocks, NOALLOC_THREADS, 0, s>>>(model, data, mask, maskmode, region, n,
                                                                     (long long)ny * nx, sigma2, eps2, scratch);
        if (cudaGetLastError() != cudaSuccess) return BBGPU_ERR_CUDA;
    }
    k_sumsq_final<<<1, NOALLOC_THREADS, 0, s>>>(scratch, (int)nblocks, out2);
    if (cudaGetLastError() != cudaSuccess) return BBGPU_ERR_CUDA;
    return BBGPU_OK;
}
