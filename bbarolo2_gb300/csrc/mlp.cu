// The surrogate of the log-likelihood: a multilayer perceptron (d -> 256 -> 256 -> 256 -> 1, GELU) trained online on
// the likelihood evaluations a sampler makes, with fused BF16 kernels of this library (no counterpart in the
// reference, whose nested sampler trains its own neural bounds in numba, bbarolo/bayesian/nautilus/mlp.py:18-118).
//
// Precision: the weights used by the products and the activations are BF16; products accumulate in FP32 on the
// tensor cores (mma.sync m16n8k16: the layers are small GEMMs, at most a few thousand rows, far from the sizes where
// tcgen05 pipelines pay); pre-activations, gradients, the FP32 master weights and Adam's moments are FP32.
//
// Kernels: one strided GEMM C[m][j] = sum_t A(m, t) B(t, j) (operands staged through shared memory as BF16 tiles)
// with fused epilogues (bias + GELU for the forward layers, the GELU derivative for the backward chain, plain FP32
// for the weight gradients), the output layer and the loss, column sums for the bias gradients, and Adam.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/bbgpu.h"

namespace {

constexpr int GT = 64;       // tile of m and of j
constexpr int GK = 32;       // chunk of t
constexpr int GPAD = 8;      // (padding of the shared-memory rows: no bank conflicts on the fragment loads)
constexpr int KSPLIT = 8;    // K ranges of the weight-gradient products (K = the batch rows)

enum Epi { EPI_BIAS_GELU = 0, EPI_GELU_GRAD = 1, EPI_F32 = 2 };

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// element (i, k) of a strided BF16 operand: p[i * si + k * sk]
__device__ __forceinline__ __nv_bfloat16 elem(const __nv_bfloat16 *p, long long off) { return p[off]; }

// C (M x N) = A (M x K) B (K x N), A(m, t) = A[m sam + t sat], B(t, j) = B[t sbt + j sbj]. Epilogues:
//  EPI_BIAS_GELU: z = C + bias[j] -> Z[m][j] (FP32), out[m][j] = gelu(z) (BF16)
//  EPI_GELU_GRAD: out[m][j] = C * gelu'(Z[m][j]) (BF16, the pre-activation gradient of the layer below), and also
//                 into F32[m][j] when given
//  EPI_F32: F32[m][j] = C (FP32)
// 128 threads: 4 warps of 32 x 32 in a 64 x 64 tile; mma.sync.m16n8k16 row.col BF16 -> FP32.
template <typename TA, typename TB, int EPI>
__global__ void __launch_bounds__(128) k_gemm(int M, int N, int K, const TA *__restrict__ A, long long sam,
                                              long long sat, const TB *__restrict__ B, long long sbt, long long sbj,
                                              const float *__restrict__ bias, float *__restrict__ Z,
                                              __nv_bfloat16 *__restrict__ out, float *__restrict__ F32) {
    __shared__ __align__(16) __nv_bfloat16 As[GT][GK + GPAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[GT][GK + GPAD];   // [j][t]
    const int m0 = blockIdx.y * GT, j0 = blockIdx.x * GT;
    // split K (EPI_F32 only): block z takes the K range [z kper, (z + 1) kper) and writes its partial product to
    // F32 + z M N (summed in order by k_sum_splits)
    const int kper = (K + gridDim.z - 1) / gridDim.z;
    const int tb = blockIdx.z * kper, te = min(K, tb + kper);
    if (EPI == EPI_F32) F32 += (size_t)blockIdx.z * M * N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wj = (warp & 1) * 32;
    const int g = lane >> 2, c = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[a][b][q] = 0.0f;
    for (int t0 = tb; t0 < te; t0 += GK) {
        for (int e = threadIdx.x; e < GT * GK; e += 128) {
            const int i = e / GK, t = e % GK;
            const int m = m0 + i, j = j0 + i, tt = t0 + t;
            As[i][t] = (m < M && tt < te) ? elem(A, (long long)m * sam + (long long)tt * sat)
                                          : __float2bfloat16_rn(0.0f);
            Bs[i][t] = (j < N && tt < te) ? elem(B, (long long)tt * sbt + (long long)j * sbj)
                                          : __float2bfloat16_rn(0.0f);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int a = 0; a < 2; a++) {
                const int r = wm + a * 16 + g;
                af[a][0] = *(const uint32_t *)&As[r][kk + 2 * c];
                af[a][1] = *(const uint32_t *)&As[r + 8][kk + 2 * c];
                af[a][2] = *(const uint32_t *)&As[r][kk + 2 * c + 8];
                af[a][3] = *(const uint32_t *)&As[r + 8][kk + 2 * c + 8];
            }
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int n = wj + b * 8 + g;
                bf[b][0] = *(const uint32_t *)&Bs[n][kk + 2 * c];
                bf[b][1] = *(const uint32_t *)&Bs[n][kk + 2 * c + 8];
            }
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 4; b++)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                        "{%8,%9}, {%0,%1,%2,%3};"
                        : "+f"(acc[a][b][0]), "+f"(acc[a][b][1]), "+f"(acc[a][b][2]), "+f"(acc[a][b][3])
                        : "r"(af[a][0]), "r"(af[a][1]), "r"(af[a][2]), "r"(af[a][3]), "r"(bf[b][0]), "r"(bf[b][1]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int m = m0 + wm + a * 16 + g + (q >= 2 ? 8 : 0);
                const int j = j0 + wj + b * 8 + 2 * c + (q & 1);
                if (m >= M || j >= N) continue;
                const size_t o = (size_t)m * N + j;
                const float v = acc[a][b][q];
                if (EPI == EPI_BIAS_GELU) {
                    const float z = v + bias[j];
                    Z[o] = z;
                    out[o] = __float2bfloat16_rn(gelu(z));
                } else if (EPI == EPI_GELU_GRAD) {
                    const float d = v * gelu_grad(Z[o]);
                    out[o] = __float2bfloat16_rn(d);
                    if (F32) F32[o] = d;
                } else {
                    F32[o] = v;
                }
            }
}

// the output layer and the loss: y[b] = a[b] . w + bias (warp per row); with targets, r = y - t, dy = 2 r / n (the
// gradient of the mean squared error) and the loss sum of r^2 into loss[0] (atomic)
__global__ void k_output(int n, int H, const __nv_bfloat16 *__restrict__ a, const __nv_bfloat16 *__restrict__ w,
                         const float *__restrict__ bias, const float *__restrict__ t, float *__restrict__ y,
                         float *__restrict__ dy, float *__restrict__ loss) {
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= n) return;
    float s = 0.0f;
    for (int k = lane; k < H; k += 32) s += __bfloat162float(a[(size_t)row * H + k]) * __bfloat162float(w[k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        const float v = s + bias[0];
        y[row] = v;
        if (t) {
            const float r = v - t[row];
            dy[row] = 2.0f * r / (float)n;
            atomicAdd(loss, r * r);
        }
    }
}

// the gradient of the last hidden layer's pre-activation: dz[b][k] = dy[b] w[k] gelu'(z[b][k]) (BF16)
__global__ void k_out_back(int n, int H, const float *__restrict__ dy, const __nv_bfloat16 *__restrict__ w,
                           const float *__restrict__ z, __nv_bfloat16 *__restrict__ dz, float *__restrict__ dz32) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * H) return;
    const int b = (int)(i / H), k = (int)(i % H);
    const float d = dy[b] * __bfloat162float(w[k]) * gelu_grad(z[i]);
    dz[i] = __float2bfloat16_rn(d);
    if (dz32) dz32[i] = d;
}

// column sums: out[j] = sum_b in[b][j] (or, with v given, sum_b v[b] a[b][j]: the output weights' gradient); a block
// of 32 columns x 32 row groups, the groups' partial sums added in shared memory
__global__ void __launch_bounds__(1024) k_colsum(int n, int N, const float *__restrict__ in,
                                                 const float *__restrict__ v, const __nv_bfloat16 *__restrict__ a,
                                                 float *__restrict__ out) {
    __shared__ float part[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + tx;
    float s = 0.0f;
    if (j < N)
        for (int b = ty; b < n; b += 32)
            s += v ? v[b] * __bfloat162float(a[(size_t)b * N + j]) : in[(size_t)b * N + j];
    part[ty][tx] = s;
    __syncthreads();
    if (ty == 0 && j < N) {
        float t = 0.0f;
        for (int k = 0; k < 32; k++) t += part[k][tx];
        out[j] = t;
    }
}

// out[i] = sum over the splits z (in order) of part[z][i]
__global__ void k_sum_splits(long long n, int nsplit, const float *__restrict__ part, float *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a = part[i];
    for (int z = 1; z < nsplit; z++) a += part[(size_t)z * n + i];
    out[i] = a;
}

__global__ void k_sum(int n, const float *__restrict__ v, float *__restrict__ out) {
    __shared__ float sh[256];
    float s = 0.0f;
    for (int i = threadIdx.x; i < n; i += 256) s += v[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int d = 128; d > 0; d >>= 1) {
        if (threadIdx.x < d) sh[threadIdx.x] += sh[threadIdx.x + d];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sh[0];
}

// Adam on the FP32 master weights, the BF16 copy rewritten (b1t, b2t: 1 - beta^t)
__global__ void k_adam(long long n, float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, __nv_bfloat16 *__restrict__ w16, float lr, float b1, float b2,
                       float b1t, float b2t, float eps) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / b1t) / (sqrtf(vi / b2t) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(long long n, const float *__restrict__ in, __nv_bfloat16 *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

// a minibatch of `rows` rows drawn with replacement from the n rows of a resident training set: row r of step
// `step` is the set's row hash(seed, step, r) mod n (inputs to BF16, targets as they are)
__global__ void k_gather_batch(int rows, int d, int n, unsigned long long seed, int step,
                               const float *__restrict__ xs, const float *__restrict__ ts,
                               __nv_bfloat16 *__restrict__ x16, float *__restrict__ t) {
    const int r = blockIdx.x;
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * ((unsigned long long)step * 0x100000001ull + r + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const long long src = (long long)(z % (unsigned long long)n);
    for (int k = threadIdx.x; k < d; k += blockDim.x) x16[(size_t)r * d + k] = __float2bfloat16_rn(xs[src * d + k]);
    if (threadIdx.x == 0) t[r] = ts[src];
}

}  // namespace

// ------------------------------------------------------------------------------------------------- host side
struct bbgpu_mlp {
    int device = 0, d = 0, H = 0;
    long long np = 0;                 // parameters: W1 (H x d), b1 (H), W2 (H x H), b2, W3 (H x H), b3, w4 (H), b4
    long long off[8] = {};
    float *w = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;   // FP32 master, gradient, Adam moments
    __nv_bfloat16 *w16 = nullptr;     // BF16 copy used by the products
    int step = 0;
    int cap = 0;                      // rows of the batch buffers
    float *xf = nullptr, *t = nullptr, *y = nullptr, *dy = nullptr, *loss = nullptr;
    __nv_bfloat16 *x16 = nullptr, *a[3] = {}, *dz[2] = {};
    float *z[3] = {}, *dz32[2] = {};
    float *set_x = nullptr, *set_t = nullptr;   // the resident training set of bbgpu_mlp_train
    float *split = nullptr;                      // the partial weight gradients of a split-K product
    long long set_cap = 0;
    cudaStream_t s = nullptr;
};

namespace {

int grow(bbgpu_mlp *m, int n) {
    if (n <= m->cap) return BBGPU_OK;
    cudaFree(m->xf); cudaFree(m->t); cudaFree(m->y); cudaFree(m->dy); cudaFree(m->x16);
    for (int i = 0; i < 3; i++) { cudaFree(m->a[i]); cudaFree(m->z[i]); }
    for (int i = 0; i < 2; i++) { cudaFree(m->dz[i]); cudaFree(m->dz32[i]); }
    const size_t nh = (size_t)n * m->H;
    bool ok = cudaMalloc(&m->xf, sizeof(float) * (size_t)n * m->d) == cudaSuccess &&
              cudaMalloc(&m->x16, sizeof(__nv_bfloat16) * (size_t)n * m->d) == cudaSuccess &&
              cudaMalloc(&m->t, sizeof(float) * n) == cudaSuccess && cudaMalloc(&m->y, sizeof(float) * n) == cudaSuccess &&
              cudaMalloc(&m->dy, sizeof(float) * n) == cudaSuccess;
    for (int i = 0; i < 3 && ok; i++)
        ok = cudaMalloc(&m->a[i], sizeof(__nv_bfloat16) * nh) == cudaSuccess &&
             cudaMalloc(&m->z[i], sizeof(float) * nh) == cudaSuccess;
    for (int i = 0; i < 2 && ok; i++)
        ok = cudaMalloc(&m->dz[i], sizeof(__nv_bfloat16) * nh) == cudaSuccess &&
             cudaMalloc(&m->dz32[i], sizeof(float) * nh) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        m->cap = 0;
        return BBGPU_ERR_NOMEM;
    }
    m->cap = n;
    return BBGPU_OK;
}

template <typename TA, typename TB, int EPI>
void gemm(cudaStream_t s, int M, int N, int K, const TA *A, long long sam, long long sat, const TB *B, long long sbt,
          long long sbj, const float *bias, float *Z, __nv_bfloat16 *out, float *F32, int nsplit = 1) {
    dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT, nsplit);
    k_gemm<TA, TB, EPI><<<grid, 128, 0, s>>>(M, N, K, A, sam, sat, B, sbt, sbj, bias, Z, out, F32);
}

// the forward pass of n rows of m->x16 (and with targets t, the loss and dy)
void forward(bbgpu_mlp *m, int n, const float *t) {
    const int d = m->d, H = m->H;
    const __nv_bfloat16 *W = m->w16;
    const float *b = m->w;
    gemm<__nv_bfloat16, __nv_bfloat16, EPI_BIAS_GELU>(m->s, n, H, d, m->x16, d, 1, W + m->off[0], 1, d,
                                                      b + m->off[1], m->z[0], m->a[0], nullptr);
    for (int l = 1; l < 3; l++)
        gemm<__nv_bfloat16, __nv_bfloat16, EPI_BIAS_GELU>(m->s, n, H, H, m->a[l - 1], H, 1, W + m->off[2 * l], 1, H,
                                                          b + m->off[2 * l + 1], m->z[l], m->a[l], nullptr);
    if (t) cudaMemsetAsync(m->loss, 0, sizeof(float), m->s);
    k_output<<<(n + 7) / 8, 256, 0, m->s>>>(n, H, m->a[2], W + m->off[6], b + m->off[7], t, m->y, m->dy, m->loss);
}

// the gradient of the mean squared error over the n rows, into m->g
void backward(bbgpu_mlp *m, int n) {
    const int d = m->d, H = m->H;
    const __nv_bfloat16 *W = m->w16;
    float *G = m->g;
    const size_t nh = (size_t)n * H;
    k_out_back<<<(unsigned)((nh + 255) / 256), 256, 0, m->s>>>(n, H, m->dy, W + m->off[6], m->z[2], m->dz[0],
                                                                m->dz32[0]);
    k_colsum<<<(H + 31) / 32, 1024, 0, m->s>>>(n, H, nullptr, m->dy, m->a[2], G + m->off[6]);
    k_sum<<<1, 256, 0, m->s>>>(n, m->dy, G + m->off[7]);
    int cur = 0;
    for (int l = 2; l >= 0; l--) {
        const __nv_bfloat16 *below = l > 0 ? m->a[l - 1] : m->x16;
        const int kin = l > 0 ? H : d;
        // weight gradient: G[j][k] = sum_b dz[b][j] below[b][k]; bias gradient: column sums of dz
        // (K = the batch rows: split in KSPLIT ranges, the partial products summed in order)
        const int ns = std::max(1, std::min(KSPLIT, n / 128));
        gemm<__nv_bfloat16, __nv_bfloat16, EPI_F32>(m->s, H, kin, n, m->dz[cur], 1, H, below, kin, 1, nullptr,
                                                    nullptr, nullptr, ns > 1 ? m->split : G + m->off[2 * l], ns);
        if (ns > 1) {
            const long long nn = (long long)H * kin;
            k_sum_splits<<<(unsigned)((nn + 255) / 256), 256, 0, m->s>>>(nn, ns, m->split, G + m->off[2 * l]);
        }
        k_colsum<<<(H + 31) / 32, 1024, 0, m->s>>>(n, H, m->dz32[cur], nullptr, nullptr, G + m->off[2 * l + 1]);
        if (l > 0)   // the layer below: dz'[b][k] = (sum_j dz[b][j] W[j][k]) gelu'(z'[b][k])
            gemm<__nv_bfloat16, __nv_bfloat16, EPI_GELU_GRAD>(m->s, n, H, H, m->dz[cur], H, 1, W + m->off[2 * l], H,
                                                              1, nullptr, m->z[l - 1], m->dz[1 - cur],
                                                              m->dz32[1 - cur]);
        cur = 1 - cur;
    }
}

int load_x(bbgpu_mlp *m, const float *x, int n) {
    int rc = grow(m, n);
    if (rc) return rc;
    const size_t nx = (size_t)n * m->d;
    if (cudaMemcpyAsync(m->xf, x, sizeof(float) * nx, cudaMemcpyHostToDevice, m->s) != cudaSuccess)
        return BBGPU_ERR_CUDA;
    k_to_bf16<<<(unsigned)((nx + 255) / 256), 256, 0, m->s>>>((long long)nx, m->xf, m->x16);
    return BBGPU_OK;
}

int finish(bbgpu_mlp *m) {
    cudaError_t e = cudaStreamSynchronize(m->s);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? BBGPU_OK : BBGPU_ERR_CUDA;
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" int bbgpu_mlp_create(bbgpu_mlp **out, int device, int d_in, int hidden, uint64_t seed) {
    if (!out || d_in < 1 || d_in > 4096 || hidden < 8 || hidden > 4096) return BBGPU_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return BBGPU_ERR_CUDA;
    bbgpu_mlp *m = new bbgpu_mlp();
    m->device = device;
    m->d = d_in;
    m->H = hidden;
    const long long H = hidden, d = d_in;
    const long long sizes[8] = {H * d, H, H * H, H, H * H, H, H, 1};
    for (int i = 0; i < 8; i++) {
        m->off[i] = m->np;
        m->np += sizes[i];
    }
    // initial weights uniform in +-1/sqrt(fan in), biases zero
    std::vector<float> w(m->np, 0.0f);
    const long long fan[4] = {d, H, H, H};
    for (int l = 0; l < 4; l++) {
        const float a = 1.0f / sqrtf((float)fan[l]);
        for (long long i = 0; i < sizes[2 * l]; i++)
            w[m->off[2 * l] + i] = a * (2.0f * (float)((splitmix(seed) >> 11) * (1.0 / 9007199254740992.0)) - 1.0f);
    }
    bool ok = cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&m->w, sizeof(float) * m->np) == cudaSuccess &&
              cudaMalloc(&m->g, sizeof(float) * m->np) == cudaSuccess &&
              cudaMalloc(&m->m1, sizeof(float) * m->np) == cudaSuccess &&
              cudaMalloc(&m->m2, sizeof(float) * m->np) == cudaSuccess &&
              cudaMalloc(&m->w16, sizeof(__nv_bfloat16) * m->np) == cudaSuccess &&
              cudaMalloc(&m->split, sizeof(float) * KSPLIT * (size_t)hidden * std::max(hidden, d_in)) == cudaSuccess &&
              cudaMalloc(&m->loss, sizeof(float)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        bbgpu_mlp_destroy(m);
        return BBGPU_ERR_NOMEM;
    }
    int rc = bbgpu_mlp_set_params(m, w.data());
    if (rc) {
        bbgpu_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return BBGPU_OK;
}

extern "C" int bbgpu_mlp_destroy(bbgpu_mlp *m) {
    if (!m) return BBGPU_ERR_ARG;
    cudaSetDevice(m->device);
    cudaFree(m->w); cudaFree(m->g); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->w16); cudaFree(m->loss);
    cudaFree(m->xf); cudaFree(m->t); cudaFree(m->y); cudaFree(m->dy); cudaFree(m->x16);
    for (int i = 0; i < 3; i++) { cudaFree(m->a[i]); cudaFree(m->z[i]); }
    for (int i = 0; i < 2; i++) { cudaFree(m->dz[i]); cudaFree(m->dz32[i]); }
    cudaFree(m->set_x); cudaFree(m->set_t); cudaFree(m->split);
    if (m->s) cudaStreamDestroy(m->s);
    delete m;
    return BBGPU_OK;
}

extern "C" long long bbgpu_mlp_nparams(const bbgpu_mlp *m) { return m ? m->np : 0; }

extern "C" int bbgpu_mlp_set_params(bbgpu_mlp *m, const float *p) {
    if (!m || !p) return BBGPU_ERR_ARG;
    if (cudaSetDevice(m->device) != cudaSuccess) return BBGPU_ERR_CUDA;
    cudaMemcpyAsync(m->w, p, sizeof(float) * m->np, cudaMemcpyHostToDevice, m->s);
    cudaMemsetAsync(m->m1, 0, sizeof(float) * m->np, m->s);
    cudaMemsetAsync(m->m2, 0, sizeof(float) * m->np, m->s);
    k_to_bf16<<<(unsigned)((m->np + 255) / 256), 256, 0, m->s>>>(m->np, m->w, m->w16);
    m->step = 0;
    return finish(m);
}

extern "C" int bbgpu_mlp_get_params(const bbgpu_mlp *m, float *p) {
    if (!m || !p) return BBGPU_ERR_ARG;
    if (cudaSetDevice(m->device) != cudaSuccess) return BBGPU_ERR_CUDA;
    return cudaMemcpy(p, m->w, sizeof(float) * m->np, cudaMemcpyDeviceToHost) == cudaSuccess ? BBGPU_OK
                                                                                             : BBGPU_ERR_CUDA;
}

extern "C" int bbgpu_mlp_predict(bbgpu_mlp *m, const float *x, int n, float *y) {
    if (!m || (!x && n) || (!y && n) || n < 0) return BBGPU_ERR_ARG;
    if (n == 0) return BBGPU_OK;
    if (cudaSetDevice(m->device) != cudaSuccess) return BBGPU_ERR_CUDA;
    int rc = load_x(m, x, n);
    if (rc) return rc;
    forward(m, n, nullptr);
    cudaMemcpyAsync(y, m->y, sizeof(float) * n, cudaMemcpyDeviceToHost, m->s);
    return finish(m);
}

extern "C" int bbgpu_mlp_gradients(bbgpu_mlp *m, const float *x, const float *t, int n, float *grads, float *loss) {
    if (!m || !x || !t || n < 1) return BBGPU_ERR_ARG;
    if (cudaSetDevice(m->device) != cudaSuccess) return BBGPU_ERR_CUDA;
    int rc = load_x(m, x, n);
    if (rc) return rc;
    cudaMemcpyAsync(m->t, t, sizeof(float) * n, cudaMemcpyHostToDevice, m->s);
    forward(m, n, m->t);
    backward(m, n);
    float ls = 0.0f;
    if (grads) cudaMemcpyAsync(grads, m->g, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->s);
    cudaMemcpyAsync(&ls, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->s);
    rc = finish(m);
    if (loss) *loss = ls / (float)n;
    return rc;
}

namespace {

// one Adam step on the rows already in x16 / t
void adam_step(bbgpu_mlp *m, int n, float lr) {
    forward(m, n, m->t);
    backward(m, n);
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    k_adam<<<(unsigned)((m->np + 255) / 256), 256, 0, m->s>>>(m->np, m->w, m->m1, m->m2, m->g, m->w16, lr, b1, b2,
                                                              1.0f - powf(b1, (float)m->step),
                                                              1.0f - powf(b2, (float)m->step), 1e-8f);
}

}  // namespace

extern "C" int bbgpu_mlp_train(bbgpu_mlp *m, const float *x, const float *t, long long n, int steps, int batch,
                               float lr, uint64_t seed, float *loss) {
    if (!m || !x || !t || n < 1 || n > 0x7fffffffLL || steps < 1 || batch < 1 || !(lr > 0)) return BBGPU_ERR_ARG;
    if (cudaSetDevice(m->device) != cudaSuccess) return BBGPU_ERR_CUDA;
    int rc = grow(m, batch);
    if (rc) return rc;
    if (n > m->set_cap) {
        cudaFree(m->set_x);
        cudaFree(m->set_t);
        m->set_x = m->set_t = nullptr;
        m->set_cap = 0;
        if (cudaMalloc(&m->set_x, sizeof(float) * (size_t)n * m->d) != cudaSuccess ||
            cudaMalloc(&m->set_t, sizeof(float) * (size_t)n) != cudaSuccess) {
            cudaGetLastError();
            return BBGPU_ERR_NOMEM;
        }
        m->set_cap = n;
    }
    cudaMemcpyAsync(m->set_x, x, sizeof(float) * (size_t)n * m->d, cudaMemcpyHostToDevice, m->s);
    cudaMemcpyAsync(m->set_t, t, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, m->s);
    for (int k = 0; k < steps; k++) {
        k_gather_batch<<<batch, 64, 0, m->s>>>(batch, m->d, (int)n, seed, k, m->set_x, m->set_t, m->x16, m->t);
        adam_step(m, batch, lr);
    }
    float ls = 0.0f;
    cudaMemcpyAsync(&ls, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->s);
    rc = finish(m);
    if (loss) *loss = ls / (float)batch;
    return rc;
}

extern "C" int bbgpu_mlp_train_step(bbgpu_mlp *m, const float *x, const float *t, int n, float lr, float *loss) {
    if (!m || !x || !t || n < 1 || !(lr > 0)) return BBGPU_ERR_ARG;
    if (cudaSetDevice(m->device) != cudaSuccess) return BBGPU_ERR_CUDA;
    int rc = load_x(m, x, n);
    if (rc) return rc;
    cudaMemcpyAsync(m->t, t, sizeof(float) * n, cudaMemcpyHostToDevice, m->s);
    adam_step(m, n, lr);
    float ls = 0.0f;
    cudaMemcpyAsync(&ls, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->s);
    rc = finish(m);
    if (loss) *loss = ls / (float)n;
    return rc;
}
