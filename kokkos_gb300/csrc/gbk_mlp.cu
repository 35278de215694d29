// FP32 MLP cost model for the learned tuner: D -> 64 -> 64 -> 1, ReLU.
// Training and inference run on these kernels (no library GEMM): the layers
// are tiny, so each CTA takes S samples, keeps their activations and the
// 64x64 weights in shared memory, and computes one (sample, unit) output per
// thread and step; weight gradients are reduced over the CTA's samples in
// shared memory and added to the global gradient with one atomicAdd per
// parameter per CTA.
#include "../../include/gbk_tools.h"
#include "gbk_internal.cuh"

namespace gbk {
namespace {

constexpr int H = 64;
constexpr int S = 16;       // samples per CTA
constexpr int TPB = 256;    // threads per CTA
constexpr int DMAX = 64;    // largest input width

struct Off {
  int64_t w1, b1, w2, b2, w3, b3, total;
};
__host__ __device__ inline Off offsets(int D) {
  Off o;
  o.w1 = 0;
  o.b1 = o.w1 + (int64_t)D * H;
  o.w2 = o.b1 + H;
  o.b2 = o.w2 + H * H;
  o.w3 = o.b2 + H;
  o.b3 = o.w3 + H;
  o.total = o.b3 + 1;
  return o;
}

__global__ void __launch_bounds__(TPB)
    k_mlp_fwd(const float* __restrict__ X, int64_t B, int D, const float* __restrict__ P, float* __restrict__ A,
              float* __restrict__ Y) {
  const Off o = offsets(D);
  __shared__ float sx[S][DMAX];
  __shared__ float s1[S][H];
  __shared__ float s2[S][H];
  __shared__ float sw2[H][H + 1];
  const int64_t b0 = (int64_t)blockIdx.x * S;
  for (int i = threadIdx.x; i < S * D; i += TPB) {
    const int s = i / D, d = i % D;
    sx[s][d] = (b0 + s < B) ? X[(b0 + s) * D + d] : 0.f;
  }
  for (int i = threadIdx.x; i < H * H; i += TPB) sw2[i / H][i % H] = P[o.w2 + i];
  __syncthreads();
  for (int i = threadIdx.x; i < S * H; i += TPB) {
    const int s = i / H, j = i % H;
    float z = P[o.b1 + j];
    for (int d = 0; d < D; ++d) z = fmaf(sx[s][d], P[o.w1 + (int64_t)d * H + j], z);
    s1[s][j] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < S * H; i += TPB) {
    const int s = i / H, j = i % H;
    float z = P[o.b2 + j];
#pragma unroll 8
    for (int k = 0; k < H; ++k) z = fmaf(s1[s][k], sw2[k][j], z);
    s2[s][j] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  // outputs and saved activations
  for (int i = threadIdx.x; i < S * H; i += TPB) {
    const int s = i / H, j = i % H;
    if (b0 + s < B) {
      A[(b0 + s) * (2 * H) + j] = s1[s][j];
      A[(b0 + s) * (2 * H) + H + j] = s2[s][j];
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int s = warp; s < S; s += TPB / 32) {
    float v = s2[s][lane] * P[o.w3 + lane] + s2[s][lane + 32] * P[o.w3 + lane + 32];
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    if (lane == 0 && b0 + s < B) Y[b0 + s] = v + P[o.b3];
  }
}

__global__ void __launch_bounds__(TPB)
    k_mlp_bwd(const float* __restrict__ X, int64_t B, int D, const float* __restrict__ P, const float* __restrict__ A,
              const float* __restrict__ dY, float* __restrict__ G) {
  const Off o = offsets(D);
  __shared__ float sx[S][DMAX];
  __shared__ float s1[S][H];   // A1, then reused
  __shared__ float s2[S][H];   // A2
  __shared__ float dz2[S][H];
  __shared__ float dz1[S][H];
  __shared__ float sdy[S];
  __shared__ float sw2[H][H + 1];
  const int64_t b0 = (int64_t)blockIdx.x * S;
  for (int i = threadIdx.x; i < S * D; i += TPB) {
    const int s = i / D, d = i % D;
    sx[s][d] = (b0 + s < B) ? X[(b0 + s) * D + d] : 0.f;
  }
  for (int i = threadIdx.x; i < S * H; i += TPB) {
    const int s = i / H, j = i % H;
    const bool ok = b0 + s < B;
    s1[s][j] = ok ? A[(b0 + s) * (2 * H) + j] : 0.f;
    s2[s][j] = ok ? A[(b0 + s) * (2 * H) + H + j] : 0.f;
  }
  for (int i = threadIdx.x; i < S; i += TPB) sdy[i] = (b0 + i < B) ? dY[b0 + i] : 0.f;
  for (int i = threadIdx.x; i < H * H; i += TPB) sw2[i / H][i % H] = P[o.w2 + i];
  __syncthreads();
  // layer 3 and dZ2
  for (int i = threadIdx.x; i < S * H; i += TPB) {
    const int s = i / H, j = i % H;
    dz2[s][j] = s2[s][j] > 0.f ? sdy[s] * P[o.w3 + j] : 0.f;
  }
  if (threadIdx.x < H) {
    float g = 0.f;
    for (int s = 0; s < S; ++s) g = fmaf(sdy[s], s2[s][threadIdx.x], g);
    atomicAdd(G + o.w3 + threadIdx.x, g);
  }
  if (threadIdx.x == H) {
    float g = 0.f;
    for (int s = 0; s < S; ++s) g += sdy[s];
    atomicAdd(G + o.b3, g);
  }
  __syncthreads();
  // dZ1 = (dZ2 W2^T) * relu'(A1)
  for (int i = threadIdx.x; i < S * H; i += TPB) {
    const int s = i / H, k = i % H;
    float z = 0.f;
#pragma unroll 8
    for (int j = 0; j < H; ++j) z = fmaf(dz2[s][j], sw2[k][j], z);
    dz1[s][k] = s1[s][k] > 0.f ? z : 0.f;
  }
  // dW2[k][j] = sum_s A1[s][k] dZ2[s][j]; db2[j] = sum_s dZ2[s][j]
  for (int i = threadIdx.x; i < H * H; i += TPB) {
    const int k = i / H, j = i % H;
    float g = 0.f;
    for (int s = 0; s < S; ++s) g = fmaf(s1[s][k], dz2[s][j], g);
    atomicAdd(G + o.w2 + i, g);
  }
  if (threadIdx.x < H) {
    float g = 0.f;
    for (int s = 0; s < S; ++s) g += dz2[s][threadIdx.x];
    atomicAdd(G + o.b2 + threadIdx.x, g);
  }
  __syncthreads();
  // dW1[d][j] = sum_s X[s][d] dZ1[s][j]; db1[j] = sum_s dZ1[s][j]
  for (int i = threadIdx.x; i < D * H; i += TPB) {
    const int d = i / H, j = i % H;
    float g = 0.f;
    for (int s = 0; s < S; ++s) g = fmaf(sx[s][d], dz1[s][j], g);
    atomicAdd(G + o.w1 + i, g);
  }
  if (threadIdx.x < H) {
    float g = 0.f;
    for (int s = 0; s < S; ++s) g += dz1[s][threadIdx.x];
    atomicAdd(G + o.b1 + threadIdx.x, g);
  }
}

__global__ void k_mlp_mse(const float* __restrict__ Y, const float* __restrict__ T, int64_t B, float* __restrict__ dY,
                          float* __restrict__ loss) {
  __shared__ float sm[32];
  float acc = 0.f;
  for (int64_t i = threadIdx.x; i < B; i += blockDim.x) {
    const float e = Y[i] - T[i];
    dY[i] = 2.f * e / (float)B;
    acc = fmaf(e, e, acc);
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < blockDim.x / 32 ? sm[threadIdx.x] : 0.f;
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    if (threadIdx.x == 0) loss[0] = v / (float)B;
  }
}

__global__ void k_mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int64_t gbk_mlp_param_count(int D) { return D > 0 ? offsets(D).total : 0; }

int gbk_mlp_forward(const float* X, int64_t B, int D, const float* params, float* acts, float* Y, gbk_stream_t s) {
  if (B < 0 || D < 1 || D > DMAX || (B > 0 && (!X || !params || !acts || !Y))) return GBK_ERR_INVALID_ARGUMENT;
  if (B == 0) return GBK_OK;
  const int64_t grid = (B + S - 1) / S;
  k_mlp_fwd<<<(unsigned)grid, TPB, 0, (cudaStream_t)s>>>(X, B, D, params, acts, Y);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int gbk_mlp_backward(const float* X, int64_t B, int D, const float* params, const float* acts, const float* dY,
                     float* grads, gbk_stream_t s) {
  if (B < 0 || D < 1 || D > DMAX || !grads || (B > 0 && (!X || !params || !acts || !dY)))
    return GBK_ERR_INVALID_ARGUMENT;
  GBK_CUDA_TRY(cudaMemsetAsync(grads, 0, sizeof(float) * (size_t)offsets(D).total, (cudaStream_t)s));
  if (B == 0) return GBK_OK;
  const int64_t grid = (B + S - 1) / S;
  k_mlp_bwd<<<(unsigned)grid, TPB, 0, (cudaStream_t)s>>>(X, B, D, params, acts, dY, grads);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int gbk_mlp_mse(const float* Y, const float* T, int64_t B, float* dY, float* loss, gbk_stream_t s) {
  if (B <= 0 || !Y || !T || !dY || !loss) return GBK_ERR_INVALID_ARGUMENT;
  k_mlp_mse<<<1, 1024, 0, (cudaStream_t)s>>>(Y, T, B, dY, loss);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int gbk_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t P, float lr, float beta1, float beta2,
                 float eps, int t, gbk_stream_t s) {
  if (P <= 0 || !params || !grads || !m || !v || t < 1) return GBK_ERR_INVALID_ARGUMENT;
  const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
  int64_t grid = (P + 255) / 256;
  if (grid > 1024) grid = 1024;
  k_mlp_adam<<<(unsigned)grid, 256, 0, (cudaStream_t)s>>>(params, grads, m, v, P, lr, beta1, beta2, eps, c1, c2);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
