// Where the time of a 2^24-element Sum goes: copies of the library's double
// Sum (k_sum_f64_split: 5 vectors per tile, 2 of them on the FP64 pipe, the
// rest exact on the integer pipes) and of an int64 flat Sum of the same
// shape, each stamping %globaltimer per CTA at entry, after its first tile,
// at the end of its share, after the CTA tree and after the grid finish.
// Measurement program only (the library kernels carry no stamps); prints,
// per CTAs-per-SM count, the spread of each phase over the CTAs beside the
// launch's CUDA-event time, then back-to-back launch times.
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
//        -o phase_stamps kokkos_gb300/bench_phase_stamps.cu && ./phase_stamps
#include "csrc/gbk_fixsum.cuh"
#include "csrc/gbk_reduce_impl.cuh"
#include <cstdio>
#include <vector>
#include <algorithm>
using namespace gbk;

__device__ __forceinline__ unsigned long long gt() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

struct Stamp { unsigned long long entry, first, loop_end, reduced, done; };

template <int BLOCK, int UNROLL, int FPV>
__global__ void __launch_bounds__(BLOCK)
    k_split_st(const double* __restrict__ x, int64_t n, double* partials, unsigned* counter, double* out, Stamp* st) {
  constexpr int IPI = 2 * (UNROLL - FPV);
  __shared__ double sm[BLOCK / 32];
  double fa = 0.0, fb = 0.0;
  FixAcc a;
  fix_init(a);
  unsigned long long t_entry = gt(), t_first = 0;
  const double* xb = x;
  const int64_t nvec = n / 2;
  constexpr int64_t TILE = (int64_t)BLOCK * UNROLL;
  const int64_t per = nvec / gridDim.x, rem = nvec % gridDim.x;
  const int64_t v0 = (int64_t)blockIdx.x * per + ((int64_t)blockIdx.x < rem ? blockIdx.x : rem);
  const int64_t v1 = v0 + per + ((int64_t)blockIdx.x < rem ? 1 : 0);
  int64_t vb = v0 + threadIdx.x;
  bool have = vb + (int64_t)(UNROLL - 1) * BLOCK < v1;
  uint4 cur[UNROLL], nxt[UNROLL];
  if (have) {
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = ld_stream16(xb + (vb + (int64_t)u * BLOCK) * 2);
  }
  int since = 0;
  bool first = true;
  while (have) {
    const int64_t vn = vb + TILE;
    const bool hn = vn + (int64_t)(UNROLL - 1) * BLOCK < v1;
    if (hn) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) nxt[u] = ld_stream16(xb + (vn + (int64_t)u * BLOCK) * 2);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const uint64_t b0 = ((uint64_t)cur[u].y << 32) | cur[u].x;
      const uint64_t b1 = ((uint64_t)cur[u].w << 32) | cur[u].z;
      if (u < FPV) {
        fa += __longlong_as_double((long long)b0);
        fb += __longlong_as_double((long long)b1);
      } else {
        fix_add2(a, fa, b0, b1);
      }
    }
    if (first) { t_first = gt() + (unsigned long long)(fa == 12345.0); first = false; }
    since += IPI;
    if (since >= (1 << 14)) { fb += fix_to_double(a); since = 0; }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = nxt[u];
    vb = vn;
    have = hn;
  }
  for (; vb < v1; vb += BLOCK) {
    const uint4 v = ld_stream16(xb + vb * 2);
    fix_add2(a, fa, ((uint64_t)v.y << 32) | v.x, ((uint64_t)v.w << 32) | v.z);
  }
  const double acc0 = fa + fb + fix_to_double(a);
  unsigned long long t_loop = gt() + (unsigned long long)(acc0 == 12345.0);
  __syncthreads();
  unsigned long long t_red = gt();
  grid_finish<RSum<double>, BLOCK>(acc0, partials, counter, out, sm);
  if (threadIdx.x == 0) {
    st[blockIdx.x] = Stamp{t_entry, t_first, t_loop, t_red, gt()};
  }
}

template <int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK)
    k_i64_st(const long long* __restrict__ x, int64_t n, long long* partials, unsigned* counter, long long* out, Stamp* st) {
  __shared__ long long sm[BLOCK / 32];
  long long acc = 0;
  unsigned long long t_entry = gt(), t_first = 0;
  const int64_t nvec = n / 2;
  constexpr int64_t TILE = (int64_t)BLOCK * UNROLL;
  const int64_t per = nvec / gridDim.x, rem = nvec % gridDim.x;
  const int64_t v0 = (int64_t)blockIdx.x * per + ((int64_t)blockIdx.x < rem ? blockIdx.x : rem);
  const int64_t v1 = v0 + per + ((int64_t)blockIdx.x < rem ? 1 : 0);
  int64_t vb = v0 + threadIdx.x;
  bool have = vb + (int64_t)(UNROLL - 1) * BLOCK < v1;
  uint4 cur[UNROLL], nxt[UNROLL];
  if (have) {
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = ld_stream16(x + (vb + (int64_t)u * BLOCK) * 2);
  }
  bool first = true;
  while (have) {
    const int64_t vn = vb + TILE;
    const bool hn = vn + (int64_t)(UNROLL - 1) * BLOCK < v1;
    if (hn) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) nxt[u] = ld_stream16(x + (vn + (int64_t)u * BLOCK) * 2);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u)
      acc += (long long)(((uint64_t)cur[u].y << 32) | cur[u].x) + (long long)(((uint64_t)cur[u].w << 32) | cur[u].z);
    if (first) { t_first = gt() + (unsigned long long)(acc == 12345); first = false; }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = nxt[u];
    vb = vn;
    have = hn;
  }
  for (; vb < v1; vb += BLOCK) {
    const uint4 v = ld_stream16(x + vb * 2);
    acc += (long long)(((uint64_t)v.y << 32) | v.x) + (long long)(((uint64_t)v.w << 32) | v.z);
  }
  unsigned long long t_loop = gt() + (unsigned long long)(acc == 12345);
  __syncthreads();
  unsigned long long t_red = gt();
  grid_finish<RSum<long long>, BLOCK>(acc, partials, counter, out, sm);
  if (threadIdx.x == 0) st[blockIdx.x] = Stamp{t_entry, t_first, t_loop, t_red, gt()};
}

static void report(const char* name, std::vector<Stamp>& h, float ev_us) {
  unsigned long long t0 = ~0ull, emax = 0, fmin = ~0ull, fmax = 0, lmin = ~0ull, lmax = 0, dmax = 0, rmax = 0;
  std::vector<double> loopd;
  for (auto& s : h) {
    t0 = std::min(t0, s.entry); emax = std::max(emax, s.entry);
    fmin = std::min(fmin, s.first); fmax = std::max(fmax, s.first);
    lmin = std::min(lmin, s.loop_end); lmax = std::max(lmax, s.loop_end);
    rmax = std::max(rmax, s.reduced); dmax = std::max(dmax, s.done);
    loopd.push_back((double)(s.loop_end - s.entry) / 1e3);
  }
  std::sort(loopd.begin(), loopd.end());
  std::printf("%s: event %.2f us | entries spread %.2f | first tile done %.2f..%.2f | loop end %.2f..%.2f | "
              "reduced max %.2f | finish %.2f | per-CTA loop us p10 %.2f p50 %.2f p90 %.2f max %.2f\n",
              name, ev_us, (emax - t0) / 1e3, (fmin - t0) / 1e3, (fmax - t0) / 1e3, (lmin - t0) / 1e3,
              (lmax - t0) / 1e3, (rmax - t0) / 1e3, (dmax - t0) / 1e3, loopd[loopd.size() / 10],
              loopd[loopd.size() / 2], loopd[loopd.size() * 9 / 10], loopd.back());
}

int main() {
  const int64_t n = 1 << 24;
  const int COPIES = 4;
  double* x;
  cudaMalloc(&x, (size_t)n * 8 * COPIES);
  std::vector<double> hx(n);
  for (int64_t i = 0; i < n; ++i) hx[i] = (double)((i * 2654435761ull) % 1000003) / 1000003.0;
  for (int c = 0; c < COPIES; ++c) cudaMemcpy(x + (size_t)c * n, hx.data(), (size_t)n * 8, cudaMemcpyHostToDevice);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int r1 = 0, r2 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r1, k_split_st<256, 5, 2>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r2, k_i64_st<256, 4>, 256, 0);
  double* part; unsigned* cnt; double* out; Stamp* st;
  cudaMalloc(&part, 1 << 20); cudaMalloc(&cnt, 64); cudaMemset(cnt, 0, 64); cudaMalloc(&out, 64);
  cudaMalloc(&st, sizeof(Stamp) * 8192);
  cudaEvent_t a, b;
  cudaEventCreate(&a); cudaEventCreate(&b);
  for (int variant = 0; variant < 2; ++variant) {
    for (int cps = 1; cps <= (variant == 0 ? r1 : r2); ++cps) {
      const int grid = sms * cps;
      for (int it = 0; it < 8; ++it) {
        const int c = it % COPIES;
        cudaEventRecord(a);
        if (variant == 0) k_split_st<256, 5, 2><<<grid, 256>>>(x + (size_t)c * n, n, part, cnt, out, st);
        else k_i64_st<256, 4><<<grid, 256>>>((const long long*)(x + (size_t)c * n), n, (long long*)part, cnt, (long long*)out, st);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (it == 7) {
          std::vector<Stamp> h(grid);
          cudaMemcpy(h.data(), st, sizeof(Stamp) * grid, cudaMemcpyDeviceToHost);
          char nm[64];
          std::snprintf(nm, sizeof nm, "%s cps=%d grid=%d", variant == 0 ? "split_f64" : "sum_i64", cps, grid);
          report(nm, h, ms * 1000);
        }
      }
    }
  }
  // back-to-back timing (no per-launch sync), 20 launches, rotated inputs
  for (int variant = 0; variant < 2; ++variant) {
    const int grid = sms * (variant == 0 ? r1 : r2);
    cudaEventRecord(a);
    for (int it = 0; it < 20; ++it) {
      const int c = it % COPIES;
      if (variant == 0) k_split_st<256, 5, 2><<<grid, 256>>>(x + (size_t)c * n, n, part, cnt, out, st);
      else k_i64_st<256, 4><<<grid, 256>>>((const long long*)(x + (size_t)c * n), n, (long long*)part, cnt, (long long*)out, st);
    }
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    std::printf("%s back-to-back: %.2f us per launch\n", variant == 0 ? "split_f64" : "sum_i64", ms * 1000 / 20);
  }
  std::printf("err=%s\n", cudaGetErrorString(cudaDeviceSynchronize()));
  return 0;
}
