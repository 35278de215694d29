// Host -> device bandwidth of the host link on one GPU: 256 MiB copies from
// pinned host memory through the copy engines (one copy, one copy cut into
// 2 / 4 / 8 pieces on as many streams, two copies at once) and through a
// kernel whose threads read the pinned memory directly (16-byte loads, 4 or
// 8 in flight per thread, 1 / 2 / 4 CTAs per SM), then a device -> host copy.
// CUDA events around 10 repetitions of each.  Measurement program only: it
// bounds the end-to-end figure of the bench step, whose inputs cross this
// link every step.
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
//        -o host_link kokkos_gb300/bench_host_link.cu && ./host_link
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#define CK(x) do { cudaError_t ck_ = (x); if (ck_ != cudaSuccess) { printf("err %s line %d\n", cudaGetErrorString(ck_), __LINE__); return 1; } } while (0)

template <int U>
__global__ void __launch_bounds__(256) k_pull(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16) {
  const size_t stride = (size_t)gridDim.x * 256;
  size_t i = (size_t)blockIdx.x * 256 + threadIdx.x;
  for (; i + (U - 1) * stride < n16; i += U * stride) {
    uint4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = src[i + u * stride];
#pragma unroll
    for (int u = 0; u < U; ++u) dst[i + u * stride] = v[u];
  }
  for (; i < n16; i += stride) dst[i] = src[i];
}

int main() {
  const size_t B = 268435456;  // bytes per buffer
  void *h0, *h1, *d0, *d1;
  CK(cudaHostAlloc(&h0, B, cudaHostAllocDefault));
  CK(cudaHostAlloc(&h1, B, cudaHostAllocDefault));
  CK(cudaMalloc(&d0, B));
  CK(cudaMalloc(&d1, B));
  memset(h0, 1, B); memset(h1, 2, B);
  int sms = 0; CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  int ce = 0; CK(cudaDeviceGetAttribute(&ce, cudaDevAttrAsyncEngineCount, 0));
  printf("sms %d async_engines %d\n", sms, ce);
  cudaStream_t s[8];
  for (int i = 0; i < 8; ++i) CK(cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
  std::vector<cudaEvent_t> done(8);
  for (auto& e : done) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  auto run = [&](const char* name, int reps, auto&& body, double bytes) -> int {
    body(); CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(e0, s[0]));
    for (int r = 0; r < reps; ++r) {
      // s[1..7] wait for s[0]'s start, s[0] waits for them at the end
      CK(cudaEventRecord(done[0], s[0]));
      for (int i = 1; i < 8; ++i) CK(cudaStreamWaitEvent(s[i], done[0], 0));
      body();
      for (int i = 1; i < 8; ++i) { CK(cudaEventRecord(done[i], s[i])); CK(cudaStreamWaitEvent(s[0], done[i], 0)); }
    }
    CK(cudaEventRecord(e1, s[0]));
    CK(cudaEventSynchronize(e1));
    float ms = 0; CK(cudaEventElapsedTime(&ms, e0, e1));
    ms /= reps;
    printf("%-40s %8.3f ms  %7.1f GB/s\n", name, ms, bytes / (ms * 1e-3) / 1e9);
    return 0;
  };
  auto chunks = [&](void* d, void* h, size_t bytes, int k, int s_off) {
    const size_t c = (bytes / k + 4095) / 4096 * 4096;
    for (int i = 0; i < k; ++i) {
      const size_t o = (size_t)i * c;
      if (o >= bytes) break;
      const size_t len = o + c <= bytes ? c : bytes - o;
      cudaMemcpyAsync((char*)d + o, (char*)h + o, len, cudaMemcpyHostToDevice, s[(s_off + i) % 8]);
    }
  };
  run("1 copy, 1 stream", 10, [&] { chunks(d0, h0, B, 1, 0); }, B);
  run("1 copy in 2 streams", 10, [&] { chunks(d0, h0, B, 2, 0); }, B);
  run("1 copy in 4 streams", 10, [&] { chunks(d0, h0, B, 4, 0); }, B);
  run("1 copy in 8 streams", 10, [&] { chunks(d0, h0, B, 8, 0); }, B);
  run("2 copies, 2 streams", 10, [&] { chunks(d0, h0, B, 1, 0); chunks(d1, h1, B, 1, 1); }, 2.0 * B);
  run("2 copies, 4+4 streams", 10, [&] { chunks(d0, h0, B, 4, 0); chunks(d1, h1, B, 4, 4); }, 2.0 * B);
  const size_t n16 = B / 16;
  for (int cps : {1, 2, 4}) {
    char nm[64];
    snprintf(nm, 64, "pull kernel U4, %d CTA/SM", cps);
    run(nm, 10, [&] { k_pull<4><<<sms * cps, 256, 0, s[0]>>>((const uint4*)h0, (uint4*)d0, n16); }, B);
    snprintf(nm, 64, "pull kernel U8, %d CTA/SM", cps);
    run(nm, 10, [&] { k_pull<8><<<sms * cps, 256, 0, s[0]>>>((const uint4*)h0, (uint4*)d0, n16); }, B);
  }
  run("pull kernel U8 2 CTA/SM, both buffers", 10, [&] {
    k_pull<8><<<sms * 2, 256, 0, s[0]>>>((const uint4*)h0, (uint4*)d0, n16);
    k_pull<8><<<sms * 2, 256, 0, s[1]>>>((const uint4*)h1, (uint4*)d1, n16); }, 2.0 * B);
  run("copy engine + pull kernel together", 10, [&] {
    chunks(d0, h0, B, 1, 0);
    k_pull<8><<<sms * 2, 256, 0, s[1]>>>((const uint4*)h1, (uint4*)d1, n16); }, 2.0 * B);
  // device -> host, small and large
  run("d2h 256 MiB, 1 stream", 5, [&] { cudaMemcpyAsync(h0, d0, B, cudaMemcpyDeviceToHost, s[0]); }, B);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  // check the pull copies landed
  std::vector<unsigned char> chk(4096);
  CK(cudaMemcpy(chk.data(), (char*)d1 + B - 4096, 4096, cudaMemcpyDeviceToHost));
  printf("check %d\n", (int)chk[100]);
  return 0;
}
