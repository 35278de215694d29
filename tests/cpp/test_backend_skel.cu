// The kernel skeletons of the GB300 Kokkos backend
// (include/gb300_backend/GB300/Kokkos_GB300_Skeletons.hpp) on the GPU, without
// the Kokkos headers: the closures below have the shape the backend's pattern
// specialisations build from a Kokkos functor and its FunctorAnalysis reducer
// (pointer-based init / join / final on an opaque value, the functor called as
// f(i, update) or f(i, update, final_pass)), so these checks cover the device
// code every parallel_for / parallel_reduce / parallel_scan / TeamPolicy
// launch on the GB300 space runs.  Each check compares with a host
// computation and prints "ok <name>" or "FAIL <name>".
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gb300_backend/GB300/Kokkos_GB300_Skeletons.hpp"

using namespace gbk_skel;

static int g_fail = 0;
static void report(bool ok, const char* name) {
  std::printf("%s %s\n", ok ? "ok" : "FAIL", name);
  if (!ok) ++g_fail;
}
#define CK(x)                                                                   \
  do {                                                                          \
    cudaError_t e_ = (x);                                                       \
    if (e_ != cudaSuccess) {                                                    \
      std::printf("FAIL cuda %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return;                                                                   \
    }                                                                           \
  } while (0)
#define GK(x)                                                             \
  do {                                                                    \
    int s_ = (x);                                                         \
    if (s_ != GBK_OK) {                                                   \
      std::printf("FAIL gbk %s at %s:%d\n", gbk_status_string(s_), __FILE__, __LINE__); \
      return;                                                             \
    }                                                                     \
  } while (0)

struct Ws {
  char* base;
  unsigned* ctr;
  int* err;
};
static Ws ws(cudaStream_t s, size_t bytes) {
  Ws w{};
  void* p = nullptr;
  gbk_workspace_acquire((gbk_stream_t)s, (int64_t)bytes, &p, &w.ctr, &w.err);
  w.base = (char*)p;
  return w;
}

// ---- closures in the shape of the backend's adapters ----------------------
struct SumD {  // Sum<double>: the reducer's algebra + functor u += x(i)
  const double* x;
  __device__ void init(void* v) const { *(double*)v = 0.0; }
  __device__ void join(void* d, const void* s) const { *(double*)d += *(const double*)s; }
  __device__ void final_(void*) const {}
  __device__ void exec(int64_t i, void* v) const { *(double*)v += x[i]; }
};
struct Moments {  // array reduction, runtime count 3 (value_type double[])
  const double* x;
  __device__ void init(void* v) const {
    double* a = (double*)v;
    a[0] = a[1] = a[2] = 0.0;
  }
  __device__ void join(void* d, const void* s) const {
    for (int k = 0; k < 3; ++k) ((double*)d)[k] += ((const double*)s)[k];
  }
  __device__ void final_(void*) const {}
  __device__ void exec(int64_t i, void* v) const {
    double* a = (double*)v;
    a[0] += x[i];
    a[1] += x[i] * x[i];
    a[2] += 1.0;
  }
};
struct MinLocI {  // MinLoc<int, int64>: ties keep the smaller loc
  const int* x;
  struct V {
    int val;
    int64_t loc;
  };
  __device__ void init(void* v) const { *(V*)v = V{INT32_MAX, INT64_MAX}; }
  __device__ void join(void* d, const void* s) const {
    V& a = *(V*)d;
    const V& b = *(const V*)s;
    if (b.val < a.val || (b.val == a.val && b.loc < a.loc)) a = b;
  }
  __device__ void final_(void*) const {}
  __device__ void exec(int64_t i, void* v) const {
    V& a = *(V*)v;
    if (x[i] < a.val) a = V{x[i], i};
  }
};
struct MeanD : SumD {  // a reducer with final(): the mean, count in the second word
  __device__ void init(void* v) const { ((double*)v)[0] = ((double*)v)[1] = 0.0; }
  __device__ void join(void* d, const void* s) const {
    ((double*)d)[0] += ((const double*)s)[0];
    ((double*)d)[1] += ((const double*)s)[1];
  }
  __device__ void final_(void* v) const { ((double*)v)[0] /= ((double*)v)[1]; }
  __device__ void exec(int64_t i, void* v) const {
    ((double*)v)[0] += x[i];
    ((double*)v)[1] += 1.0;
  }
};
struct Fill {
  double* y;
  __device__ void exec(int64_t i) const { y[i] = 0.5 * (double)(i % 7); }
};
struct ExScan {  // exclusive scan functor: if (final) y(i) = u; u += x(i)
  const int32_t* x;
  int64_t* y;
  __device__ void init(void* v) const { *(int64_t*)v = 0; }
  __device__ void join(void* d, const void* s) const { *(int64_t*)d += *(const int64_t*)s; }
  __device__ void final_(void*) const {}
  __device__ void exec(int64_t i, void* v, bool fin) const {
    if (fin) y[i] = *(int64_t*)v;
    *(int64_t*)v += x[i];
  }
};
struct TeamRows {  // each team sums its row; thread order strided by team size
  const double* a;
  double* rows;
  int len;
  __device__ void init(void* v) const { *(double*)v = 0.0; }
  __device__ void join(void* d, const void* s) const { *(double*)d += *(const double*)s; }
  __device__ void final_(void*) const {}
  __device__ void exec_team(int64_t lr, int64_t, unsigned char* sm, void* v) const {
    double s = 0;
    for (int j = threadIdx.x; j < len; j += blockDim.x) s += a[lr * len + j];
    *(double*)v += s;
    // a team-wide sum through the team's shared memory (the level-0 scratch)
    double* buf = (double*)sm;
    buf[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int k = 0; k < (int)blockDim.x; ++k) t += buf[k];
      rows[lr] = t;
    }
    __syncthreads();
  }
};

template <int VB, class C>
static bool run_reduce(cudaStream_t s, const C& c, int64_t n, void* host_out, size_t bytes) {
  const int64_t g = std::min<int64_t>(std::max<int64_t>((n + kBlock - 1) / kBlock, 1), 152 * 8);
  Ws w = ws(s, 256 + (g + 1) * sizeof(Val<VB>));
  Val<VB>* out = (Val<VB>*)(w.base + 256);
  k_reduce<VB, C><<<(unsigned)g, kBlock, 0, s>>>(c, 0, n, out + 1, w.ctr + kSlotReduce, out, w.err);
  if (cudaMemcpyAsync(host_out, out, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return false;
  return gbk_stream_check((gbk_stream_t)s) == GBK_OK;
}

static void reduce_and_for() {
  cudaStream_t s;
  CK(cudaStreamCreate(&s));
  for (int64_t n : {int64_t(0), int64_t(1), int64_t(1000), int64_t((1 << 22) + 77)}) {
    double* x = nullptr;
    CK(cudaMalloc(&x, (n > 0 ? n : 1) * sizeof(double)));
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>((n + kBlock - 1) / kBlock, 152 * 8));
    if (n > 0) k_for<Fill><<<(unsigned)g, kBlock, 0, s>>>(Fill{x}, 0, n, nullptr);
    double want = 0, sq = 0;
    for (int64_t i = 0; i < n; ++i) {
      want += 0.5 * (i % 7);
      sq += 0.25 * (i % 7) * (i % 7);
    }
    double got = -1;
    bool ok = run_reduce<16>(s, SumD{x}, n, &got, sizeof(double));
    char nm[64];
    std::snprintf(nm, sizeof nm, "skel_for_reduce_sum_n%lld", (long long)n);
    report(ok && got == want, nm);
    double mom[3] = {-1, -1, -1};
    ok = run_reduce<kMaxValueBytes>(s, Moments{x}, n, mom, sizeof mom);
    std::snprintf(nm, sizeof nm, "skel_array_reduce_n%lld", (long long)n);
    report(ok && mom[0] == want && mom[1] == sq && mom[2] == (double)n, nm);
    if (n > 0) {
      double mean[2];
      MeanD m;
      m.x = x;
      ok = run_reduce<16>(s, m, n, mean, sizeof mean);
      std::snprintf(nm, sizeof nm, "skel_reduce_final_n%lld", (long long)n);
      report(ok && std::fabs(mean[0] - want / n) <= 1e-12 * (want / n + 1e-300), nm);
    }
    CK(cudaFree(x));
  }
  // MinLoc with ties: the smallest loc of the minimum
  const int n = 3000001;
  std::vector<int> h(n);
  for (int i = 0; i < n; ++i) h[i] = (int)((i * 7919LL) % 100003) + 10;
  h[123457] = 1;
  h[2999000] = 1;
  int* dx = nullptr;
  CK(cudaMalloc(&dx, n * sizeof(int)));
  CK(cudaMemcpy(dx, h.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  MinLocI::V r{};
  const bool ok = run_reduce<16>(s, MinLocI{dx}, n, &r, sizeof r);
  report(ok && r.val == 1 && r.loc == 123457, "skel_reduce_minloc_ties");
  CK(cudaFree(dx));
  CK(cudaStreamDestroy(s));
}

static void scans() {
  cudaStream_t s;
  CK(cudaStreamCreate(&s));
  for (int64_t n : {int64_t(1), int64_t(2047), int64_t(2048), int64_t(5 * 2048 + 3), int64_t(1 << 24)}) {
    std::vector<int32_t> hx(n);
    for (int64_t i = 0; i < n; ++i) hx[i] = (int32_t)((i * 37) % 16);
    int32_t* x = nullptr;
    int64_t* y = nullptr;
    CK(cudaMalloc(&x, n * 4));
    CK(cudaMalloc(&y, n * 8));
    CK(cudaMemcpy(x, hx.data(), n * 4, cudaMemcpyHostToDevice));
    constexpr int64_t TILE = (int64_t)kBlock * kItems;
    const int64_t nt = (n + TILE - 1) / TILE;
    const size_t fb = ((size_t)nt * 4 + 255) / 256 * 256, vb = ((size_t)nt * sizeof(Val<16>) + 255) / 256 * 256;
    Ws w = ws(s, 256 + fb + 2 * vb);
    ScanState<16> S;
    S.flags = (unsigned*)(w.base + 256);
    S.agg = (Val<16>*)(w.base + 256 + fb);
    S.incl = (Val<16>*)(w.base + 256 + fb + vb);
    S.ticket = w.ctr + kSlotScan;
    S.err = w.err;
    S.ntiles = nt;
    S.wait_limit = gbk_wait_limit();
    CK(cudaMemsetAsync(S.flags, 0, nt * 4, s));
    Val<16>* tot = (Val<16>*)w.base;
    k_scan<16, ExScan><<<(unsigned)nt, kBlock, 0, s>>>(ExScan{x, y}, 0, n, S, tot);
    int64_t total = -1;
    CK(cudaMemcpyAsync(&total, tot, 8, cudaMemcpyDeviceToHost, s));
    GK(gbk_stream_check((gbk_stream_t)s));
    std::vector<int64_t> hy(n);
    CK(cudaMemcpy(hy.data(), y, n * 8, cudaMemcpyDeviceToHost));
    int64_t run = 0;
    bool ok = true;
    for (int64_t i = 0; i < n; ++i) {
      ok &= hy[i] == run;
      run += hx[i];
    }
    char nm[64];
    std::snprintf(nm, sizeof nm, "skel_scan_exclusive_total_n%lld", (long long)n);
    report(ok && total == run, nm);
    CK(cudaFree(x));
    CK(cudaFree(y));
  }
  CK(cudaStreamDestroy(s));
}

static void teams() {
  cudaStream_t s;
  CK(cudaStreamCreate(&s));
  const int league = 5000, len = 777;
  std::vector<double> ha((size_t)league * len);
  for (int i = 0; i < league; ++i)
    for (int j = 0; j < len; ++j) ha[(size_t)i * len + j] = (i + j) % 5;
  double *a = nullptr, *rows = nullptr;
  CK(cudaMalloc(&a, ha.size() * 8));
  CK(cudaMalloc(&rows, league * 8));
  CK(cudaMemcpy(a, ha.data(), ha.size() * 8, cudaMemcpyHostToDevice));
  double want = 0;
  for (double v : ha) want += v;
  for (int ts : {128, 100, 33, 1}) {
    const int shmem = ts * 8;
    const int64_t g = std::min<int64_t>(league, 152 * (2048 / ts));
    Ws w = ws(s, 256 + (g + 1) * sizeof(Val<16>));
    Val<16>* out = (Val<16>*)(w.base + 256);
    k_team_reduce<16, TeamRows><<<(unsigned)g, ts, shmem, s>>>(TeamRows{a, rows, len}, league, out + 1,
                                                               w.ctr + kSlotReduce, out, w.err);
    double got = -1;
    CK(cudaMemcpyAsync(&got, out, 8, cudaMemcpyDeviceToHost, s));
    GK(gbk_stream_check((gbk_stream_t)s));
    std::vector<double> hr(league);
    CK(cudaMemcpy(hr.data(), rows, league * 8, cudaMemcpyDeviceToHost));
    bool ok = got == want;
    for (int i = 0; i < league; ++i) {
      double r = 0;
      for (int j = 0; j < len; ++j) r += ha[(size_t)i * len + j];
      ok &= hr[i] == r;
    }
    char nm[64];
    std::snprintf(nm, sizeof nm, "skel_team_reduce_team%d", ts);
    report(ok, nm);
  }
  CK(cudaFree(a));
  CK(cudaFree(rows));
  CK(cudaStreamDestroy(s));
}

int main() {
  reduce_and_for();
  scans();
  teams();
  std::printf("%d failures\n", g_fail);
  return g_fail;
}
