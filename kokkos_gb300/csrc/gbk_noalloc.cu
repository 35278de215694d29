// gbk_reduce_noalloc: the flat reduce (k_reduce_flat) for callers that may
// not allocate device memory.
//
// The regular entry points keep their scratch (one partial value per CTA and
// the last-CTA ticket) in a per-stream workspace that the library creates
// with cudaMalloc on first use.  Some callers cannot allow that: code that
// runs under a device-memory budget owned by someone else (a framework's
// caching allocator that has reserved the GPU's memory, an application that
// forbids allocations after start-up), and latency-critical loops that must
// not hit the implicit device-wide synchronisation cudaMalloc/cudaFree can
// cause.  This entry point uses instead a fixed array in the library's own
// device memory, declared below at file scope; every GPU that loads the
// library holds it until the process exits.
//
// The array is shared by every call on a device and keeps the last call's
// contents.  The ticket must start at zero: the first call on a device
// clears it (cudaMemsetAsync on that call's stream, not an allocation), and
// every launch leaves it at zero again (the last CTA resets it when it
// finishes the reduction).  The partials are written before they are read.
// Calls whose kernels overlap on the GPU (the same device, different streams
// not ordered by events) race on the array and must not be issued.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in).  The first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and keeps
// it; that first call should come before any stream capture.  The address is
// kept for the life of the process: a caller that resets the device
// (cudaDeviceReset) must not call this entry point afterwards, since the
// module and its array are loaded again at a new address.
#include <mutex>

#include "gbk_reduce_impl.cuh"

namespace gbk {
namespace {

constexpr int64_t NOALLOC_MAX_CTAS = 4096;   // partial values per call
constexpr size_t NOALLOC_MAX_VALUE = 32;     // largest reducer value: MinMaxLoc<double>
constexpr size_t NOALLOC_HEADER = 256;       // ticket counter, own 256-byte line
constexpr size_t NOALLOC_BYTES = NOALLOC_HEADER + (size_t)NOALLOC_MAX_CTAS * NOALLOC_MAX_VALUE;  // 128 KiB + 256 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_na_mu;
char* g_na_base[64] = {};

// Set-up, once per device with that device current: the array's device
// address, and the ticket line cleared on the first caller's stream.
int noalloc_base(char** out, cudaStream_t s) {
  int dev = 0;
  GBK_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return GBK_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_base[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return e != cudaSuccess ? cuda_status(e) : GBK_ERR_CUDA;
    GBK_CUDA_TRY(cudaMemsetAsync(p, 0, NOALLOC_HEADER, s));
    g_na_base[dev] = (char*)p;
  }
  *out = g_na_base[dev];
  return GBK_OK;
}

// Same launch shape as launch_flat<R, T, 256, 4> (the default configuration
// of gbk_reduce), with the scratch taken from the fixed array.
template <class R, class T>
int noalloc_flat(const T* x, int64_t n, void* out, cudaStream_t s, int ctas_per_sm) {
  using V = typename R::V;
  constexpr int BLOCK = 256, UNROLL = 4;
  if (sizeof(V) > NOALLOC_MAX_VALUE) return GBK_ERR_SCRATCH_LIMIT;
  if (n <= 0) {
    k_write_identity<R><<<1, 32, 0, s>>>((V*)out);
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  constexpr int VEC = 16 / sizeof(T);
  const uintptr_t a = (uintptr_t)x;
  int64_t head = (int64_t)(((16 - (a & 15)) & 15) / sizeof(T));
  if (head > n) head = n;
  const int64_t nvec = (n - head) / VEC;
  const int64_t tiles = (nvec + (int64_t)BLOCK * UNROLL - 1) / ((int64_t)BLOCK * UNROLL);
  int64_t grid = (int64_t)sm_count() * (ctas_per_sm > 0 ? ctas_per_sm : 8);
  if (grid > tiles) grid = tiles;
  if (grid < 1) grid = 1;
  const int64_t tail = (n - head) - nvec * VEC;
  while (grid * BLOCK < head || grid * BLOCK < tail) ++grid;
  if (grid > NOALLOC_MAX_CTAS) return GBK_ERR_SCRATCH_LIMIT;
  char* base = nullptr;
  const int st = noalloc_base(&base, s);
  if (st) return st;
  unsigned* ticket = (unsigned*)base;  // zero here: cleared at set-up, reset by every launch's last CTA
  V* partials = (V*)(base + NOALLOC_HEADER);
  k_reduce_flat<R, T, BLOCK, UNROLL><<<(unsigned)grid, BLOCK, 0, s>>>(x, n, head, 0, partials, ticket, (V*)out);
  note_launch();
  return cuda_status(cudaGetLastError());
}

template <class T>
int noalloc_typed(int op, const T* x, int64_t n, void* out, cudaStream_t s, int cps) {
  constexpr bool INT = !(std::is_same<T, float>::value || std::is_same<T, double>::value);
  switch (op) {
    case GBK_SUM: return noalloc_flat<RSum<T>, T>(x, n, out, s, cps);
    case GBK_PROD: return noalloc_flat<RProd<T>, T>(x, n, out, s, cps);
    case GBK_MIN: return noalloc_flat<RMin<T>, T>(x, n, out, s, cps);
    case GBK_MAX: return noalloc_flat<RMax<T>, T>(x, n, out, s, cps);
    case GBK_MINLOC: return noalloc_flat<RMinLoc<T>, T>(x, n, out, s, cps);
    case GBK_MAXLOC: return noalloc_flat<RMaxLoc<T>, T>(x, n, out, s, cps);
    case GBK_MINMAX: return noalloc_flat<RMinMax<T>, T>(x, n, out, s, cps);
    case GBK_MINMAXLOC: return noalloc_flat<RMinMaxLoc<T>, T>(x, n, out, s, cps);
    default: break;
  }
  if constexpr (INT) {
    switch (op) {
      case GBK_LAND: return noalloc_flat<RLAnd<T>, T>(x, n, out, s, cps);
      case GBK_LOR: return noalloc_flat<RLOr<T>, T>(x, n, out, s, cps);
      case GBK_BAND: return noalloc_flat<RBAnd<T>, T>(x, n, out, s, cps);
      case GBK_BOR: return noalloc_flat<RBOr<T>, T>(x, n, out, s, cps);
      default: break;
    }
  }
  return GBK_ERR_UNSUPPORTED;
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" int gbk_reduce_noalloc(gbk_reducer_t op, gbk_dtype_t dt, const void* x, int64_t n, void* result,
                                  gbk_stream_t stream, int32_t ctas_per_sm) {
  if (op < GBK_SUM || op > GBK_MINMAXLOC || dt < GBK_I32 || dt > GBK_F64) return GBK_ERR_UNSUPPORTED;
  if ((dt == GBK_F32 || dt == GBK_F64) && op >= GBK_LAND && op <= GBK_BOR) return GBK_ERR_UNSUPPORTED;
  if (n < 0 || !result || (n > 0 && !x) || ctas_per_sm < 0) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)x % dtype_size(dt)) return GBK_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  switch (dt) {
    case GBK_I32: return noalloc_typed<int32_t>(op, (const int32_t*)x, n, result, s, ctas_per_sm);
    case GBK_I64: return noalloc_typed<int64_t>(op, (const int64_t*)x, n, result, s, ctas_per_sm);
    case GBK_U32: return noalloc_typed<uint32_t>(op, (const uint32_t*)x, n, result, s, ctas_per_sm);
    case GBK_U64: return noalloc_typed<uint64_t>(op, (const uint64_t*)x, n, result, s, ctas_per_sm);
    case GBK_F32: return noalloc_typed<float>(op, (const float*)x, n, result, s, ctas_per_sm);
    case GBK_F64: return noalloc_typed<double>(op, (const double*)x, n, result, s, ctas_per_sm);
  }
  return GBK_ERR_UNSUPPORTED;
}
