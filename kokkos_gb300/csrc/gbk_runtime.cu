// Runtime of libgbk: per-stream workspaces, the device error word, device
// queries, wait limits and the launch counter.
//
// One Workspace per (device, stream), created on first use and guarded by
// its own mutex; launches on one stream are serialised by the stream, as
// the reference serialises kernels on one OpenMP instance with its instance
// mutex (core/src/OpenMP/Kokkos_OpenMP_Parallel_Reduce.hpp:87).
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <cstdlib>
#include <mutex>
#include <utility>
#include <vector>

#include "gbk_internal.cuh"

namespace gbk {

namespace {
std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, Workspace*> g_ws;
std::atomic<int64_t> g_launches{0};
std::atomic<int64_t> g_wait_limit{int64_t(1) << 22};  // polls with ~256 ns back-off: about a second
int g_sm[64];
bool g_sm_init[64];

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
  return st != cudaStreamCaptureStatusNone;
}
}  // namespace

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return GBK_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GBK_ERR_NO_DEVICE;
  return GBK_ERR_CUDA;
}

int sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev < 0 || dev >= 64) return 0;
  if (!g_sm_init[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    g_sm[dev] = v;
    g_sm_init[dev] = true;
  }
  return g_sm[dev];
}

int64_t wait_limit() { return g_wait_limit.load(); }

bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBK_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}
void note_launch(int64_t k) { g_launches += k; }

Workspace* ws_get(cudaStream_t s, int* status) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { *status = cuda_status(e); return nullptr; }
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(dev, s);
  auto it = g_ws.find(key);
  if (it != g_ws.end()) return it->second;
  if (capturing(s)) { *status = GBK_ERR_OUT_OF_WORKSPACE; return nullptr; }
  Workspace* w = new Workspace();
  w->stream = s;
  w->device = dev;
  void* p = nullptr;
  e = cudaMalloc(&p, 64 * sizeof(unsigned) + 256);
  if (e != cudaSuccess) { delete w; *status = cuda_status(e); return nullptr; }
  e = cudaMemset(p, 0, 64 * sizeof(unsigned) + 256);
  if (e != cudaSuccess) { cudaFree(p); delete w; *status = cuda_status(e); return nullptr; }
  w->counters = (unsigned*)p;
  w->err = (int*)((char*)p + 64 * sizeof(unsigned));
  g_ws[key] = w;
  return w;
}

static char* grow(Workspace* w, char** buf, size_t* have, size_t bytes, int* status) {
  if (bytes <= *have) return *buf;
  if (capturing(w->stream)) { *status = GBK_ERR_OUT_OF_WORKSPACE; return nullptr; }
  // The old buffer may still be in use by queued work on this stream.
  cudaError_t e = cudaStreamSynchronize(w->stream);
  if (e != cudaSuccess) { *status = cuda_status(e); return nullptr; }
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  size_t want = bytes + bytes / 4 + (1u << 20);
  void* p = nullptr;
  e = cudaMalloc(&p, want);
  if (e != cudaSuccess) { *status = cuda_status(e); return nullptr; }
  // Scratch starts zeroed: tile-status words rely on it.
  e = cudaMemset(p, 0, want);
  if (e != cudaSuccess) { cudaFree(p); *status = cuda_status(e); return nullptr; }
  *buf = (char*)p;
  *have = want;
  return *buf;
}

char* ws_scratch(Workspace* w, size_t bytes, int* status) {
  return grow(w, &w->scratch, &w->scratch_bytes, bytes, status);
}
char* ws_stage(Workspace* w, size_t bytes, int* status) { return grow(w, &w->stage, &w->stage_bytes, bytes, status); }

// Look-back status words.  Uncaptured launches tag their words with a fresh
// 30-bit epoch (2, 3, ...; a wrap clears the buffer), so no clearing is
// needed per launch.  A launch being captured into a CUDA graph replays with
// the same arguments every time, so it clears its words with a memset node
// and uses the reserved epoch 1, which uncaptured launches never use.
unsigned* ws_flags(Workspace* w, size_t count, unsigned* epoch, int* status) {
  char* f = grow(w, &w->flags, &w->flags_bytes, count * sizeof(unsigned), status);
  if (!f) return nullptr;
  if (capturing(w->stream)) {
    cudaError_t e = cudaMemsetAsync(f, 0, count * sizeof(unsigned), w->stream);
    if (e != cudaSuccess) { *status = cuda_status(e); return nullptr; }
    *epoch = 1;
    return (unsigned*)f;
  }
  w->epoch = (w->epoch + 1) & 0x3FFFFFFFu;
  if (w->epoch < 2) {
    cudaError_t e = cudaMemsetAsync(f, 0, w->flags_bytes, w->stream);
    if (e != cudaSuccess) { *status = cuda_status(e); return nullptr; }
    w->epoch = 2;
  }
  *epoch = w->epoch;
  return (unsigned*)f;
}

}  // namespace gbk

namespace gbk {
namespace {
// deep_copy(view, value): 16-byte streaming stores of a pattern that repeats
// the value (its size divides 16, so every aligned vector holds whole
// values in phase); grid-stride over the vectors.
__global__ void k_fill16(uint4* __restrict__ d, int64_t nvec, uint4 pat) {
  pdl_entry();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvec; i += stride) __stcs(d + i, pat);
}
// The elements before the first and after the last whole vector: element e
// of [0, nhead) at head, of [nhead, nhead + ntail) at tail.
__global__ void k_fill_edges(unsigned char* head, int64_t nhead, unsigned char* tail, int64_t ntail, int eb,
                             uint4 pat) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nhead + ntail) return;
  unsigned char* p = e < nhead ? head + e * eb : tail + (e - nhead) * eb;
  const unsigned char* v = reinterpret_cast<const unsigned char*>(&pat);
  switch (eb) {
    case 1: *p = v[0]; break;
    case 2: *reinterpret_cast<unsigned short*>(p) = *reinterpret_cast<const unsigned short*>(v); break;
    case 4: *reinterpret_cast<unsigned*>(p) = pat.x; break;
    default: *reinterpret_cast<unsigned long long*>(p) = *reinterpret_cast<const unsigned long long*>(v); break;
  }
}
}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_version(void) { return 100; }

const char* gbk_status_string(int s) {
  switch (s) {
    case GBK_OK: return "ok";
    case GBK_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GBK_ERR_UNSUPPORTED: return "unsupported reducer/dtype combination";
    case GBK_ERR_CUDA: return "CUDA error";
    case GBK_ERR_DEVICE_TIMEOUT: return "device-side wait exceeded its bound";
    case GBK_ERR_OUT_OF_WORKSPACE: return "workspace too small (reserve it before stream capture)";
    case GBK_ERR_KEY_OUT_OF_RANGE: return "key outside the bin range (skipped)";
    case GBK_ERR_NO_DEVICE: return "no CUDA device";
    case GBK_ERR_DEVICE_ABORT: return "a kernel called abort in device code";
    case GBK_ERR_SCRATCH_LIMIT: return "request needs more CTAs than the fixed scratch of gbk_reduce_noalloc holds (4096)";
  }
  return "unknown status";
}

int gbk_device_info(int* sm, int* major, int* minor, int64_t* l2) {
  int dev = 0;
  GBK_CUDA_TRY(cudaGetDevice(&dev));
  int v = 0;
  if (sm) { GBK_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev)); *sm = v; }
  if (major) { GBK_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, dev)); *major = v; }
  if (minor) { GBK_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, dev)); *minor = v; }
  if (l2) { GBK_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev)); *l2 = v; }
  return GBK_OK;
}

int gbk_stream_check(gbk_stream_t stream) { return gbk_fence_read(stream, nullptr, nullptr, 0); }

int gbk_fence_read(gbk_stream_t stream, const void* device_src, void* host_dst, int64_t bytes) {
  if (bytes < 0 || bytes > 256 || (bytes > 0 && (!device_src || !host_dst))) return GBK_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  int st = GBK_OK;
  Workspace* w = ws_get(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->slot_mu);
  if (!w->host_slot) {
    void* p = nullptr;
    GBK_CUDA_TRY(cudaHostAlloc(&p, 512, cudaHostAllocDefault));
    w->host_slot = (char*)p;
  }
  // Both copies queue behind all earlier work on the stream, so the error
  // word holds every status the stream's kernels raised; one synchronisation.
  if (bytes) GBK_CUDA_TRY(cudaMemcpyAsync(w->host_slot + 256, device_src, (size_t)bytes, cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaMemcpyAsync(w->host_slot, w->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  int bits = 0;
  std::memcpy(&bits, w->host_slot, sizeof(int));
  if (bytes) std::memcpy(host_dst, w->host_slot + 256, (size_t)bytes);
  if (bits) {
    GBK_CUDA_TRY(cudaMemsetAsync(w->err, 0, sizeof(int), s));
    // After a timed-out wait the ticket counters may be left non-zero.
    if (bits & (GBK_EBIT_TIMEOUT | GBK_EBIT_BAD_STATE)) {
      GBK_CUDA_TRY(cudaMemsetAsync(w->counters, 0, 64 * sizeof(unsigned), s));
      if (w->scratch) GBK_CUDA_TRY(cudaMemsetAsync(w->scratch, 0, w->scratch_bytes, s));
    }
    GBK_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (bits & GBK_EBIT_TIMEOUT) return GBK_ERR_DEVICE_TIMEOUT;
  if (bits & GBK_EBIT_BAD_STATE) return GBK_ERR_CUDA;
  if (bits & GBK_EBIT_KEY_RANGE) return GBK_ERR_KEY_OUT_OF_RANGE;
  if (bits & GBK_EBIT_ABORT) return GBK_ERR_DEVICE_ABORT;
  return GBK_OK;
}

int gbk_workspace_reserve(gbk_stream_t stream, int64_t bytes) {
  if (bytes < 0) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  if (!ws_scratch(w, (size_t)bytes, &st)) return st;
  // Status words: a scan keeps two values of up to 8 bytes per tile in
  // scratch and one 4-byte status word, so a quarter of the scratch size
  // covers every launch the scratch can serve.
  if (!grow(w, &w->flags, &w->flags_bytes, (size_t)bytes / 4 + 4096, &st)) return st;
  return GBK_OK;
}

int gbk_workspace_release_all(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_ws) {
    Workspace* w = kv.second;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(w->device);
    cudaStreamSynchronize(w->stream);
    if (w->counters) cudaFree(w->counters);
    if (w->scratch) cudaFree(w->scratch);
    if (w->stage) cudaFree(w->stage);
    if (w->flags) cudaFree(w->flags);
    cudaSetDevice(cur);
    delete w;
  }
  g_ws.clear();
  return GBK_OK;
}

int gbk_workspace_acquire(gbk_stream_t stream, int64_t scratch_bytes, void** scratch, unsigned** counters,
                          int** error_word) {
  if (scratch_bytes < 0) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  char* s = ws_scratch(w, (size_t)(scratch_bytes > 0 ? scratch_bytes : 1), &st);
  if (!s) return st;
  if (scratch) *scratch = s;
  if (counters) *counters = w->counters;
  if (error_word) *error_word = w->err;
  return GBK_OK;
}

int gbk_note_launches(int64_t count) {
  if (count < 0) return GBK_ERR_INVALID_ARGUMENT;
  note_launch(count);
  return GBK_OK;
}

int gbk_set_wait_limit(int64_t polls) {
  if (polls < 1) return GBK_ERR_INVALID_ARGUMENT;
  g_wait_limit = polls;
  return GBK_OK;
}

int64_t gbk_wait_limit(void) { return g_wait_limit.load(); }

int64_t gbk_launch_count(void) { return g_launches.load(); }

int gbk_deep_copy(void* dst, const void* src, int64_t bytes, gbk_stream_t stream) {
  if (bytes < 0 || (bytes > 0 && (!dst || !src))) return GBK_ERR_INVALID_ARGUMENT;
  if (bytes == 0) return GBK_OK;
  GBK_CUDA_TRY(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, (cudaStream_t)stream));
  return GBK_OK;
}

struct gbk_graph_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t kernels = 0;  // kernel nodes, added to the launch count per replay
};

int gbk_graph_begin(gbk_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!s) return GBK_ERR_INVALID_ARGUMENT;  // the legacy stream cannot be captured
  GBK_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  return GBK_OK;
}

int gbk_graph_end(gbk_stream_t stream, gbk_graph_t* out) {
  if (!out) return GBK_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaGraph_t g = nullptr;
  GBK_CUDA_TRY(cudaStreamEndCapture((cudaStream_t)stream, &g));
  cudaGraphExec_t e = nullptr;
  cudaError_t err = cudaGraphInstantiate(&e, g, 0);
  if (err != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_status(err);
  }
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  int64_t kernels = 0;
  if (nn) {
    std::vector<cudaGraphNode_t> nodes(nn);
    cudaGraphGetNodes(g, nodes.data(), &nn);
    for (size_t i = 0; i < nn; ++i) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
    }
  }
  // The captured launches were counted once at capture; count replays only.
  g_launches -= kernels;
  gbk_graph_s* h = new gbk_graph_s();
  h->graph = g;
  h->exec = e;
  h->kernels = kernels;
  *out = h;
  return GBK_OK;
}

int gbk_graph_launch(gbk_graph_t h, gbk_stream_t stream) {
  if (!h || !h->exec) return GBK_ERR_INVALID_ARGUMENT;
  GBK_CUDA_TRY(cudaGraphLaunch(h->exec, (cudaStream_t)stream));
  g_launches += h->kernels;
  return GBK_OK;
}

int gbk_graph_destroy(gbk_graph_t h) {
  if (!h) return GBK_OK;
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  delete h;
  return GBK_OK;
}

int gbk_memset(void* dst, int value, int64_t bytes, gbk_stream_t stream) {
  if (bytes < 0 || (bytes > 0 && !dst)) return GBK_ERR_INVALID_ARGUMENT;
  if (bytes == 0) return GBK_OK;
  GBK_CUDA_TRY(cudaMemsetAsync(dst, value, (size_t)bytes, (cudaStream_t)stream));
  return GBK_OK;
}

int gbk_fill(void* dst, const void* value, int elem_bytes, int64_t n, gbk_stream_t stream) {
  if (n < 0 || !value || (elem_bytes != 1 && elem_bytes != 2 && elem_bytes != 4 && elem_bytes != 8 && elem_bytes != 16))
    return GBK_ERR_INVALID_ARGUMENT;
  if (n == 0) return GBK_OK;
  if (!dst || (uintptr_t)dst % (uintptr_t)elem_bytes) return GBK_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  uint4 pat;
  unsigned char* pb = reinterpret_cast<unsigned char*>(&pat);
  for (int o = 0; o < 16; o += elem_bytes) std::memcpy(pb + o, value, (size_t)elem_bytes);
  unsigned char* d = (unsigned char*)dst;
  int64_t nhead = (int64_t)(((16 - ((uintptr_t)d & 15)) & 15) / (uintptr_t)elem_bytes);
  if (nhead > n) nhead = n;
  const int64_t body_bytes = (n - nhead) * elem_bytes;
  const int64_t nvec = body_bytes / 16;
  const int64_t ntail = (body_bytes - nvec * 16) / elem_bytes;
  unsigned char* body = d + nhead * elem_bytes;
  if (nvec > 0) {
    int64_t grid = (nvec + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 8;
    if (grid > cap) grid = cap;
    GBK_CUDA_TRY(launch_pdl(k_fill16, dim3((unsigned)grid), dim3(256), 0, s, reinterpret_cast<uint4*>(body), nvec, pat));
    note_launch();
  }
  if (nhead + ntail > 0) {
    k_fill_edges<<<(unsigned)((nhead + ntail + 255) / 256), 256, 0, s>>>(d, nhead, body + nvec * 16, ntail,
                                                                          elem_bytes, pat);
    note_launch();
    GBK_CUDA_TRY(cudaGetLastError());
  }
  return GBK_OK;
}

}  // extern "C"
