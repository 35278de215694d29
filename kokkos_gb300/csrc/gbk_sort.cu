// Stable LSD radix sort (onesweep: Adinets & Merrill, "Onesweep: A Faster
// Least Significant Digit Radix Sort for GPUs", 2022), sort_by_key and
// BinSort.  Replaces Kokkos::sort / Experimental::sort_by_key on a device
// space (algorithms/src/sorting/Kokkos_SortPublicAPI.hpp:31-196,
// Kokkos_SortByKeyPublicAPI.hpp:30-114; the reference CUDA path calls
// thrust::sort / thrust::sort_by_key, impl/Kokkos_SortImpl.hpp:204-219,
// impl/Kokkos_SortByKeyImpl.hpp:125-138) and BinSort
// (algorithms/src/sorting/Kokkos_BinSortPublicAPI.hpp:27-408).
//
// Sorting is by the key's radix image: unsigned keys as is, signed keys with
// the sign bit flipped, IEEE floats with all bits flipped when negative and
// the sign bit flipped otherwise (so -0.0 sorts before +0.0).  Keys are
// moved with their original bits.
//
// 1. k_digit_hist: one read of the keys builds the 256-bin histogram of every
//    8-bit digit position (shared-memory counters, a warp that sees one digit
//    in all lanes adds once).  The host reads the KB*256 counts back (one
//    16 KiB copy and a stream sync per sort) and skips every pass whose digit
//    is the same for all keys.
// 2. k_onesweep (one launch per remaining pass): tiles of BLOCK*KPT keys in
//    ticket order.  Each warp ranks its keys row by row with eight ballots
//    per row (lanes holding the same digit), keeping per-warp digit counters
//    in shared memory, so the rank of a key is its position among equal
//    digits: the pass is stable.  The tile's 256 digit counts are published
//    for a per-digit decoupled look-back (one status word per tile and
//    digit: 2 flag bits + 30 count bits, single-copy atomic), giving each
//    digit's global start; the tile is reordered by digit in shared memory
//    and written out in runs.  Waits are bounded.
#include <algorithm>
#include <vector>

#include "gbk_internal.cuh"

namespace gbk {
namespace {

constexpr unsigned SF_A = 1u << 30;  // aggregate
constexpr unsigned SF_P = 2u << 30;  // inclusive prefix
constexpr unsigned SF_MASK = 3u << 30;
constexpr unsigned SV_MASK = (1u << 30) - 1;

// radix images
template <int DT> struct Radix;
template <> struct Radix<GBK_U32> { using K = uint32_t; __device__ static uint32_t img(uint32_t k) { return k; } };
template <> struct Radix<GBK_U64> { using K = uint64_t; __device__ static uint64_t img(uint64_t k) { return k; } };
template <> struct Radix<GBK_I32> { using K = uint32_t; __device__ static uint32_t img(uint32_t k) { return k ^ 0x80000000u; } };
template <> struct Radix<GBK_I64> { using K = uint64_t; __device__ static uint64_t img(uint64_t k) { return k ^ 0x8000000000000000ull; } };
template <> struct Radix<GBK_F32> {
  using K = uint32_t;
  __device__ static uint32_t img(uint32_t k) { return (k & 0x80000000u) ? ~k : (k | 0x80000000u); }
};
template <> struct Radix<GBK_F64> {
  using K = uint64_t;
  __device__ static uint64_t img(uint64_t k) {
    return (k & 0x8000000000000000ull) ? ~k : (k | 0x8000000000000000ull);
  }
};

template <int DT, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_digit_hist(const typename Radix<DT>::K* __restrict__ keys, int64_t n, unsigned long long* __restrict__ hist) {
  using K = typename Radix<DT>::K;
  constexpr int KB = sizeof(K);
  __shared__ unsigned sh[KB * 256];
  for (int i = threadIdx.x; i < KB * 256; i += BLOCK) sh[i] = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  // Every warp runs the same trip count so the shuffles see all lanes.
  const int64_t stride = (int64_t)gridDim.x * BLOCK;
  const int64_t iters = (n + stride - 1) / stride;
  for (int64_t it = 0; it < iters; ++it) {
    const int64_t i = it * stride + (int64_t)blockIdx.x * BLOCK + threadIdx.x;
    const bool ok = i < n;
    const K img = ok ? Radix<DT>::img(keys[i]) : K(0);
    const unsigned okm = __ballot_sync(0xffffffffu, ok);
    if (!okm) continue;
#pragma unroll
    for (int p = 0; p < KB; ++p) {
      const unsigned d = (unsigned)(img >> (8 * p)) & 255u;
      const unsigned d0 = __shfl_sync(0xffffffffu, d, __ffs(okm) - 1);
      const bool same = __all_sync(0xffffffffu, !ok || d == d0);
      if (same) {
        if (lane == __ffs(okm) - 1) atomicAdd(sh + p * 256 + d0, (unsigned)__popc(okm));
      } else if (ok) {
        atomicAdd(sh + p * 256 + d, 1u);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < KB * 256; i += BLOCK)
    if (sh[i]) atomicAdd(hist + i, (unsigned long long)sh[i]);
}

template <int VB> struct ValT;
template <> struct ValT<0> { using T = char; };
template <> struct ValT<4> { using T = uint32_t; };
template <> struct ValT<8> { using T = uint64_t; };

struct PassArgs {
  unsigned* status;        // [ntiles][256]
  const int64_t* offsets;  // [256] exclusive digit starts for this pass
  unsigned* ticket;
  int* err;
  int64_t ntiles;
  int64_t wait_limit;
  int shift;
};

template <int DT, int VB, int BLOCK, int KPT>
__global__ void __launch_bounds__(BLOCK)
    k_onesweep(const typename Radix<DT>::K* __restrict__ kin, typename Radix<DT>::K* __restrict__ kout,
               const typename ValT<VB>::T* __restrict__ vin, typename ValT<VB>::T* __restrict__ vout, int64_t n,
               PassArgs A) {
  using K = typename Radix<DT>::K;
  using V = typename ValT<VB>::T;
  constexpr int WARPS = BLOCK / 32;
  constexpr int TILE = BLOCK * KPT;
  static_assert(BLOCK == 256, "one thread per digit");
  __shared__ unsigned s_whist[WARPS][256];
  __shared__ unsigned s_start[256];
  __shared__ long long s_gbase[256];
  __shared__ unsigned s_wsum[WARPS];
  __shared__ int s_timeout;
  __shared__ unsigned s_tile;
  extern __shared__ __align__(16) unsigned char s_dyn[];
  K* s_keys = reinterpret_cast<K*>(s_dyn);
  V* s_vals = reinterpret_cast<V*>(s_dyn + sizeof(K) * TILE);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(A.ticket, 1u);
    if ((int64_t)t == A.ntiles - 1) *A.ticket = 0u;
    s_tile = t;
    s_timeout = 0;
  }
  for (int i = lane; i < 256; i += 32) s_whist[warp][i] = 0u;
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t tbase = tile * (int64_t)TILE;
  const int cnt = (int)((n - tbase) < TILE ? (n - tbase) : TILE);
  const int wb = warp * 32 * KPT;  // warp's first slot in the tile

  // ---- load (warp-striped) and rank within the warp ------------------------
  K key[KPT];
  V val[KPT];
  unsigned short rk[KPT];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const int slot = wb + k * 32 + lane;
    const bool ok = slot < cnt;
    key[k] = ok ? kin[tbase + slot] : K(0);
    if (VB) val[k] = ok ? vin[tbase + slot] : V(0);
  }
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const int slot = wb + k * 32 + lane;
    const bool ok = slot < cnt;
    const unsigned d = (unsigned)(Radix<DT>::img(key[k]) >> A.shift) & 255u;
    unsigned m = __ballot_sync(0xffffffffu, ok);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const unsigned bb = __ballot_sync(0xffffffffu, (d >> b) & 1u);
      m &= ((d >> b) & 1u) ? bb : ~bb;
    }
    unsigned base = 0;
    const int leader = __ffs(m) - 1;
    if (ok && lane == leader) {
      base = s_whist[warp][d];
      s_whist[warp][d] = base + __popc(m);
    }
    base = __shfl_sync(0xffffffffu, base, leader < 0 ? lane : leader);
    rk[k] = (unsigned short)(base + __popc(m & lt));
    __syncwarp();
  }
  __syncthreads();
  // ---- per-digit totals, warp offsets and tile-local starts ----------------
  const unsigned d_me = threadIdx.x;  // this thread's digit
  unsigned tot = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    const unsigned c = s_whist[w][d_me];
    s_whist[w][d_me] = tot;
    tot += c;
  }
  {
    // exclusive scan of tot over the 256 digits
    unsigned inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) s_wsum[warp] = inc;
    __syncthreads();
    unsigned pre = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w)
      if (w < warp) pre += s_wsum[w];
    s_start[d_me] = pre + inc - tot;
  }
  // ---- per-digit decoupled look-back ---------------------------------------
  unsigned* st = A.status + tile * 256;
  long long excl = 0;
  if (tile == 0) {
    st_release_u32(st + d_me, SF_P | tot);
  } else {
    st_release_u32(st + d_me, SF_A | tot);
    int64_t pt = tile - 1;
    while (true) {
      unsigned s = 0;
      int64_t polls = 0;
      unsigned ns = 0;
      while (true) {
        s = ld_acquire_u32(A.status + pt * 256 + d_me);
        if (s & SF_MASK) break;
        if (++polls > A.wait_limit || *(volatile int*)&s_timeout) {
          s = SF_P;
          atomicExch(&s_timeout, 1);
          break;
        }
        if (polls > 4) {
          ns = ns ? (ns < 256 ? ns * 2 : 256) : 32;
          __nanosleep(ns);
        }
      }
      excl += (long long)(s & SV_MASK);
      if ((s & SF_MASK) == SF_P) break;
      --pt;
    }
    st_release_u32(st + d_me, SF_P | (unsigned)((excl + tot) & SV_MASK));
  }
  s_gbase[d_me] = (long long)A.offsets[d_me] + excl - (long long)s_start[d_me];
  __syncthreads();
  if (threadIdx.x == 0 && s_timeout) atomicOr(A.err, GBK_EBIT_TIMEOUT);
  // ---- reorder the tile by digit in shared memory --------------------------
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const int slot = wb + k * 32 + lane;
    if (slot < cnt) {
      const unsigned d = (unsigned)(Radix<DT>::img(key[k]) >> A.shift) & 255u;
      const unsigned r = s_start[d] + s_whist[warp][d] + rk[k];
      s_keys[r] = key[k];
      if (VB) s_vals[r] = val[k];
    }
  }
  __syncthreads();
  // ---- write runs of equal digits -------------------------------------------
  for (int i = threadIdx.x; i < cnt; i += BLOCK) {
    const K kk = s_keys[i];
    const unsigned d = (unsigned)(Radix<DT>::img(kk) >> A.shift) & 255u;
    const long long pos = s_gbase[d] + i;
    kout[pos] = kk;
    if (VB) vout[pos] = s_vals[i];
  }
}

// ---- host driver ------------------------------------------------------------
template <int DT, int VB>
int sort_impl(void* keys, void* vals, int64_t n, Workspace* w) {
  using K = typename Radix<DT>::K;
  using V = typename ValT<VB>::T;
  constexpr int KB = sizeof(K);
  constexpr int BLOCK = 256, KPT = 16, TILE = BLOCK * KPT;
  cudaStream_t s = w->stream;
  if (n <= 1) return GBK_OK;
  if (n >= (int64_t)SV_MASK) return GBK_ERR_INVALID_ARGUMENT;  // 30-bit status counts
  const int64_t ntiles = (n + TILE - 1) / TILE;
  // scratch: histogram | offsets | status | key temp | value temp
  const size_t hb = (size_t)KB * 256 * 8, ob = (size_t)KB * 256 * 8;
  const size_t sb = ((size_t)ntiles * 256 * 4 + 255) / 256 * 256;
  const size_t kb = ((size_t)n * sizeof(K) + 255) / 256 * 256;
  const size_t vb = VB ? ((size_t)n * VB + 255) / 256 * 256 : 0;
  int st = GBK_OK;
  char* scr = ws_scratch(w, hb + ob + sb + kb + vb, &st);
  if (!scr) return st;
  unsigned long long* d_hist = (unsigned long long*)scr;
  int64_t* d_off = (int64_t*)(scr + hb);
  unsigned* d_status = (unsigned*)(scr + hb + ob);
  K* ktmp = (K*)(scr + hb + ob + sb);
  V* vtmp = VB ? (V*)(scr + hb + ob + sb + kb) : nullptr;

  GBK_CUDA_TRY(cudaMemsetAsync(d_hist, 0, hb, s));
  {
    int64_t grid = (int64_t)sm_count() * 4;
    const int64_t need = (n + BLOCK * 4 - 1) / (BLOCK * 4);
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    k_digit_hist<DT, 512><<<(unsigned)grid, 512, 0, s>>>((const K*)keys, n, d_hist);
    note_launch();
    GBK_CUDA_TRY(cudaGetLastError());
  }
  std::vector<unsigned long long> h(KB * 256);
  GBK_CUDA_TRY(cudaMemcpyAsync(h.data(), d_hist, hb, cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<int64_t> offs(KB * 256);
  std::vector<int> passes;
  for (int p = 0; p < KB; ++p) {
    int64_t run = 0;
    bool constant = false;
    for (int d = 0; d < 256; ++d) {
      offs[p * 256 + d] = run;
      run += (int64_t)h[p * 256 + d];
      if ((int64_t)h[p * 256 + d] == n) constant = true;
    }
    if (run != n) return GBK_ERR_CUDA;  // histogram inconsistent
    if (!constant) passes.push_back(p);
  }
  if (passes.empty()) return GBK_OK;
  GBK_CUDA_TRY(cudaMemcpyAsync(d_off, offs.data(), ob, cudaMemcpyHostToDevice, s));
  // The host vector must outlive the copy.
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  const size_t dyn = (size_t)TILE * (sizeof(K) + (VB ? VB : 0));
  auto kfn = k_onesweep<DT, VB, BLOCK, KPT>;
  GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  K* kin = (K*)keys;
  K* kout = ktmp;
  V* vin = (V*)vals;
  V* vout = vtmp;
  for (size_t i = 0; i < passes.size(); ++i) {
    const int p = passes[i];
    GBK_CUDA_TRY(cudaMemsetAsync(d_status, 0, (size_t)ntiles * 256 * 4, s));
    PassArgs A;
    A.status = d_status;
    A.offsets = d_off + p * 256;
    A.ticket = w->counters + SLOT_SORT;
    A.err = w->err;
    A.ntiles = ntiles;
    A.wait_limit = wait_limit();
    A.shift = 8 * p;
    kfn<<<(unsigned)ntiles, BLOCK, dyn, s>>>(kin, kout, vin, vout, n, A);
    note_launch();
    GBK_CUDA_TRY(cudaGetLastError());
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != (K*)keys) {
    GBK_CUDA_TRY(cudaMemcpyAsync(keys, kin, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, s));
    if (VB) GBK_CUDA_TRY(cudaMemcpyAsync(vals, vin, (size_t)n * VB, cudaMemcpyDeviceToDevice, s));
  }
  return GBK_OK;
}

template <int DT>
int sort_vb(void* keys, void* vals, int vbytes, int64_t n, Workspace* w) {
  switch (vbytes) {
    case 0: return sort_impl<DT, 0>(keys, nullptr, n, w);
    case 4: return sort_impl<DT, 4>(keys, vals, n, w);
    case 8: return sort_impl<DT, 8>(keys, vals, n, w);
  }
  return GBK_ERR_UNSUPPORTED;
}

int sort_any(int kdt, void* keys, void* vals, int vbytes, int64_t n, Workspace* w) {
  switch (kdt) {
    case GBK_U32: return sort_vb<GBK_U32>(keys, vals, vbytes, n, w);
    case GBK_U64: return sort_vb<GBK_U64>(keys, vals, vbytes, n, w);
    case GBK_I32: return sort_vb<GBK_I32>(keys, vals, vbytes, n, w);
    case GBK_I64: return sort_vb<GBK_I64>(keys, vals, vbytes, n, w);
    case GBK_F32: return sort_vb<GBK_F32>(keys, vals, vbytes, n, w);
    case GBK_F64: return sort_vb<GBK_F64>(keys, vals, vbytes, n, w);
  }
  return GBK_ERR_UNSUPPORTED;
}

// ---- BinSort ------------------------------------------------------------------
// BinOp1D bin index (algorithms/src/sorting/Kokkos_BinOpsPublicAPI.hpp:56-59):
// (int)(mul * (double(key) - min)); computed with IEEE double arithmetic
// (__dmul_rn / __dsub_rn, no contraction) so it matches the host exactly.
template <class KT>
__global__ void k_bin_ids(const KT* __restrict__ keys, int64_t n, double kmin, double mul, int64_t nbins,
                          uint32_t* __restrict__ bins, uint32_t* __restrict__ iota, int* err) {
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double b = __dmul_rn(mul, __dsub_rn((double)keys[i], kmin));
    int64_t bi = (int64_t)(int)b;
    if (bi < 0 || bi >= nbins) {
      bad = true;
      bi = bi < 0 ? 0 : nbins - 1;
    }
    if (bins) bins[i] = (uint32_t)bi;
    if (iota) iota[i] = (uint32_t)i;
  }
  if (bad) atomicOr(err, GBK_EBIT_KEY_RANGE);
}

// starts[b] = first index of the sorted bin ids whose id is >= b (binary
// search), b in [0, nbins]; starts[nbins] = n.
__global__ void k_bin_starts(const uint32_t* __restrict__ sorted, int64_t n, int64_t nbins, int64_t* __restrict__ starts) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= nbins; b += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if ((int64_t)sorted[mid] < b) lo = mid + 1; else hi = mid;
    }
    starts[b] = lo;
  }
}

__global__ void k_bin_finish(const int64_t* __restrict__ starts, int64_t nbins, int32_t* __restrict__ counts,
                             int64_t* __restrict__ offsets) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += (int64_t)gridDim.x * blockDim.x) {
    counts[b] = (int32_t)(starts[b + 1] - starts[b]);
    offsets[b] = starts[b];
  }
}

__global__ void k_widen_perm(const uint32_t* __restrict__ p32, int64_t n, int64_t* __restrict__ perm) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    perm[i] = (int64_t)p32[i];
}

template <class T>
__global__ void k_permute(const T* __restrict__ src, const int64_t* __restrict__ perm, int64_t n, T* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}

unsigned grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_sort(gbk_dtype_t kdt, void* keys, int64_t n, gbk_stream_t stream) {
  if (n < 0 || (n > 1 && !keys)) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)keys % dtype_size(kdt)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return sort_any(kdt, keys, nullptr, 0, n, w);
}

int gbk_sort_by_key(gbk_dtype_t kdt, void* keys, int value_bytes, void* vals, int64_t n, gbk_stream_t stream) {
  if (value_bytes != 4 && value_bytes != 8) return GBK_ERR_UNSUPPORTED;
  if (n < 0 || (n > 1 && (!keys || !vals))) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)keys % dtype_size(kdt) || (uintptr_t)vals % value_bytes) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return sort_any(kdt, keys, vals, value_bytes, n, w);
}

int gbk_sort_u64(uint64_t* keys, int64_t n, gbk_stream_t stream) { return gbk_sort(GBK_U64, keys, n, stream); }

int gbk_sort_by_key_u64_i32(uint64_t* keys, int32_t* vals, int64_t n, gbk_stream_t stream) {
  return gbk_sort_by_key(GBK_U64, keys, 4, vals, n, stream);
}

int gbk_binsort_u64(const uint64_t* keys, int64_t n, int64_t nbins, double kmin, double mul, int sort_within_bins,
                    int32_t* bin_count, int64_t* bin_offsets, int64_t* perm, gbk_stream_t stream) {
  if (n < 0 || nbins <= 0 || nbins >= 0x7FFFFFFF || (n > 0 && (!keys || !perm)) || !bin_count || !bin_offsets)
    return GBK_ERR_INVALID_ARGUMENT;
  if (n >= (int64_t)0xFFFFFFFFu) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Workspace* w = ws_get(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  // stage: bin ids | iota | bin starts (nbins + 1) | key copy (within-bin sort)
  const size_t b4 = ((size_t)n * 4 + 255) / 256 * 256;
  const size_t sb = ((size_t)(nbins + 1) * 8 + 255) / 256 * 256;
  const size_t kb = sort_within_bins ? ((size_t)n * 8 + 255) / 256 * 256 : 0;
  char* d = ws_stage(w, 2 * b4 + sb + kb + 256, &st);
  if (!d) return st;
  uint32_t* ids = (uint32_t*)d;
  uint32_t* iota = (uint32_t*)(d + b4);
  int64_t* starts = (int64_t*)(d + 2 * b4);
  if (n > 0) {
    if (sort_within_bins) {
      // Bins are monotone in the key, so a stable sort by key orders by bin
      // and by key inside each bin.
      uint64_t* kc = (uint64_t*)(d + 2 * b4 + sb);
      GBK_CUDA_TRY(cudaMemcpyAsync(kc, keys, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
      k_bin_ids<uint64_t><<<grid_for(n, 256), 256, 0, s>>>(keys, n, kmin, mul, nbins, nullptr, iota, w->err);
      note_launch();
      st = sort_impl<GBK_U64, 4>(kc, iota, n, w);
      if (st) return st;
      // bin ids of the sorted keys
      k_bin_ids<uint64_t><<<grid_for(n, 256), 256, 0, s>>>(kc, n, kmin, mul, nbins, ids, nullptr, w->err);
      note_launch();
      GBK_CUDA_TRY(cudaGetLastError());
    } else {
      k_bin_ids<uint64_t><<<grid_for(n, 256), 256, 0, s>>>(keys, n, kmin, mul, nbins, ids, iota, w->err);
      note_launch();
      st = sort_impl<GBK_U32, 4>(ids, iota, n, w);
      if (st) return st;
    }
  }
  k_bin_starts<<<grid_for(nbins + 1, 256), 256, 0, s>>>(ids, n, nbins, starts);
  k_bin_finish<<<grid_for(nbins, 256), 256, 0, s>>>(starts, nbins, bin_count, bin_offsets);
  note_launch(2);
  if (n > 0) {
    k_widen_perm<<<grid_for(n, 256), 256, 0, s>>>(iota, n, perm);
    note_launch();
  }
  return cuda_status(cudaGetLastError());
}

int gbk_permute(int value_bytes, const void* src, const int64_t* perm, int64_t n, void* dst, gbk_stream_t stream) {
  if (n < 0 || (n > 0 && (!src || !perm || !dst)) || src == dst) return GBK_ERR_INVALID_ARGUMENT;
  if (n == 0) return GBK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  switch (value_bytes) {
    case 1: k_permute<uint8_t><<<grid_for(n, 256), 256, 0, s>>>((const uint8_t*)src, perm, n, (uint8_t*)dst); break;
    case 2: k_permute<uint16_t><<<grid_for(n, 256), 256, 0, s>>>((const uint16_t*)src, perm, n, (uint16_t*)dst); break;
    case 4: k_permute<uint32_t><<<grid_for(n, 256), 256, 0, s>>>((const uint32_t*)src, perm, n, (uint32_t*)dst); break;
    case 8: k_permute<uint64_t><<<grid_for(n, 256), 256, 0, s>>>((const uint64_t*)src, perm, n, (uint64_t*)dst); break;
    default: return GBK_ERR_UNSUPPORTED;
  }
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
