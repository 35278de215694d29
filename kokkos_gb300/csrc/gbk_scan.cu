// Single-pass prefix scan with decoupled look-back (Merrill & Garland,
// "Single-pass Parallel Prefix Scan with Decoupled Look-back", NVIDIA
// NVR-2016-002).  Replaces the two-launch, two-read CUDA ParallelScan of
// core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:390-700 (and the
// ParallelScanWithTotal variant :704-1053): one read of x, one write of y.
//
// Tiles of BLOCK * IPT 16-byte input vectors.  A CTA takes its tile index
// from an atomic ticket, so every tile it waits on belongs to a CTA that is
// already running: the look-back cannot deadlock whatever the occupancy.
// Each warp owns a contiguous slice of the tile in warp-striped order
// (vector k of lane l at slice + (32k + l) * VEC), so loads and stores are
// coalesced without a shared-memory transpose; the scan inside the warp is a
// shuffle scan per row k with a running carry.  Tile status words carry the
// launch epoch in their upper 30 bits, so stale words from earlier launches
// read as "not ready" and no memset is needed per launch.  Every wait polls
// with a back-off and gives up after the library's wait limit, setting the
// timeout bit of the stream's error word instead of hanging.
#include <type_traits>

#include "gbk_internal.cuh"

namespace gbk {
namespace {

constexpr unsigned FLAG_A = 1;  // tile aggregate available
constexpr unsigned FLAG_P = 2;  // inclusive prefix available

template <class TO>
struct ScanState {
  unsigned* flags;
  TO* agg;
  TO* incl;
  unsigned* ticket;
  int* err;
  unsigned epoch;  // 30 bits
  int64_t ntiles;
  int64_t wait_limit;
};

template <class T> __device__ __forceinline__ T shup(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
template <class T> __device__ __forceinline__ T shidx(T v, int l) { return __shfl_sync(0xffffffffu, v, l); }

// Inclusive warp scan (Kogge-Stone).
template <class T>
__device__ __forceinline__ T warp_iscan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = shup(v, d);
    if (lane >= d) v = o + v;
  }
  return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  return v;
}

template <class TO>
__device__ __forceinline__ TO ld_relaxed_val(const TO* p) {
  if constexpr (sizeof(TO) == 8) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    TO r;
    memcpy(&r, &v, 8);
    return r;
  } else {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    TO r;
    memcpy(&r, &v, 4);
    return r;
  }
}

template <class TI, class TO, bool INCL, bool ALIGNED, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK)
    k_scan(const TI* __restrict__ x, TO* __restrict__ y, int64_t n, TO init, ScanState<TO> S, TO* total) {
  constexpr int VEC = 16 / sizeof(TI);
  constexpr int WARPS = BLOCK / 32;
  constexpr int64_t TILE = (int64_t)BLOCK * IPT * VEC;
  constexpr int64_t WSLICE = 32LL * IPT * VEC;
  __shared__ int64_t s_tile;
  __shared__ TO s_warp[WARPS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(S.ticket, 1u);
    if ((int64_t)t == S.ntiles - 1) *S.ticket = 0u;  // every tile has been claimed
    s_tile = (int64_t)t;
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t tbase = tile * TILE;
  const int64_t wbase = tbase + warp * WSLICE;
  const bool full = tbase + TILE <= n;

  // ---- load (warp-striped) and thread-local inclusive scans --------------
  // Inputs stay in the input type (fewer registers for widening scans); the
  // in-chunk prefix is recomputed when the outputs are formed.
  TI v[IPT][VEC];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int64_t e0 = wbase + ((int64_t)k * 32 + lane) * VEC;
    if (ALIGNED && full) {
      Vec16<TI> u;
      u.u = ld_stream16(x + e0);
#pragma unroll
      for (int j = 0; j < VEC; ++j) v[k][j] = u.v[j];
    } else {
#pragma unroll
      for (int j = 0; j < VEC; ++j) v[k][j] = (e0 + j < n) ? x[e0 + j] : TI(0);
    }
  }
  // ---- warp scan over chunks in (k, lane) order ---------------------------
  TO chunk_ex[IPT];
  TO carry = TO(0);
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    TO c = (TO)v[k][0];
#pragma unroll
    for (int j = 1; j < VEC; ++j) c = c + (TO)v[k][j];
    const TO inc = warp_iscan(c);
    TO ex = shup(inc, 1);
    if (lane == 0) ex = TO(0);
    chunk_ex[k] = carry + ex;
    carry = carry + shidx(inc, 31);
  }
  if (lane == 0) s_warp[warp] = carry;
  __syncthreads();
  TO warp_pre = TO(0), tile_agg = TO(0);
  {
    // Every thread walks the (few) warp totals: deterministic, no extra sync.
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      if (w == warp) warp_pre = tile_agg;
      tile_agg = tile_agg + s_warp[w];
    }
  }
  // ---- decoupled look-back, the whole CTA as one BLOCK-tile window ----------
  // Thread i examines predecessor tile (window start - i).  The window sums
  // aggregates back to the nearest tile with an inclusive prefix; windows
  // step back by BLOCK tiles until one holds such a tile.  A whole-CTA
  // window keeps the walk short when hundreds of tiles are in flight.
  const unsigned ep = S.epoch << 2;
  __shared__ int s_near;
  __shared__ int s_timeout;
  __shared__ TO s_wsum[WARPS];
  TO excl = TO(0);
  if (tile == 0) {
    if (threadIdx.x == 0) {
      S.incl[0] = tile_agg;
      st_release_u32(S.flags, ep | FLAG_P);
    }
  } else {
    if (threadIdx.x == 0) {
      S.agg[tile] = tile_agg;
      st_release_u32(S.flags + tile, ep | FLAG_A);
      s_timeout = 0;
    }
    int64_t pt0 = tile - 1;
    while (true) {
      const int64_t pt = pt0 - threadIdx.x;
      unsigned f = ep | FLAG_P;
      TO val = TO(0);
      if (threadIdx.x == 0) s_near = BLOCK;
      __syncthreads();
      if (pt >= 0) {
        int64_t polls = 0;
        unsigned ns = 0;
        while (true) {
          f = ld_relaxed_u32(S.flags + pt);
          if ((f & ~3u) == ep && (f & 3u)) break;
          if (++polls > S.wait_limit || *(volatile int*)&s_timeout) {
            f = ep | FLAG_P;  // give up: treat as a zero prefix
            atomicExch(&s_timeout, 1);
            break;
          }
          if (polls > 8) {
            ns = ns ? (ns < 256 ? ns * 2 : 256) : 32;
            __nanosleep(ns);
          }
        }
        __threadfence();  // acquire: the value below is at least as new as the flag
        if (!*(volatile int*)&s_timeout) val = ((f & 3u) == FLAG_P) ? ld_relaxed_val(S.incl + pt) : ld_relaxed_val(S.agg + pt);
      }
      if ((f & 3u) == FLAG_P) atomicMin(&s_near, (int)threadIdx.x);
      __syncthreads();
      const int near = s_near;
      // Fixed-order sum of the window entries up to the nearest prefix.
      TO c = ((int)threadIdx.x <= near) ? val : TO(0);
      c = warp_sum(c);
      if (lane == 0) s_wsum[warp] = c;
      __syncthreads();
#pragma unroll
      for (int w = 0; w < WARPS; ++w) excl = excl + s_wsum[w];
      if (near < BLOCK) break;
      pt0 -= BLOCK;
      __syncthreads();  // s_wsum / s_near are rewritten by the next window
    }
    if (threadIdx.x == 0) {
      if (s_timeout) atomicOr(S.err, GBK_EBIT_TIMEOUT);
      S.incl[tile] = excl + tile_agg;
      st_release_u32(S.flags + tile, ep | FLAG_P);
    }
  }
  const TO tile_pre = excl;
  if (total && tile == S.ntiles - 1 && threadIdx.x == 0) *total = INCL ? tile_pre + tile_agg : init + (tile_pre + tile_agg);

  // ---- write ---------------------------------------------------------------
  const TO base = INCL ? tile_pre + warp_pre : init + (tile_pre + warp_pre);
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int64_t e0 = wbase + ((int64_t)k * 32 + lane) * VEC;
    TO run = base + chunk_ex[k];
    TO o[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      if (INCL) {
        run = run + (TO)v[k][j];
        o[j] = run;
      } else {
        o[j] = run;
        run = run + (TO)v[k][j];
      }
    }
    if (ALIGNED && full) {
      constexpr int OV = 16 / sizeof(TO);
#pragma unroll
      for (int j = 0; j < VEC; j += OV) {
        Vec16<TO> u;
#pragma unroll
        for (int q = 0; q < OV; ++q) u.v[q] = o[j + q];
        __stcs(reinterpret_cast<uint4*>(y + e0 + j), u.u);
      }
    } else {
#pragma unroll
      for (int j = 0; j < VEC; ++j)
        if (e0 + j < n) y[e0 + j] = o[j];
    }
  }
}

template <class TI, class TO, bool INCL>
int launch_scan_t(const TI* x, TO* y, int64_t n, TO init, TO* total, Workspace* w, const gbk_tuning_t* t) {
  cudaStream_t s = w->stream;
  if (n <= 0) {
    if (total) {
      GBK_CUDA_TRY(cudaMemcpyAsync(total, &init, sizeof(TO), cudaMemcpyHostToDevice, s));
      // init lives on this call's stack: make the copy finish before return.
      GBK_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return GBK_OK;
  }
  constexpr int VEC = 16 / sizeof(TI);
  const int ipt = t && t->items_per_thread ? t->items_per_thread : 4;
  const int64_t tile = (int64_t)256 * ipt * VEC;
  const int64_t ntiles = (n + tile - 1) / tile;
  if (ntiles >= (int64_t)0xFFFFFFFFu) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  const size_t vbytes = ((size_t)ntiles * sizeof(TO) + 255) / 256 * 256;
  char* scr = ws_scratch(w, 2 * vbytes, &st);
  if (!scr) return st;
  ScanState<TO> S;
  S.flags = ws_flags(w, (size_t)ntiles, &S.epoch, &st);
  if (!S.flags) return st;
  S.agg = (TO*)scr;
  S.incl = (TO*)(scr + vbytes);
  S.ticket = w->counters + SLOT_SCAN_TILE;
  S.err = w->err;
  S.ntiles = ntiles;
  S.wait_limit = wait_limit();
  const bool aligned = ((uintptr_t)x % 16 == 0) && ((uintptr_t)y % 16 == 0);
  const unsigned grid = (unsigned)ntiles;
#define GBK_SCAN_LAUNCH(AL, IPT) k_scan<TI, TO, INCL, AL, 256, IPT><<<grid, 256, 0, s>>>(x, y, n, init, S, total)
  if (ipt == 2) {
    if (aligned) GBK_SCAN_LAUNCH(true, 2); else GBK_SCAN_LAUNCH(false, 2);
  } else if (ipt == 8) {
    if (aligned) GBK_SCAN_LAUNCH(true, 8); else GBK_SCAN_LAUNCH(false, 8);
  } else {
    if (aligned) GBK_SCAN_LAUNCH(true, 4); else GBK_SCAN_LAUNCH(false, 4);
  }
#undef GBK_SCAN_LAUNCH
  note_launch();
  return cuda_status(cudaGetLastError());
}

template <class TI, class TO>
int launch_scan(int incl, const void* x, void* y, int64_t n, const void* init, void* total, Workspace* w,
                const gbk_tuning_t* t) {
  TO iv = TO(0);
  if (init && !incl) memcpy(&iv, init, sizeof(TO));
  if (incl) return launch_scan_t<TI, TO, true>((const TI*)x, (TO*)y, n, TO(0), (TO*)total, w, t);
  return launch_scan_t<TI, TO, false>((const TI*)x, (TO*)y, n, iv, (TO*)total, w, t);
}

int scan_any(int incl, int din, int dout, const void* x, int64_t n, const void* init, void* y, void* total,
             Workspace* w, const gbk_tuning_t* t) {
#define GBK_SCAN_CASE(A, TA, B, TB) \
  if (din == A && dout == B) return launch_scan<TA, TB>(incl, x, y, n, init, total, w, t);
  GBK_SCAN_CASE(GBK_I32, int32_t, GBK_I32, int32_t)
  GBK_SCAN_CASE(GBK_I32, int32_t, GBK_I64, int64_t)
  GBK_SCAN_CASE(GBK_I64, int64_t, GBK_I64, int64_t)
  GBK_SCAN_CASE(GBK_U32, uint32_t, GBK_U32, uint32_t)
  GBK_SCAN_CASE(GBK_U32, uint32_t, GBK_U64, uint64_t)
  GBK_SCAN_CASE(GBK_U64, uint64_t, GBK_U64, uint64_t)
  GBK_SCAN_CASE(GBK_F32, float, GBK_F32, float)
  GBK_SCAN_CASE(GBK_F32, float, GBK_F64, double)
  GBK_SCAN_CASE(GBK_F64, double, GBK_F64, double)
#undef GBK_SCAN_CASE
  return GBK_ERR_UNSUPPORTED;
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_scan(int inclusive, gbk_dtype_t din, gbk_dtype_t dout, const void* x, int64_t n, const void* init, void* y,
             void* total, gbk_stream_t stream, const gbk_tuning_t* tune) {
  const bool pair_ok = (din == dout && din >= GBK_I32 && din <= GBK_F64) || (din == GBK_I32 && dout == GBK_I64) ||
                       (din == GBK_U32 && dout == GBK_U64) || (din == GBK_F32 && dout == GBK_F64);
  if (!pair_ok) return GBK_ERR_UNSUPPORTED;
  if (n < 0 || (n > 0 && (!x || !y))) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)x % dtype_size(din) || (uintptr_t)y % dtype_size(dout)) return GBK_ERR_INVALID_ARGUMENT;
  if (n > 0 && x == y && din != dout) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  gbk_tuning_t tt;
  if (!tune) tune = tuned_config(TUNE_SCAN, inclusive ? 1 : 0, din * 8 + dout, n, 0, &tt);
  std::lock_guard<std::mutex> lk(w->mu);
  return scan_any(inclusive ? 1 : 0, din, dout, x, n, init, y, total, w, tune);
}

int gbk_exclusive_scan_i32_i64(const int32_t* x, int64_t n, int64_t init, int64_t* y, gbk_stream_t stream) {
  return gbk_scan(0, GBK_I32, GBK_I64, x, n, &init, y, nullptr, stream, nullptr);
}

int gbk_inclusive_scan_i32(const int32_t* x, int64_t n, int32_t* y, gbk_stream_t stream) {
  return gbk_scan(1, GBK_I32, GBK_I32, x, n, nullptr, y, nullptr, stream, nullptr);
}

int gbk_inclusive_scan_f64(const double* x, int64_t n, double* y, gbk_stream_t stream) {
  return gbk_scan(1, GBK_F64, GBK_F64, x, n, nullptr, y, nullptr, stream, nullptr);
}

int gbk_exclusive_scan_i32_i64_host(const int32_t* hx, int64_t n, int64_t init, int64_t* hy, gbk_stream_t stream) {
  if (n < 0 || (n > 0 && (!hx || !hy))) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Workspace* w = ws_get(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  const size_t ib = (size_t)n * 4, ipad = (ib + 255) / 256 * 256;
  char* d = ws_stage(w, ipad + (size_t)n * 8 + 256, &st);
  if (!d) return st;
  if (n == 0) return GBK_OK;
  GBK_CUDA_TRY(cudaMemcpyAsync(d, hx, ib, cudaMemcpyHostToDevice, s));
  st = scan_any(0, GBK_I32, GBK_I64, d, n, &init, d + ipad, nullptr, w, nullptr);
  if (st) return st;
  GBK_CUDA_TRY(cudaMemcpyAsync(hy, d + ipad, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  return GBK_OK;
}

}  // extern "C"
