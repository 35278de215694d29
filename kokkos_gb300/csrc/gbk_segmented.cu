// Batched segmented reduce and scan: thousands of uneven segments in one
// launch.  Replaces the TeamPolicy league pattern "one team per segment,
// TeamThreadRange reduce / scan inside" (core/src/OpenMP/Kokkos_OpenMP_Parallel_Reduce.hpp:332-530,
// core/src/Cuda/Kokkos_Cuda_Parallel_Team.hpp:589-980) and the loop of one
// parallel_reduce / inclusive_scan launch per segment.
//
// Segments are given by offsets[0..nseg] (segment s = [offsets[s],
// offsets[s+1]), non-decreasing, offsets[nseg] = n).  The concatenated array
// is cut into fixed tiles of BLOCK*IPT*VEC elements, independent of the
// segment lengths, so the work is balanced whatever the length
// distribution.  Per tile:
//   * warp 0 finds the segment starts that fall in the tile with a 32-ary
//     search of offsets and the CTA marks them in a shared-memory bitmap;
//   * a segmented scan (pairs (head-seen, value), operator
//     (h1,v1).(h2,v2) = (h1|h2, h2 ? v2 : v1 op v2)) runs in registers, then
//     across warps;
//   * the carry into the tile comes from a decoupled look-back over the
//     predecessor tiles that stops at the first tile holding a segment head
//     (normally the previous tile), so long segments chain and short ones
//     never wait long;
//   * REDUCE mode writes each segment's total at its last element; scan
//     modes write every element.
// Tile status words are epoch-tagged (no memset per launch) and every wait is
// bounded.
#include <type_traits>

#include "gbk_internal.cuh"

namespace gbk {
namespace {

enum { M_INCL = 0, M_EXCL = 1, M_REDUCE = 2 };

template <class T, int OP> struct SOp;
template <class T> struct SOp<T, GBK_SUM> {
  __device__ static T id() { return T(0); }
  __device__ static T f(T a, T b) { return a + b; }
};
template <class T> struct SOp<T, GBK_MIN> {
  __device__ static T id() { return lim<T>::hi(); }
  __device__ static T f(T a, T b) { return b < a ? b : a; }
};
template <class T> struct SOp<T, GBK_MAX> {
  __device__ static T id() { return lim<T>::lo(); }
  __device__ static T f(T a, T b) { return b > a ? b : a; }
};

template <class TO>
struct SegState {
  unsigned* flags;  // epoch << 2 | status: 1 = aggregate, 3 = aggregate of a tile holding a head, 2 = prefix
  TO* agg;
  TO* incl;
  unsigned* ticket;
  int* err;
  unsigned epoch;  // 30 bits, shared with the plain scan's status words
  int64_t ntiles;
  int64_t wait_limit;
};

template <class T> __device__ __forceinline__ T sh_up(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }

template <class TO>
__device__ __forceinline__ TO ld_relaxed_any(const TO* p) {
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

// First index s in [lo, hi) with offsets[s] >= key (hi if none), by one
// warp: each round 32 lanes probe evenly spaced indices.
__device__ int64_t warp_lower_bound(const int64_t* __restrict__ offsets, int64_t lo, int64_t hi, int64_t key) {
  const int lane = threadIdx.x & 31;
  while (hi - lo > 32) {
    const int64_t step = (hi - lo + 31) / 32;
    const int64_t idx = lo + lane * step;
    const bool ge = idx < hi ? (__ldg(offsets + idx) >= key) : true;
    const unsigned m = __ballot_sync(0xffffffffu, ge);
    const int first = m ? __ffs(m) - 1 : 32;  // first probe with offsets >= key
    const int64_t nlo = first == 0 ? lo : lo + (int64_t)(first - 1) * step;
    const int64_t nhi = first == 32 ? hi : (lo + (int64_t)first * step < hi ? lo + (int64_t)first * step : hi);
    lo = nlo;
    hi = (nhi > lo) ? nhi : lo;
    if (first == 0) { hi = lo; break; }
  }
  const int64_t idx = lo + lane;
  const bool ge = idx < hi ? (__ldg(offsets + idx) >= key) : true;
  const unsigned m = __ballot_sync(0xffffffffu, ge);
  const int first = m ? __ffs(m) - 1 : 32;
  const int64_t r = lo + first;
  return r < hi ? r : hi;
}

template <class TI, class TO, int OP, int MODE, bool ALIGNED, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK)
    k_segmented(const TI* __restrict__ x, TO* __restrict__ y, int64_t n, const int64_t* __restrict__ offsets,
                int64_t nseg, SegState<TO> S) {
  using O = SOp<TO, OP>;
  constexpr int VEC = 16 / sizeof(TI);
  constexpr int WARPS = BLOCK / 32;
  constexpr int TILE = BLOCK * IPT * VEC;
  constexpr int WSLICE = 32 * IPT * VEC;
  constexpr int BMW = TILE / 32 + 2;  // bitmap words covering [tbase, tbase + TILE]
  __shared__ unsigned s_bm[BMW];
  __shared__ int64_t s_tile, s_lo, s_hi;
  __shared__ TO s_wv[WARPS];
  __shared__ unsigned s_wh[WARPS];
  __shared__ int s_near, s_timeout;
  __shared__ TO s_wsum[WARPS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(S.ticket, 1u);
    if ((int64_t)t == S.ntiles - 1) *S.ticket = 0u;
    s_tile = (int64_t)t;
    s_timeout = 0;
  }
  for (int i = threadIdx.x; i < BMW; i += BLOCK) s_bm[i] = 0u;
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t tbase = tile * (int64_t)TILE;
  if (MODE == M_REDUCE) {
    // Empty segments get the identity (their start is shared with the next).
    for (int64_t s = tile * BLOCK + threadIdx.x; s < nseg; s += S.ntiles * BLOCK)
      if (offsets[s + 1] == offsets[s]) y[s] = O::id();
  }
  if (warp == 0) {
    const int64_t lo = warp_lower_bound(offsets, 0, nseg + 1, tbase);
    const int64_t hi = warp_lower_bound(offsets, lo, nseg + 1, tbase + TILE + 1);
    if (lane == 0) { s_lo = lo; s_hi = hi; }
  }
  __syncthreads();
  for (int64_t s = s_lo + threadIdx.x; s < s_hi; s += BLOCK) {
    const int64_t p = offsets[s] - tbase;  // in [0, TILE]
    atomicOr(&s_bm[p >> 5], 1u << (p & 31));
  }
  __syncthreads();
  auto head = [&](int64_t e) -> unsigned {  // e relative to tbase, 0..TILE
    return (s_bm[e >> 5] >> (e & 31)) & 1u;
  };

  const int wb = warp * WSLICE;
  const bool full = tbase + TILE <= n;
  TI v[IPT][VEC];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int64_t e0 = tbase + wb + (k * 32 + lane) * VEC;
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
  // chunk aggregates (head seen, value after the last head)
  TO cv[IPT];
  unsigned ch[IPT];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int r0 = wb + (k * 32 + lane) * VEC;
    TO a = O::id();
    unsigned h = 0;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      const bool valid = tbase + r0 + j < n;
      const unsigned hj = head(r0 + j);
      if (hj) { a = O::id(); h = 1; }
      if (valid) a = O::f(a, (TO)v[k][j]);
    }
    cv[k] = a;
    ch[k] = h;
  }
  // warp segmented scan over chunks in (k, lane) order: exclusive carry per chunk
  TO cin[IPT];
  unsigned cinh[IPT];  // a head occurs in this warp before the chunk
  TO carry = O::id();
  unsigned carry_h = 0;
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    TO iv = cv[k];
    unsigned ih = ch[k];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const TO ov = sh_up(iv, d);
      const unsigned oh = sh_up(ih, d);
      if (lane >= d) {
        if (!ih) iv = O::f(ov, iv);
        ih |= oh;
      }
    }
    // exclusive within the row, then apply the row carry
    TO ev = sh_up(iv, 1);
    unsigned eh = sh_up(ih, 1);
    if (lane == 0) { ev = O::id(); eh = 0; }
    cin[k] = eh ? ev : O::f(carry, ev);
    cinh[k] = eh | carry_h;
    const TO rv = __shfl_sync(0xffffffffu, iv, 31);
    const unsigned rh = __shfl_sync(0xffffffffu, ih, 31);
    carry = rh ? rv : O::f(carry, rv);
    carry_h |= rh;
  }
  if (lane == 0) { s_wv[warp] = carry; s_wh[warp] = carry_h; }
  __syncthreads();
  // carry into this warp from earlier warps of the tile, and the tile aggregate
  TO wpre = O::id(), tagg = O::id();
  unsigned wpre_h = 0, tagg_h = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    if (w == warp) { wpre = tagg; wpre_h = tagg_h; }
    tagg = s_wh[w] ? s_wv[w] : O::f(tagg, s_wv[w]);
    tagg_h |= s_wh[w];
  }
  // ---- look-back: carry from predecessor tiles ------------------------------
  const unsigned ep = S.epoch << 2;
  TO excl = O::id();
  if (tile == 0) {
    if (threadIdx.x == 0) {
      S.incl[0] = tagg;
      st_release_u32(S.flags, ep | 2u);
    }
  } else {
    if (threadIdx.x == 0) {
      S.agg[tile] = tagg;
      st_release_u32(S.flags + tile, ep | (tagg_h ? 3u : 1u));
    }
    int64_t pt0 = tile - 1;
    while (true) {
      const int64_t pt = pt0 - threadIdx.x;
      unsigned f = ep | 2u;
      TO val = O::id();
      if (threadIdx.x == 0) s_near = BLOCK;
      __syncthreads();
      if (pt >= 0) {
        int64_t polls = 0;
        unsigned ns = 0;
        while (true) {
          f = ld_relaxed_u32(S.flags + pt);
          if ((f & ~3u) == ep && (f & 3u)) break;
          if (++polls > S.wait_limit || *(volatile int*)&s_timeout) {
            f = ep | 2u;
            atomicExch(&s_timeout, 1);
            break;
          }
          if (polls > 8) {
            ns = ns ? (ns < 256 ? ns * 2 : 256) : 32;
            __nanosleep(ns);
          }
        }
        __threadfence();
        if (!*(volatile int*)&s_timeout) val = ((f & 3u) == 2u) ? ld_relaxed_any(S.incl + pt) : ld_relaxed_any(S.agg + pt);
      }
      // stop at the nearest tile that is complete (P) or holds a segment head
      if (f & 2u) atomicMin(&s_near, (int)threadIdx.x);  // prefix, or a tile holding a head
      __syncthreads();
      const int near = s_near;
      TO c = ((int)threadIdx.x <= near) ? val : O::id();
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) c = O::f(c, __shfl_xor_sync(0xffffffffu, c, m));
      if (lane == 0) s_wsum[warp] = c;
      __syncthreads();
#pragma unroll
      for (int w = 0; w < WARPS; ++w) excl = O::f(excl, s_wsum[w]);
      if (near < BLOCK) break;
      pt0 -= BLOCK;
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      if (s_timeout) atomicOr(S.err, GBK_EBIT_TIMEOUT);
      // inclusive prefix value at the end of this tile
      S.incl[tile] = tagg_h ? tagg : O::f(excl, tagg);
      st_release_u32(S.flags + tile, ep | 2u);
    }
  }
  // ---- outputs ---------------------------------------------------------------
  const TO wbase_v = wpre_h ? wpre : O::f(excl, wpre);
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int r0 = wb + (k * 32 + lane) * VEC;
    const int64_t e0 = tbase + r0;
    // Carry into the chunk: cin[k] covers the warp's earlier chunks; the
    // carry from earlier warps and tiles applies unless a head came first.
    TO run = cin[k];
    if (!cinh[k]) run = O::f(wbase_v, run);
    TO o[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      const bool valid = e0 + j < n;
      if (head(r0 + j)) run = O::id();
      if (MODE == M_EXCL) o[j] = run;
      if (valid) run = O::f(run, (TO)v[k][j]);
      if (MODE == M_INCL) o[j] = run;
      if (MODE == M_REDUCE && valid && head(r0 + j + 1)) {
        // last element of its segment: find the (non-empty) segment s with
        // offsets[s] <= e < offsets[s+1]
        const int64_t e = e0 + j;
        int64_t lo = s_lo > 0 ? s_lo - 1 : 0, hi = s_hi;  // s in [lo, hi)
        while (hi - lo > 1) {
          const int64_t mid = lo + (hi - lo) / 2;
          if (offsets[mid] <= e) lo = mid; else hi = mid;
        }
        y[lo] = run;
      }
    }
    if (MODE != M_REDUCE) {
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
}

template <class TI, class TO, int OP, int MODE, int IPT>
int launch_seg_ipt(const TI* x, TO* y, int64_t n, const int64_t* offsets, int64_t nseg, Workspace* w) {
  constexpr int BLOCK = 256, VEC = 16 / sizeof(TI);
  constexpr int64_t TILE = (int64_t)BLOCK * IPT * VEC;
  cudaStream_t s = w->stream;
  const int64_t nt = (n + TILE - 1) / TILE;
  const int64_t ntiles = nt > 0 ? nt : 1;  // one tile still writes empty-segment identities
  if (ntiles >= (int64_t)0x7FFFFFFF) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  const size_t vb = ((size_t)ntiles * sizeof(TO) + 255) / 256 * 256;
  char* scr = ws_scratch(w, 2 * vb, &st);
  if (!scr) return st;
  SegState<TO> S;
  unsigned ep = 0;
  S.flags = ws_flags(w, (size_t)ntiles, &ep, &st);
  if (!S.flags) return st;
  S.epoch = ep;
  S.agg = (TO*)scr;
  S.incl = (TO*)(scr + vb);
  S.ticket = w->counters + SLOT_SEG;
  S.err = w->err;
  S.ntiles = ntiles;
  S.wait_limit = wait_limit();
  const bool aligned = ((uintptr_t)x % 16 == 0) && (MODE == M_REDUCE || (uintptr_t)y % 16 == 0);
  if (aligned)
    k_segmented<TI, TO, OP, MODE, true, BLOCK, IPT><<<(unsigned)ntiles, BLOCK, 0, s>>>(x, y, n, offsets, nseg, S);
  else
    k_segmented<TI, TO, OP, MODE, false, BLOCK, IPT><<<(unsigned)ntiles, BLOCK, 0, s>>>(x, y, n, offsets, nseg, S);
  note_launch();
  return cuda_status(cudaGetLastError());
}

// items_per_thread (16-byte vectors per thread per tile): 2, 4 (default), 8.
template <class TI, class TO, int OP, int MODE>
int launch_seg(const TI* x, TO* y, int64_t n, const int64_t* offsets, int64_t nseg, Workspace* w,
               const gbk_tuning_t* t) {
  const int ipt = t && t->items_per_thread ? t->items_per_thread : 4;
  if (ipt == 2) return launch_seg_ipt<TI, TO, OP, MODE, 2>(x, y, n, offsets, nseg, w);
  if (ipt == 8) return launch_seg_ipt<TI, TO, OP, MODE, 8>(x, y, n, offsets, nseg, w);
  return launch_seg_ipt<TI, TO, OP, MODE, 4>(x, y, n, offsets, nseg, w);
}

template <class T>
int seg_reduce_t(int op, const void* x, const int64_t* offs, int64_t nseg, int64_t n, void* out, Workspace* w,
                 const gbk_tuning_t* t) {
  switch (op) {
    case GBK_SUM: return launch_seg<T, T, GBK_SUM, M_REDUCE>((const T*)x, (T*)out, n, offs, nseg, w, t);
    case GBK_MIN: return launch_seg<T, T, GBK_MIN, M_REDUCE>((const T*)x, (T*)out, n, offs, nseg, w, t);
    case GBK_MAX: return launch_seg<T, T, GBK_MAX, M_REDUCE>((const T*)x, (T*)out, n, offs, nseg, w, t);
  }
  return GBK_ERR_UNSUPPORTED;
}

// Tuning-table extra for segmented calls: log2 of the mean segment length.
int seg_extra(int64_t n, int64_t nseg) {
  int64_t mean = nseg > 0 ? n / nseg : n;
  int l = 0;
  while (((int64_t)1 << l) < mean && l < 62) ++l;
  return l;
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_segmented_reduce(gbk_reducer_t op, gbk_dtype_t dt, const void* x, const int64_t* offsets, int64_t nseg,
                         int64_t n, void* out, gbk_stream_t stream, const gbk_tuning_t* tune) {
  if (op != GBK_SUM && op != GBK_MIN && op != GBK_MAX) return GBK_ERR_UNSUPPORTED;
  if (nseg < 0 || n < 0 || (nseg > 0 && (!offsets || !out)) || (n > 0 && !x)) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)x % dtype_size(dt) || (uintptr_t)out % dtype_size(dt)) return GBK_ERR_INVALID_ARGUMENT;
  if (nseg == 0) return GBK_OK;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  gbk_tuning_t tt;
  if (!tune) tune = tuned_config(TUNE_SEG, op, dt, n, seg_extra(n, nseg), &tt);
  std::lock_guard<std::mutex> lk(w->mu);
  switch (dt) {
    case GBK_I32: return seg_reduce_t<int32_t>(op, x, offsets, nseg, n, out, w, tune);
    case GBK_I64: return seg_reduce_t<int64_t>(op, x, offsets, nseg, n, out, w, tune);
    case GBK_U32: return seg_reduce_t<uint32_t>(op, x, offsets, nseg, n, out, w, tune);
    case GBK_U64: return seg_reduce_t<uint64_t>(op, x, offsets, nseg, n, out, w, tune);
    case GBK_F32: return seg_reduce_t<float>(op, x, offsets, nseg, n, out, w, tune);
    case GBK_F64: return seg_reduce_t<double>(op, x, offsets, nseg, n, out, w, tune);
  }
  return GBK_ERR_UNSUPPORTED;
}

int gbk_segmented_scan(int inclusive, gbk_dtype_t din, gbk_dtype_t dout, const void* x, const int64_t* offsets,
                       int64_t nseg, int64_t n, void* y, gbk_stream_t stream, const gbk_tuning_t* tune) {
  if (nseg < 0 || n < 0 || (n > 0 && (!x || !y || !offsets))) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)x % dtype_size(din) || (uintptr_t)y % dtype_size(dout)) return GBK_ERR_INVALID_ARGUMENT;
  if (n == 0) return GBK_OK;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  gbk_tuning_t tt;
  if (!tune) tune = tuned_config(TUNE_SEG, 16 + (inclusive ? 1 : 0), din * 8 + dout, n, seg_extra(n, nseg), &tt);
  std::lock_guard<std::mutex> lk(w->mu);
#define GBK_SEGSCAN(A, TA, B, TB)                                                                              \
  if (din == A && dout == B)                                                                                   \
    return inclusive ? launch_seg<TA, TB, GBK_SUM, M_INCL>((const TA*)x, (TB*)y, n, offsets, nseg, w, tune)     \
                     : launch_seg<TA, TB, GBK_SUM, M_EXCL>((const TA*)x, (TB*)y, n, offsets, nseg, w, tune);
  GBK_SEGSCAN(GBK_I32, int32_t, GBK_I32, int32_t)
  GBK_SEGSCAN(GBK_I32, int32_t, GBK_I64, int64_t)
  GBK_SEGSCAN(GBK_I64, int64_t, GBK_I64, int64_t)
  GBK_SEGSCAN(GBK_F32, float, GBK_F32, float)
  GBK_SEGSCAN(GBK_F64, double, GBK_F64, double)
#undef GBK_SEGSCAN
  return GBK_ERR_UNSUPPORTED;
}

}  // extern "C"
