// Decoupled look-back over tile descriptors (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", NVIDIA NVR-2016-002), shared
// by the plain scan (gbk_scan.cu) and the batched segmented reduce / scan
// (gbk_segmented.cu).
//
// A tile's descriptor is 16 bytes: two 64-bit words, each {tag (32 bits) :
// half of the value (32 bits)}, tag = (epoch << 2) | status with status 1 =
// aggregate, 2 = inclusive prefix.  Each word is a single-copy-atomic access
// and every (epoch, status) of a tile is published once, so a reader that
// finds the same tag in both words holds both halves of that publication; a
// torn read shows two tags and counts as not ready.  No fence on either side.
// (128-bit single-copy-atomic loads would do the same in one access, but those
// were served one at a time, about 850 cycles each under load.)  The epoch
// (30 bits, fresh per launch) makes stale descriptors read as "not ready", so
// nothing is cleared per launch.  Descriptors sit one per 128-byte line:
// hundreds of look-backs poll the few KB behind the frontier, and packed 16
// bytes apart they loaded a handful of L2 slices (round trips of several
// microseconds).
#pragma once

#include "gbk_internal.cuh"

namespace gbk {

constexpr unsigned LB_FLAG_A = 1;  // tile aggregate available
constexpr unsigned LB_FLAG_P = 2;  // inclusive prefix available
constexpr int LB_DESC_STRIDE = 8;  // TileDesc units between descriptors (128 bytes)

struct alignas(16) TileDesc {
  unsigned long long w0, w1;
};

struct LbState {
  TileDesc* desc;
  int* err;
  unsigned epoch;  // 30 bits
  int64_t ntiles;
  int64_t wait_limit;
};

// Status words needed for `ntiles` descriptors (in u32 units, for ws_flags).
inline size_t lb_flag_words(int64_t ntiles) {
  return (size_t)ntiles * LB_DESC_STRIDE * (sizeof(TileDesc) / sizeof(unsigned));
}

__device__ __forceinline__ TileDesc* lb_desc(const LbState& S, int64_t t) { return S.desc + t * LB_DESC_STRIDE; }

__device__ __forceinline__ void lb_store(TileDesc* p, unsigned tag, unsigned long long bits) {
  const unsigned long long w0 = ((unsigned long long)tag << 32) | (bits & 0xFFFFFFFFull);
  const unsigned long long w1 = ((unsigned long long)tag << 32) | (bits >> 32);
  asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(w0), "l"(w1) : "memory");
}
// tag = 0 (never a valid tag: epochs start at 1) when the two words disagree.
__device__ __forceinline__ void lb_load(const TileDesc* p, unsigned* tag, unsigned long long* bits) {
  unsigned long long w0, w1;
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(w0), "=l"(w1) : "l"(p) : "memory");
  const unsigned t0 = (unsigned)(w0 >> 32), t1 = (unsigned)(w1 >> 32);
  *tag = t0 == t1 ? t0 : 0u;
  *bits = (w0 & 0xFFFFFFFFull) | (w1 << 32);
}
template <class TO>
__device__ __forceinline__ unsigned long long lb_bits(TO v) {
  unsigned long long b = 0;
  memcpy(&b, &v, sizeof(TO));
  return b;
}
template <class TO>
__device__ __forceinline__ TO lb_value(unsigned long long b) {
  TO v;
  memcpy(&v, &b, sizeof(TO));
  return v;
}
// Publish a tile's aggregate or inclusive prefix.
template <class TO>
__device__ __forceinline__ void lb_publish(const LbState& S, int64_t tile, unsigned status, TO v) {
  lb_store(lb_desc(S, tile), (S.epoch << 2) | status, lb_bits(v));
}

// Commutative operators of the look-back (sum, min, max).
template <class T> struct LbSum {
  __device__ static T id() { return T(0); }
  __device__ static T f(T a, T b) { return a + b; }
};

// Descriptors per lane in a look-back window: 256 predecessors per round trip
// for 4-byte values, 128 for 8-byte values (register budget).
template <class TO> constexpr int lb_k() { return sizeof(TO) == 8 ? 4 : 8; }

// Look-back for `tile` (> 0, its aggregate or prefix already published) by one
// full warp: combines predecessors' aggregates back to the nearest inclusive
// prefix; returns the exclusive prefix (in every lane).  When `publish` is
// set, the tile's inclusive prefix f(exclusive, agg) goes out.  A window is
// 32 * K descriptors, lane l holding distances l*K .. l*K+K-1 from the window
// start, all loaded at once.  `bad` is set when a wait gave up; the missing
// prefix then counts as the identity.
template <class TO, int K, class OP>
__device__ __forceinline__ TO look_back(const LbState& S, int64_t tile, TO agg, bool publish, bool* bad) {
  static_assert(K >= 1 && K <= 16, "descriptors per lane");
  const int lane = threadIdx.x & 31;
  const unsigned ep = S.epoch << 2;
  constexpr unsigned ALL = (1u << K) - 1u;
  TO excl = OP::id();
  int64_t base = tile - 1;
  while (true) {
    unsigned long long val[K];
    unsigned okm = 0, pm = 0;  // per entry: status valid / inclusive prefix
    const int64_t p0 = base - (int64_t)lane * K;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      val[j] = lb_bits(OP::id());
      if (p0 - j < 0) {  // before tile 0: the identity, as a prefix
        okm |= 1u << j;
        pm |= 1u << j;
      } else {
        unsigned tg;
        lb_load(lb_desc(S, p0 - j), &tg, &val[j]);
        if ((tg & ~3u) == ep && (tg & 3u)) okm |= 1u << j;
        if (tg == (ep | LB_FLAG_P)) pm |= 1u << j;
      }
    }
    int64_t polls = 0;
    unsigned ns = 0, need, lanes_p;
    while (true) {
      // Entries that count: everything before the nearest prefix and that
      // prefix itself (lowest lane holding one, then its lowest entry).
      lanes_p = __ballot_sync(0xffffffffu, pm != 0);
      const int lp = lanes_p ? __ffs(lanes_p) - 1 : 32;
      need = lane < lp ? ALL : (lane == lp ? (pm ^ (pm - 1u)) & ALL : 0u);
      const unsigned miss = need & ~okm;
      if (!__ballot_sync(0xffffffffu, miss != 0)) break;
      if (++polls > S.wait_limit) {
        // Give up; still publish, so that successors do not wait as well.
        *bad = true;
        if (lane == 0 && publish) lb_publish(S, tile, LB_FLAG_P, agg);
        return OP::id();
      }
      if (polls > 2) {
        ns = ns ? (ns < 256 ? ns * 2 : 256) : 32;
        __nanosleep(ns);
      }
#pragma unroll
      for (int j = 0; j < K; ++j) {
        if ((miss >> j) & 1u) {
          unsigned tg;
          lb_load(lb_desc(S, p0 - j), &tg, &val[j]);
          if ((tg & ~3u) == ep && (tg & 3u)) okm |= 1u << j;
          if (tg == (ep | LB_FLAG_P)) pm |= 1u << j;
        }
      }
    }
    TO v = OP::id();
#pragma unroll
    for (int j = 0; j < K; ++j)
      if ((need >> j) & 1u) v = OP::f(v, lb_value<TO>(val[j]));
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v = OP::f(v, __shfl_xor_sync(0xffffffffu, v, m));
    excl = OP::f(excl, v);
    if (lanes_p) break;
    base -= 32 * K;
  }
  if (lane == 0 && publish) lb_publish(S, tile, LB_FLAG_P, OP::f(excl, agg));
  return excl;
}

}  // namespace gbk
