// Batched segmented reduce and scan: thousands of uneven segments in one
// launch.  Replaces the TeamPolicy league pattern "one team per segment,
// TeamThreadRange reduce / scan inside" (core/src/OpenMP/Kokkos_OpenMP_Parallel_Reduce.hpp:332-530,
// core/src/Cuda/Kokkos_Cuda_Parallel_Team.hpp:589-980) and the loop of one
// parallel_reduce / inclusive_scan launch per segment.
//
// Segments are given by offsets[0..nseg] (segment s = [offsets[s],
// offsets[s+1]), non-decreasing, offsets[0] = 0, offsets[nseg] = n).  The
// concatenated array is cut into fixed tiles of 256 * IPT 16-byte vectors,
// independent of the segment lengths, so the work is balanced whatever the
// length distribution.  One persistent, warp-specialised kernel on a
// cooperative (co-resident) grid, CTA b owning tiles b, b + G, ...:
//   * phase 0 (all threads): zero a head bitmap (one bit per element), grid
//     barrier, then one bit per segment start and, per tile, the first
//     segment starting in it; identities for empty segments (reduce); grid
//     barrier.  Bounded waits;
//   * the tile pipeline of the plain scan (gbk_scan.cu): each tile's input
//     and its bitmap row arrive by one bulk copy into a two-stage ring; the
//     compute warps do the tile sums of tile i+1 and then the outputs of tile
//     i; look-back warps resolve the carry into each tile.  The operator is
//     the segmented one on pairs (head seen, value):
//     (h1, v1) . (h2, v2) = (h1 | h2, h2 ? v2 : v1 op v2).  A tile holding a
//     head publishes its inclusive prefix (the value after its last head) at
//     once, so long chains only form inside long segments;
//   * reduce mode writes each segment's total at its last element; scan
//     modes write every element through a shared-memory out tile.
#include <algorithm>
#include <type_traits>

#include "gbk_lookback.cuh"

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

constexpr int SEG_COMPUTE = 256;  // compute threads
constexpr int SEG_NLB = 4;        // look-back warps, tile slots round-robin
constexpr int SEG_BLOCK = SEG_COMPUTE + 32 * SEG_NLB;
constexpr int SBAR_INFO = 1, SBAR_PREFIX = 1 + SEG_NLB, SBAR_COMPUTE = 1 + 2 * SEG_NLB;
constexpr int SBAR_HANDOFF = SEG_COMPUTE + 32;
static_assert(SBAR_COMPUTE <= 15, "named barrier ids");

struct SegArgs {
  const int64_t* offsets;
  int64_t nseg;
  unsigned* bitmap;   // (ntiles + 1) rows of TILE / 32 words, then 4 spare words
  int64_t* tile_lo;   // [ntiles + 1]: first segment s with offsets[s] >= t * TILE
  unsigned* arrive;   // grid barrier counters (zero between launches)
  unsigned* depart;
};

// Bounded grid barrier of a co-resident grid; `target` counts CTAs arrived so
// far over all barriers of the launch.  False when it gave up.
__device__ bool grid_barrier(unsigned* arrive, unsigned target, int64_t limit, int* s_ok) {
  __threadfence();  // every thread's writes, before the CTA's arrival
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(arrive, 1u);
    int64_t polls = 0;
    int ok = 1;
    while (ld_acquire_u32(arrive) < target) {
      if (++polls > limit) {
        ok = 0;
        break;
      }
      __nanosleep(polls < 8 ? 32 : 256);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

// Phase 0: head bitmap, per-tile first segment, empty-segment identities.
template <class TO, int OP, int MODE>
__device__ void seg_phase0(const SegArgs& A, TO* y, int64_t n, int64_t tile_elems, int64_t ntiles,
                           int64_t wait_limit, bool* bad, int* s_ok) {
  using O = SOp<TO, OP>;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int64_t words = (ntiles + 1) * (tile_elems / 32) + 4;
  for (int64_t i = tid; i < words; i += nthr) A.bitmap[i] = 0u;
  if (!grid_barrier(A.arrive, gridDim.x, wait_limit, s_ok)) *bad = true;
  for (int64_t s = tid; s <= A.nseg; s += nthr) {
    const int64_t p = A.offsets[s];
    if (s < A.nseg && p < n) atomicOr(A.bitmap + p / 32, 1u << (p & 31));
    // Tiles whose first element falls in (offsets[s-1], offsets[s]] start at s.
    const int64_t prev = s > 0 ? A.offsets[s - 1] : -1;
    int64_t t0 = prev < 0 ? 0 : prev / tile_elems + 1;
    const int64_t t1 = p / tile_elems;  // last tile t with t * tile_elems <= p
    for (int64_t t = t0; t <= t1 && t <= ntiles; ++t) A.tile_lo[t] = s;
    if (MODE == M_REDUCE && s < A.nseg && A.offsets[s + 1] == p) y[s] = O::id();
  }
  // Tiles past the last segment start (only when offsets end below n).
  for (int64_t t = A.offsets[A.nseg] / tile_elems + 1 + tid; t <= ntiles; t += nthr) A.tile_lo[t] = A.nseg + 1;
  if (!grid_barrier(A.arrive, 2 * gridDim.x, wait_limit, s_ok)) *bad = true;
}

template <class T> __device__ __forceinline__ T sh_up(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }

// FAST: x (and, for scans, y) 16-byte aligned: input tiles by bulk copy,
// scan outputs through the out tile.  Otherwise direct element loads and
// stores with the same mapping.  Compute thread i owns the C = IPT * VEC
// consecutive elements starting at i * C (IPT odd: conflict-free shared
// reads); C <= 32, so its head bits (and the next element's) sit in one
// 64-bit window of the bitmap row.
template <class TI, class TO, int OP, int MODE, bool FAST, int IPT, int STG>
__global__ void __launch_bounds__(SEG_BLOCK, 2)
    k_seg(const TI* __restrict__ x, TO* __restrict__ y, int64_t n, SegArgs A, LbState S) {
  using O = SOp<TO, OP>;
  constexpr int VEC = 16 / sizeof(TI);
  constexpr int C = IPT * VEC;
  constexpr int WARPS = SEG_COMPUTE / 32;
  constexpr int OVN = (int)(VEC * sizeof(TO) / 16);
  constexpr int OV = 16 / sizeof(TO);
  constexpr int64_t TILE = (int64_t)SEG_COMPUTE * C;
  constexpr unsigned long long CMASK = (1ull << C) - 1ull;  // head bits of this thread's C elements
  constexpr unsigned IN_BYTES = (unsigned)SEG_COMPUTE * IPT * 16;
  constexpr unsigned BM_BYTES = (unsigned)(TILE / 8) + 16;  // the tile's row and the next row's first word
  constexpr unsigned STAGE_BYTES = (IN_BYTES + BM_BYTES + 127) / 128 * 128;
  constexpr bool OUT_TILE = FAST && MODE != M_REDUCE;
  static_assert(IPT % 2 == 1 && C <= 32, "odd vector count, at most 32 elements per thread");
  static_assert(OVN == 1 || OVN == 2, "output at most twice the input width");
  static_assert(STG >= 2, "the stage of tile i+1 is summed while tile i is written");
  extern __shared__ __align__(128) unsigned char dsm[];  // STG stages {input, bitmap row}, then the out tile
  __shared__ __align__(8) unsigned long long s_bar[STG];
  __shared__ int64_t s_info_tile[SEG_NLB];
  __shared__ TO s_info_agg[SEG_NLB];
  __shared__ unsigned s_info_h[SEG_NLB];  // head / first-element head / segment end flags
  __shared__ TO s_excl[SEG_NLB];
  __shared__ TO s_wv[2][WARPS];
  __shared__ unsigned s_wh[2][WARPS];
  __shared__ int s_bad, s_ok;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nin = FAST ? n / VEC * VEC : 0;
  const int64_t nout = OUT_TILE ? n / OV * OV : 0;
  unsigned char* outt = dsm + (size_t)STG * STAGE_BYTES;
  auto tile_of = [&](int j) { return (int64_t)blockIdx.x + (int64_t)j * gridDim.x; };

  if (threadIdx.x == 0) {
    s_bad = 0;
#pragma unroll
    for (int q = 0; q < STG; ++q) mbar_init(&s_bar[q], 1);
    fence_mbar_init();
  }
  bool bad = false;
  seg_phase0<TO, OP, MODE>(A, y, n, TILE, S.ntiles, S.wait_limit, &bad, &s_ok);

  // Thread 0 only: start the copies of the CTA's j-th tile (input and bitmap row).
  auto fill = [&](int j) {
    const int64_t t = tile_of(j);
    if (t >= S.ntiles) return;
    const int s = j % STG;
    unsigned char* stg = dsm + (size_t)s * STAGE_BYTES;
    const int64_t e0 = t * TILE;
    const int64_t cnt = FAST ? (nin - e0 < TILE ? nin - e0 : TILE) : 0;
    const unsigned in_bytes = cnt > 0 ? (unsigned)(cnt * (int64_t)sizeof(TI)) : 0u;
    mbar_arrive_expect_tx(&s_bar[s], in_bytes + BM_BYTES);
    if (in_bytes) bulk_g2s(stg, x + e0, in_bytes, &s_bar[s]);
    bulk_g2s(stg + IN_BYTES, A.bitmap + t * (TILE / 32), BM_BYTES, &s_bar[s]);
  };
  if (threadIdx.x == 0) {
    // The bitmap was written through the generic proxy; the bulk copies read
    // it through the async proxy.
    asm volatile("fence.proxy.async;" ::: "memory");
#pragma unroll
    for (int q = 0; q < STG; ++q) fill(q);
  }
  __syncthreads();

  if (warp >= WARPS) {
    // ---- look-back warp k: the CTA's tile slots k, k + NLB, ... -------------
    const int k = warp - WARPS;
    while (true) {
      bar_sync(SBAR_INFO + k, SBAR_HANDOFF);
      const int64_t tile = s_info_tile[k];
      if (tile >= S.ntiles) break;
      const TO agg = s_info_agg[k];
      const unsigned hf = s_info_h[k];
      // No carry needed when the tile starts a segment, nor (reduce) when no
      // segment ends in it: its aggregate is all that later tiles need.  A
      // tile holding a head has published its prefix already.
      const bool skip = tile == 0 || (hf & 2u) || (MODE == M_REDUCE && !(hf & 4u));
      const TO excl = skip ? O::id() : look_back<TO, lb_k<TO>(), O>(S, tile, agg, !(hf & 1u), &bad);
      if (lane == 0) s_excl[k] = excl;
      bar_arrive(SBAR_PREFIX + k, SBAR_HANDOFF);
    }
  } else {
    // ---- compute warps ------------------------------------------------------
    const int r0 = threadIdx.x * C;  // this thread's first element in the tile
    auto load_vec = [&](int s, int64_t tbase, int jj, TI (&v)[VEC]) {
      const int64_t e0 = tbase + r0 + jj * VEC;
      const unsigned char* stg = dsm + (size_t)s * STAGE_BYTES;
      if (FAST && tbase + TILE <= nin) {
        Vec16<TI> u;
        u.u = reinterpret_cast<const uint4*>(stg)[threadIdx.x * IPT + jj];
#pragma unroll
        for (int q = 0; q < VEC; ++q) v[q] = u.v[q];
      } else if (FAST) {
        const TI* sv = reinterpret_cast<const TI*>(stg) + r0 + jj * VEC;
#pragma unroll
        for (int q = 0; q < VEC; ++q) v[q] = e0 + q < nin ? sv[q] : (e0 + q < n ? x[e0 + q] : TI(0));
      } else {
#pragma unroll
        for (int q = 0; q < VEC; ++q) v[q] = e0 + q < n ? x[e0 + q] : TI(0);
      }
    };
    // Elements of this thread's C that exist in a tile starting at tbase
    // (C for every tile but the last): one small-integer compare per element.
    auto thread_valid = [&](int64_t tbase) -> int {
      const int64_t rem = n - (tbase + r0);
      return rem <= 0 ? 0 : (rem >= C ? C : (int)rem);
    };
    // Head bits of this thread's elements (bit k: element r0 + k) and the next.
    auto head_bits = [&](int s) -> unsigned long long {
      const unsigned* bm = reinterpret_cast<const unsigned*>(dsm + (size_t)s * STAGE_BYTES + IN_BYTES);
      const int w = r0 >> 5;
      return ((unsigned long long)bm[w] | ((unsigned long long)bm[w + 1] << 32)) >> (r0 & 31);
    };
    // Tile sums of the CTA's j-th tile: this thread's exclusive pair within
    // its warp (eh, ev) and its warp's within the tile (wh, wv); thread 0
    // publishes the tile's aggregate (its prefix, if it holds a head).
    auto tile_sums = [&](int j, int64_t tile, unsigned& eh, TO& ev, unsigned& wh, TO& wv) {
      const int s = j % STG;
      if (!mbar_wait(&s_bar[s], (unsigned)(j / STG) & 1u, S.wait_limit)) bad = true;
      const unsigned long long hb = head_bits(s);
      const int64_t tbase = tile * TILE;
      const int valid = thread_valid(tbase);
      TO a = O::id();
      unsigned h = 0;
      if (valid == C && (hb & CMASK) == 0) {  // no head among this thread's elements: plain fold
#pragma unroll
        for (int jj = 0; jj < IPT; ++jj) {
          TI v[VEC];
          load_vec(s, tbase, jj, v);
#pragma unroll
          for (int q = 0; q < VEC; ++q) a = O::f(a, (TO)v[q]);
        }
      } else {
#pragma unroll
        for (int jj = 0; jj < IPT; ++jj) {
          TI v[VEC];
          load_vec(s, tbase, jj, v);
#pragma unroll
          for (int q = 0; q < VEC; ++q) {
            const int kk = jj * VEC + q;
            if ((hb >> kk) & 1u) {
              a = O::id();
              h = 1;
            }
            if (kk < valid) a = O::f(a, (TO)v[q]);
          }
        }
      }
      TO iv = a;
      unsigned ih = h;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const TO ov = sh_up(iv, d);
        const unsigned oh = sh_up(ih, d);
        if (lane >= d) {
          if (!ih) iv = O::f(ov, iv);
          ih |= oh;
        }
      }
      ev = sh_up(iv, 1);
      eh = sh_up(ih, 1);
      if (lane == 0) {
        ev = O::id();
        eh = 0;
      }
      // Reduce: does a segment end among this warp's elements?  (A head at
      // element r0 + k, k = 1..C, ends the segment at r0 + k - 1.)
      bool my_end = false;
      if (MODE == M_REDUCE) {
        const int64_t e_first = tbase + r0;
        my_end = e_first < n && ((((hb >> 1) & ((1ull << C) - 1ull)) != 0) || (n - 1 < e_first + C));
      }
      const unsigned wend = __any_sync(0xffffffffu, my_end) ? 2u : 0u;
      if (lane == 31) {
        s_wv[j & 1][warp] = iv;
        s_wh[j & 1][warp] = ih | wend;
      }
      bar_sync(SBAR_COMPUTE, SEG_COMPUTE);
      TO agg = O::id();
      unsigned ah = 0, tend = 0;
      wv = O::id();
      wh = 0;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        if (w == warp) {
          wv = agg;
          wh = ah;
        }
        const TO sv = s_wv[j & 1][w];
        const unsigned shh = s_wh[j & 1][w];
        agg = (shh & 1u) ? sv : O::f(agg, sv);
        ah |= shh & 1u;
        tend |= shh >> 1;
      }
      if (threadIdx.x == 0) {
        lb_publish(S, tile, (tile == 0 || ah) ? LB_FLAG_P : LB_FLAG_A, agg);
        s_info_tile[j % SEG_NLB] = tile;
        s_info_agg[j % SEG_NLB] = agg;
        // bit 0: a head in the tile, 1: a head at its first element (thread 0
        // owns element 0), 2: a segment ends in it
        s_info_h[j % SEG_NLB] = ah | ((unsigned)(hb & 1u) << 1) | (tend << 2);
      }
    };
    auto hand_off = [&](int j) { bar_arrive(SBAR_INFO + j % SEG_NLB, SBAR_HANDOFF); };

    unsigned q_eh = 0, q_wh = 0;  // pairs of the tile summed but not yet written
    TO q_ev = O::id(), q_wv = O::id();
    if (tile_of(0) < S.ntiles) {
      tile_sums(0, tile_of(0), q_eh, q_ev, q_wh, q_wv);
      hand_off(0);
    }
    int i = 0;
    for (; tile_of(i) < S.ntiles; ++i) {
      unsigned n_eh = 0, n_wh = 0;
      TO n_ev = O::id(), n_wv = O::id();
      if (tile_of(i + 1) < S.ntiles) {
        tile_sums(i + 1, tile_of(i + 1), n_eh, n_ev, n_wh, n_wv);
        hand_off(i + 1);
      }
      bar_sync(SBAR_PREFIX + i % SEG_NLB, SBAR_HANDOFF);
      const TO excl = s_excl[i % SEG_NLB];

      // ---- output pass of the CTA's i-th tile (stage i % STG) ----------------
      const int s = i % STG;
      const int64_t tile = tile_of(i);
      const int64_t tbase = tile * TILE;
      const unsigned long long hb = head_bits(s);
      const TO v1 = q_wh ? q_wv : O::f(excl, q_wv);  // carry into this warp
      TO run = q_eh ? q_ev : O::f(v1, q_ev);         // carry into this thread
      const bool out_full = OUT_TILE && tbase + TILE <= nout;
      const int valid = thread_valid(tbase);
      // Reduce: nothing to write from a tile in which no segment ends.
      const int passes = (MODE != M_REDUCE || (s_info_h[i % SEG_NLB] & 4u)) ? IPT : 0;
      // Scans: no head among this thread's elements (segments are usually
      // far longer than C): one operator application per element.
      const bool plain = MODE != M_REDUCE && valid == C && (hb & CMASK) == 0;
#pragma unroll
      for (int jj = 0; jj < IPT; ++jj) {
        if (jj >= passes) break;
        TI v[VEC];
        load_vec(s, tbase, jj, v);
        TO o[VEC];
        if (plain) {
#pragma unroll
          for (int q = 0; q < VEC; ++q) {
            if (MODE == M_EXCL) o[q] = run;
            run = O::f(run, (TO)v[q]);
            if (MODE == M_INCL) o[q] = run;
          }
        } else {
#pragma unroll
          for (int q = 0; q < VEC; ++q) {
            const int kk = jj * VEC + q;
            const int64_t e = tbase + r0 + kk;
            if ((hb >> kk) & 1u) run = O::id();
            if (MODE == M_EXCL) o[q] = run;
            if (kk < valid) run = O::f(run, (TO)v[q]);
            if (MODE == M_INCL) o[q] = run;
            if (MODE == M_REDUCE && e < n && (((hb >> (kk + 1)) & 1u) || e == n - 1)) {
              // Last element of its segment: the segment is the last s with
              // offsets[s] <= e, among those that can touch this tile.
              int64_t lo = __ldcg(A.tile_lo + tile) - 1, hi = __ldcg(A.tile_lo + tile + 1);
              if (lo < 0) lo = 0;
              if (hi > A.nseg) hi = A.nseg;
              while (hi - lo > 1) {  // offsets[lo] <= e < offsets[hi] (or hi = nseg)
                const int64_t mid = lo + (hi - lo) / 2;
                if (__ldg(A.offsets + mid) <= e) lo = mid; else hi = mid;
              }
              y[lo] = run;
            }
          }
        }
        if (MODE != M_REDUCE) {
          if (OUT_TILE) {
            uint4* ov = reinterpret_cast<uint4*>(outt) + ((size_t)threadIdx.x * IPT + jj) * OVN;
            if constexpr (OVN == 1) {
              Vec16<TO> u;
#pragma unroll
              for (int q = 0; q < VEC; ++q) u.v[q] = o[q];
              ov[0] = u.u;
            } else {
              // Lanes 4..7 of each quarter-warp write their second vector
              // first: with the odd stride each step hits 8 bank groups.
              Vec16<TO> a, b;
#pragma unroll
              for (int q = 0; q < OV; ++q) {
                a.v[q] = o[q];
                b.v[q] = o[OV + q];
              }
              const int flip = (lane >> 2) & 1;
              ov[flip] = flip ? b.u : a.u;
              ov[flip ^ 1] = flip ? a.u : b.u;
            }
            if (!out_full) {
#pragma unroll
              for (int q = 0; q < VEC; ++q) {
                const int64_t e = tbase + r0 + jj * VEC + q;
                if (e >= nout && e < n) y[e] = o[q];
              }
            }
          } else {
#pragma unroll
            for (int q = 0; q < VEC; ++q) {
              const int64_t e = tbase + r0 + jj * VEC + q;
              if (e < n) y[e] = o[q];
            }
          }
        }
      }
      // Stage s (and the out tile) complete: refill the stage, and stream the
      // out tile in warp-striped order (512 contiguous bytes per warp
      // instruction).  The out tile is next written after the next prefix
      // barrier.
      bar_sync(SBAR_COMPUTE, SEG_COMPUTE);
      if (threadIdx.x == 0) fill(i + STG);
      if (OUT_TILE) {
        const uint4* ov = reinterpret_cast<const uint4*>(outt);
        uint4* yv = reinterpret_cast<uint4*>(y + tbase);
        const int64_t left = nout - tbase < TILE ? nout - tbase : TILE;
        const int64_t nvec = left > 0 ? left * (int64_t)sizeof(TO) / 16 : 0;
#pragma unroll
        for (int k = 0; k < IPT * OVN; ++k) {
          const int q = k * SEG_COMPUTE + threadIdx.x;
          if (out_full || q < nvec) __stcs(yv + q, ov[q]);
        }
      }
      q_eh = n_eh;
      q_ev = n_ev;
      q_wh = n_wh;
      q_wv = n_wv;
    }
    // i = the number of tiles handed off: one end mark per look-back warp.
    for (int j = i; j < i + SEG_NLB; ++j) {
      if (threadIdx.x == 0) s_info_tile[j % SEG_NLB] = S.ntiles;
      hand_off(j);
    }
  }

  if (bad) s_bad = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_bad) atomicOr(S.err, GBK_EBIT_TIMEOUT);
    // The last CTA to leave resets the barrier counters for the next launch
    // (every CTA has passed both barriers by then).
    __threadfence();
    if (atomicAdd(A.depart, 1u) == gridDim.x - 1) {
      *A.arrive = 0u;
      *A.depart = 0u;
    }
  }
}

// ---- segmented reduce over contiguous CTA shares -----------------------------
// One launch with no waits between CTAs (a plain grid, any residency).  CTA b
// owns a contiguous, balanced share [a, e) of the elements (whole 16-byte
// vectors; the last CTA also the tail) and streams it in 16 KiB chunks by bulk
// copies through a 4-stage ring, walking the segments in order:
//  * a chunk that lies inside the current segment (next segment start >= the
//    chunk's end: the common case when segments are longer than a chunk) is
//    taken into registers, its stage handed back, and folded into per-thread
//    accumulators, as the flat reduce does;
//  * a chunk holding segment starts is cut at them: the current segment's
//    piece before the first start and the piece after the last start are
//    folded by the whole CTA (element-striped, masked); every piece between
//    two starts is a whole segment, folded by one warp (pieces round-robin
//    over the warps) and written; starts are read from the offsets 256 at a
//    time;
//  * a segment that begins and ends inside the CTA is written directly; the
//    pieces of a segment that crosses a CTA boundary go to two records per
//    CTA, and the last CTA to finish (one ticket) joins each run of records
//    of one segment in CTA order and writes it.
// Empty segments get the identity in a grid-stride pre-pass.  Every join
// happens in a fixed order, so results are deterministic for a given grid.
template <class T>
struct SegRec {
  int64_t seg;  // < 0: no record
  T val;
};

struct SegRedArgs {
  const int64_t* offsets;
  int64_t nseg, n, nvec;
  void* recs;        // SegRec<T>[2 * gridDim.x]
  unsigned* ticket;  // zero between launches
  int* err;
  int64_t wait_limit;
};

constexpr int SR_BLOCK = 256, SR_CV = 1024, SR_STAGES = 4;

template <class R, class T>
struct SegRedCta {
  using V = typename R::V;
  static constexpr int VEC = 16 / sizeof(T);
  static constexpr int WARPS = SR_BLOCK / 32;
  int64_t* s_win;
  int64_t* s_wb;
  V* s_red0;
  V* s_red1;
  int64_t* s_cur;
  int64_t* s_next;
  V* s_carry;
  int* s_started;
  SegRec<T>* rec_first;

  // Refill the window of starts: s_win[t] = offsets[base + t].
  __device__ void load_window(int64_t base, const SegRedArgs& A) const {
    __syncthreads();  // earlier readers of s_win are done
    const int tid = threadIdx.x;
    s_win[tid] = base + tid <= A.nseg ? A.offsets[base + tid] : (int64_t)0x7FFFFFFFFFFFFFFFLL;
    if (tid == 0) *s_wb = base;
    __syncthreads();
  }

  // A chunk [c0, c1) that holds at least one segment start; get(i) reads
  // element i.  The starts come from the window of offsets cached in shared
  // memory (s_win[t] = offsets[*s_wb + t]), refilled only when more than its
  // 256 entries are consumed.  `acc` (the per-thread partials of the current
  // segment) joins the first piece, and is reset.
  template <class Get>
  __device__ void slow(const Get& get, int64_t c0, int64_t c1, V& acc, T* out, const SegRedArgs& A) const {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int64_t seg = *s_cur, prev = c0, first_b = c0, last_b = c0, next_start = 0;
    bool first_window = true;
    while (true) {
      const int64_t j0l = seg + 1 - *s_wb;  // window slot of the next start not yet consumed
      if (j0l >= SR_BLOCK) {
        load_window(seg + 1, A);
        continue;
      }
      const int j0 = (int)j0l;
      const int m = __syncthreads_count(tid >= j0 && s_win[tid] < c1);  // sorted: slots [j0, j0 + m)
      for (int q = warp; q < m; q += WARPS) {
        if (first_window && q == 0) continue;  // the first piece: folded by the whole CTA below
        const int jj = j0 + q;
        const int64_t lo = q == 0 ? prev : s_win[jj - 1], hi = s_win[jj];
        if (hi <= lo) continue;  // empty segment: identity from the pre-pass
        V v = R::init();
        for (int64_t i = lo + lane; i < hi; i += 32) R::template update<true>(v, get(i), 0);
        v = WarpRed<R>::run(v);
        if (lane == 0) out[seg + q] = v;  // a whole segment inside this chunk
      }
      if (m > 0) {
        if (first_window) first_b = s_win[j0];
        last_b = s_win[j0 + m - 1];
        prev = last_b;
      }
      seg += m;
      first_window = false;
      if (j0 + m < SR_BLOCK) {
        next_start = s_win[j0 + m];
        break;
      }
      load_window(seg + 1, A);
    }
    V fp = acc, lp = R::init();
    acc = R::init();
    for (int64_t i = c0 + tid; i < c1; i += SR_BLOCK) {
      if (i < first_b) R::template update<true>(fp, get(i), 0);
      else if (i >= last_b) R::template update<true>(lp, get(i), 0);
    }
    const V F = block_reduce<R, SR_BLOCK>(fp, s_red0);
    const V L = block_reduce<R, SR_BLOCK>(lp, s_red1);
    if (tid == 0) {
      V tot = *s_carry;
      R::join(tot, F);
      if (*s_started) {
        out[*s_cur] = tot;
      } else {  // began before this CTA's share: the fix-up joins it
        rec_first->seg = *s_cur;
        rec_first->val = tot;
      }
      *s_cur = seg;
      *s_carry = L;
      *s_started = 1;
      *s_next = next_start;
    }
    __syncthreads();
  }
};

template <class T>
struct SmemGet {
  const T* s;
  int64_t c0;
  __device__ T operator()(int64_t i) const { return s[i - c0]; }
};
template <class T>
struct GlobalGet {
  const T* x;
  __device__ T operator()(int64_t i) const { return x[i]; }
};

template <class R, class T>
__global__ void __launch_bounds__(SR_BLOCK) k_segred(const T* __restrict__ x, T* __restrict__ out, SegRedArgs A) {
  using V = typename R::V;
  constexpr int VEC = 16 / sizeof(T);
  constexpr unsigned CHUNK_BYTES = (unsigned)SR_CV * 16;
  constexpr int WARPS = SR_BLOCK / 32;
  extern __shared__ __align__(128) unsigned char ring[];
  __shared__ __align__(8) unsigned long long s_bar[SR_STAGES];
  __shared__ int64_t s_win[SR_BLOCK];
  __shared__ V s_red0[WARPS], s_red1[WARPS];
  __shared__ int64_t s_cur, s_next, s_lo, s_hi, s_wb;
  __shared__ V s_carry;
  __shared__ int s_started;
  __shared__ unsigned s_ticket;
  SegRec<T>* recs = (SegRec<T>*)A.recs;
  const int tid = threadIdx.x;
  const int64_t G = gridDim.x, b = blockIdx.x;
  const int64_t per = A.nvec / G, rem = A.nvec % G;
  const int64_t v0 = b * per + (b < rem ? b : rem);
  const int64_t v1 = v0 + per + (b < rem ? 1 : 0);
  const int64_t a = v0 * VEC;
  const int64_t e = b == G - 1 ? A.n : v1 * VEC;
  const int64_t nchunks = (v1 - v0 + SR_CV - 1) / SR_CV;
  // Thread 0 only: start the copy of chunk c into its stage.
  auto fill = [&](int64_t c) {
    if (c >= nchunks) return;
    const int st = (int)(c % SR_STAGES);
    const int64_t cv0 = v0 + c * SR_CV;
    const int64_t cnt = v1 - cv0 < SR_CV ? v1 - cv0 : SR_CV;
    mbar_arrive_expect_tx(&s_bar[st], (unsigned)(cnt * 16));
    bulk_g2s(ring + (size_t)st * CHUNK_BYTES, x + cv0 * VEC, (unsigned)(cnt * 16), &s_bar[st]);
  };
  if (tid == 0) {
#pragma unroll
    for (int st = 0; st < SR_STAGES; ++st) mbar_init(&s_bar[st], 1);
    fence_mbar_init();
    for (int st = 0; st < SR_STAGES; ++st) fill(st);
    recs[2 * b].seg = -1;
    recs[2 * b + 1].seg = -1;
    s_lo = 0;
    s_hi = A.nseg;
  }
  for (int64_t sg = b * SR_BLOCK + tid; sg < A.nseg; sg += G * SR_BLOCK)
    if (A.offsets[sg] == A.offsets[sg + 1]) out[sg] = R::init();
  __syncthreads();
  // The segment of element a: the largest s with offsets[s] <= a
  // (offsets[0] = 0 <= a < n = offsets[nseg]), by rounds of 256 probes.
  while (true) {
    const int64_t lo = s_lo, hi = s_hi;
    if (hi - lo <= 1) break;
    const int64_t step = (hi - lo + SR_BLOCK - 1) / SR_BLOCK;
    const int64_t p = lo + (int64_t)tid * step;
    const int cnt = __syncthreads_count(p < hi && A.offsets[p] <= a);
    if (tid == 0) {
      s_lo = lo + (int64_t)(cnt - 1) * step;
      const int64_t h2 = lo + (int64_t)cnt * step;
      s_hi = h2 < hi ? h2 : hi;
    }
    __syncthreads();
  }
  const SegRedCta<R, T> cta{s_win, &s_wb, s_red0, s_red1, &s_cur, &s_next, &s_carry, &s_started, &recs[2 * b]};
  cta.load_window(s_lo + 1, A);  // the first 256 starts after element a
  if (tid == 0) {
    s_cur = s_lo;
    s_next = s_win[0];
    s_started = A.offsets[s_lo] == a;
    s_carry = R::init();
  }
  __syncthreads();
  V acc = R::init();
  bool bad = false;
  for (int64_t c = 0; c < nchunks; ++c) {
    const int st = (int)(c % SR_STAGES);
    if (!mbar_wait(&s_bar[st], (unsigned)(c / SR_STAGES) & 1u, A.wait_limit)) bad = true;
    const int64_t cv0 = v0 + c * SR_CV;
    const int cnt = (int)(v1 - cv0 < SR_CV ? v1 - cv0 : SR_CV);
    const int64_t c0 = cv0 * VEC, c1 = c0 + (int64_t)cnt * VEC;
    const unsigned char* stage = ring + (size_t)st * CHUNK_BYTES;
    if (s_next >= c1) {
      if (cnt == SR_CV) {
        Vec16<T> u[SR_CV / SR_BLOCK];
#pragma unroll
        for (int k = 0; k < SR_CV / SR_BLOCK; ++k) u[k].u = reinterpret_cast<const uint4*>(stage)[k * SR_BLOCK + tid];
        __syncthreads();  // stage fully read: refill it
        if (tid == 0) fill(c + SR_STAGES);
#pragma unroll
        for (int k = 0; k < SR_CV / SR_BLOCK; ++k)
#pragma unroll
          for (int q = 0; q < VEC; ++q) R::template update<true>(acc, u[k].v[q], 0);
      } else {
        for (int i = tid; i < cnt; i += SR_BLOCK) {
          Vec16<T> u;
          u.u = reinterpret_cast<const uint4*>(stage)[i];
#pragma unroll
          for (int q = 0; q < VEC; ++q) R::template update<true>(acc, u.v[q], 0);
        }
        __syncthreads();
        if (tid == 0) fill(c + SR_STAGES);
      }
    } else {
      cta.slow(SmemGet<T>{reinterpret_cast<const T*>(stage), c0}, c0, c1, acc, out, A);
      if (tid == 0) fill(c + SR_STAGES);  // slow() ends with a barrier: the stage is fully read
    }
  }
  // The tail after the last whole vector (last CTA).
  const int64_t t0 = v1 * VEC;
  if (e > t0) {
    if (s_next >= e) {
      if (t0 + tid < e) R::template update<true>(acc, x[t0 + tid], 0);
    } else {
      cta.slow(GlobalGet<T>{x}, t0, e, acc, out, A);
    }
  }
  const V tot = block_reduce<R, SR_BLOCK>(acc, s_red0);
  if (tid == 0) {
    V cry = s_carry;
    R::join(cry, tot);
    if (s_started && s_next == e) {
      out[s_cur] = cry;  // began and ended inside this share
    } else {
      recs[2 * b + 1].seg = s_cur;
      recs[2 * b + 1].val = cry;
    }
    if (bad) atomicOr(A.err, GBK_EBIT_TIMEOUT);
    __threadfence();
    s_ticket = atomicAdd(A.ticket, 1u);
  }
  __syncthreads();
  if (s_ticket != (unsigned)(G - 1)) return;
  // Last CTA: every share has written its records.  Stage them in shared
  // memory (the ring is idle: every copy has landed), then each record that
  // ends a run of one segment joins the run in CTA order.
  __threadfence();
  const int64_t nr = 2 * G;
  int64_t* r_seg = reinterpret_cast<int64_t*>(ring);
  V* r_val = reinterpret_cast<V*>(ring + (size_t)nr * 8);
  for (int64_t r = tid; r < nr; r += SR_BLOCK) {
    const volatile SegRec<T>* vr = recs + r;
    r_seg[r] = vr->seg;
    r_val[r] = vr->val;
  }
  __syncthreads();
  for (int64_t r = tid; r < nr; r += SR_BLOCK) {
    const int64_t sg = r_seg[r];
    if (sg < 0) continue;
    int64_t q = r + 1;
    while (q < nr && r_seg[q] < 0) ++q;
    if (q < nr && r_seg[q] == sg) continue;  // not the run's last record
    int64_t f = r;
    for (int64_t p = r - 1; p >= 0; --p) {
      if (r_seg[p] < 0) continue;
      if (r_seg[p] != sg) break;
      f = p;
    }
    V v = R::init();
    for (int64_t p = f; p <= r; ++p)
      if (r_seg[p] == sg) R::join(v, r_val[p]);
    out[sg] = v;
  }
  if (tid == 0) *A.ticket = 0u;
}

template <class R, class T>
int launch_segred(const T* x, T* out, int64_t n, const int64_t* offsets, int64_t nseg, Workspace* w) {
  constexpr int VEC = 16 / sizeof(T);
  const int64_t nvec = n / VEC;
  const int64_t chunks = (nvec + SR_CV - 1) / SR_CV;
  auto kfn = k_segred<R, T>;
  constexpr size_t dyn = (size_t)SR_STAGES * SR_CV * 16;
  static std::atomic<int> resident{0};  // CTAs per SM, per instantiation (set once, any host thread)
  if (!resident) {
    GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int r = 0;
    GBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kfn, SR_BLOCK, dyn));
    resident = r > 0 ? r : 1;
  }
  int64_t grid = std::min<int64_t>(chunks, (int64_t)sm_count() * resident);
  if (grid < 1) grid = 1;
  // the fix-up stages 2 records per CTA (8 + sizeof(T) bytes each) in the ring
  if (grid * 2 * (8 + (int64_t)sizeof(T)) > (int64_t)dyn) grid = (int64_t)dyn / (2 * (8 + (int64_t)sizeof(T)));
  int st = GBK_OK;
  char* scr = ws_scratch(w, sizeof(SegRec<T>) * 2 * (size_t)grid + 256, &st);
  if (!scr) return st;
  SegRedArgs A;
  A.offsets = offsets;
  A.nseg = nseg;
  A.n = n;
  A.nvec = nvec;
  A.recs = scr;
  A.ticket = w->counters + SLOT_SEGRED;
  A.err = w->err;
  A.wait_limit = wait_limit();
  kfn<<<(unsigned)grid, SR_BLOCK, dyn, w->stream>>>(x, out, A);
  note_launch();
  return cuda_status(cudaGetLastError());
}

// One cooperative launch (all CTAs co-resident: the grid barriers and the
// static tile order need it): min(tiles, resident CTAs), or ctas_per_sm x SMs
// when the tuning asks for fewer.
template <class TI, class TO, int OP, int MODE, bool FAST, int IPT, int STG>
int launch_k_seg(const TI* x, TO* y, int64_t n, const int64_t* offsets, int64_t nseg, Workspace* w, int cps) {
  constexpr int VEC = 16 / sizeof(TI);
  constexpr int64_t TILE = (int64_t)SEG_COMPUTE * IPT * VEC;
  constexpr size_t IN_BYTES = (size_t)SEG_COMPUTE * IPT * 16;
  constexpr size_t STAGE_BYTES = (IN_BYTES + TILE / 8 + 16 + 127) / 128 * 128;
  constexpr size_t OUT_BYTES = (FAST && MODE != M_REDUCE) ? IN_BYTES * (sizeof(TO) / sizeof(TI)) : 0;
  const size_t dyn = STG * STAGE_BYTES + OUT_BYTES;
  const int64_t nt = (n + TILE - 1) / TILE;
  const int64_t ntiles = nt > 0 ? nt : 1;  // one tile still runs phase 0 (empty-segment identities)
  if (ntiles >= ((int64_t)1 << 31)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  const size_t bm_bytes = (((size_t)(ntiles + 1) * (TILE / 32) + 4) * 4 + 255) / 256 * 256;
  const size_t lo_bytes = ((size_t)(ntiles + 1) * 8 + 255) / 256 * 256;
  char* scr = ws_scratch(w, bm_bytes + lo_bytes, &st);
  if (!scr) return st;
  LbState S;
  S.desc = (TileDesc*)ws_flags(w, lb_flag_words(ntiles), &S.epoch, &st);
  if (!S.desc) return st;
  S.err = w->err;
  S.ntiles = ntiles;
  S.wait_limit = wait_limit();
  SegArgs A;
  A.offsets = offsets;
  A.nseg = nseg;
  A.bitmap = (unsigned*)scr;
  A.tile_lo = (int64_t*)(scr + bm_bytes);
  A.arrive = w->counters + SLOT_SEG;
  A.depart = w->counters + SLOT_SEG + 1;
  auto kfn = k_seg<TI, TO, OP, MODE, FAST, IPT, STG>;
  static std::atomic<int> resident{0};  // CTAs per SM, per instantiation (set once, any host thread)
  if (!resident) {
    GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int r = 0;
    GBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kfn, SEG_BLOCK, dyn));
    if (r < 1) return GBK_ERR_UNSUPPORTED;
    resident = r;
  }
  const int per_sm = cps > 0 && cps < resident ? cps : resident.load();
  const int64_t grid = std::min<int64_t>(ntiles, (int64_t)per_sm * sm_count());
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(SEG_BLOCK);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = w->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GBK_CUDA_TRY(cudaLaunchKernelEx(&cfg, kfn, x, y, n, A, S));
  note_launch();
  return GBK_OK;
}

// items_per_thread (16-byte vectors per thread per tile): 7, 5 or 3.  Scans
// default to 5 with three staging stages (two CTAs per SM still fit), so
// the compute warps have a second tile ahead while they wait for a carry;
// reduces of unaligned input keep 7 with three stages.  Measured on GB300,
// inclusive scans of 2^28 int32 in 10,000 lognormal segments: int32 ->
// int64 0.638 ms with 5 x 3 stages against 0.896 (7 x 2) and 0.866 (3 x 2);
// int32 -> int32 0.472 against 0.476 (7 x 2) and 0.739 (3 x 2).
template <class TI, class TO, int OP, int MODE>
int launch_seg(const TI* x, TO* y, int64_t n, const int64_t* offsets, int64_t nseg, Workspace* w,
               const gbk_tuning_t* t) {
  constexpr int DEF = MODE != M_REDUCE ? 5 : 7;
  const int want = t && t->items_per_thread > 0 ? t->items_per_thread : DEF;
  const int cps = t ? t->ctas_per_sm : 0;
  const bool fast = (uintptr_t)x % 16 == 0 && (MODE == M_REDUCE || (uintptr_t)y % 16 == 0);
  // Reduce has no out tile: a 3-deep ring keeps more of its input in flight
  // (still two CTAs per SM; four stages of 7-vector tiles would allow one).
  constexpr int STG = MODE == M_REDUCE ? 3 : 2;
  if (!fast) return launch_k_seg<TI, TO, OP, MODE, false, 7, STG>(x, y, n, offsets, nseg, w, cps);
  if (want <= 4) return launch_k_seg<TI, TO, OP, MODE, true, 3, STG>(x, y, n, offsets, nseg, w, cps);
  // 5 vectors per thread: three stages still fit two CTAs per SM
  if (want == 5 && MODE != M_REDUCE) return launch_k_seg<TI, TO, OP, MODE, true, 5, 3>(x, y, n, offsets, nseg, w, cps);
  return launch_k_seg<TI, TO, OP, MODE, true, 7, STG>(x, y, n, offsets, nseg, w, cps);
}

// Variant 0 (default): the contiguous-share kernel for 16-byte aligned input
// of at least one chunk; variant 1 (or other input): the tile pipeline.
template <class T>
int seg_reduce_t(int op, const void* x, const int64_t* offs, int64_t nseg, int64_t n, void* out, Workspace* w,
                 const gbk_tuning_t* t) {
  const bool shares = (uintptr_t)x % 16 == 0 && n >= (int64_t)SR_CV * (16 / (int64_t)sizeof(T)) &&
                      !(t && t->variant == 1);
  if (shares) {
    switch (op) {
      case GBK_SUM: return launch_segred<RSum<T>, T>((const T*)x, (T*)out, n, offs, nseg, w);
      case GBK_MIN: return launch_segred<RMin<T>, T>((const T*)x, (T*)out, n, offs, nseg, w);
      case GBK_MAX: return launch_segred<RMax<T>, T>((const T*)x, (T*)out, n, offs, nseg, w);
    }
    return GBK_ERR_UNSUPPORTED;
  }
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

