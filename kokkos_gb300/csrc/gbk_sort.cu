// Stable LSD radix sort, sort_by_key and BinSort.  Replaces Kokkos::sort /
// Experimental::sort_by_key on a device space
// (algorithms/src/sorting/Kokkos_SortPublicAPI.hpp:31-196,
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
// The array is cut into G chunks of whole tiles (G <= 2 x the SM count, two
// scatter CTAs per SM); chunk c belongs to CTA c of every scatter launch.
// 1. k_digit_hist: one read of the keys counts every 8-bit digit position,
//    for the whole array and per chunk.  k_sort_plan (one CTA) turns the
//    whole-array counts into each pass's digit starts and a plan on the
//    device: which passes have a digit that is not the same for every key,
//    which buffer each of them reads, and how each ranks.  Every pass kernel
//    reads the plan and returns at once for a constant digit, and a final
//    copy runs only when the data ended in the temporary buffers, so a sort
//    is a fixed sequence of launches with no host round trip (it can be
//    captured into a CUDA graph).
// 2. Per remaining 8-bit pass:
//    k_chunk_count (all passes but the first, whose counts come from step 1):
//      per-chunk counts of the pass's digit; keys stream through a
//      shared-memory ring filled by bulk copies.
//    k_chunk_scatter: one persistent CTA per chunk.  Its running offset for
//      digit d starts at d's global start plus d's counts in all earlier
//      chunks.  It walks its tiles in order with bulk copies running
//      STAGES tiles ahead, ranks each tile with warp ballots (stable: slot
//      order = input order), reorders the tile by digit in place in shared
//      memory and writes the runs of equal digits at the running offsets.
//    No CTA waits for another: a pass costs one extra read of the keys (the
//    counts) instead of an inter-tile look-back, whose walk grows with the
//    number of tiles in flight.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gbk_internal.cuh"

namespace gbk {
namespace {

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

template <int VB> struct ValT;
template <> struct ValT<0> { using T = char; };
template <> struct ValT<4> { using T = uint32_t; };
template <> struct ValT<8> { using T = uint64_t; };

// Keys [lo, hi) of part `part` of chunk c when each chunk of `chunk_keys`
// keys is split into `sub` parts starting on 4-key (16-byte) boundaries.
__device__ __forceinline__ void chunk_part(int64_t n, int64_t chunk_keys, int c, int part, int sub, int64_t* lo,
                                           int64_t* hi) {
  const int64_t a = (int64_t)c * chunk_keys;
  const int64_t b = a + chunk_keys < n ? a + chunk_keys : n;
  const int64_t per = ((b - a + sub - 1) / sub + 3) & ~(int64_t)3;
  const int64_t l = a + part * per;
  *lo = l < b ? l : b;
  *hi = *lo + per < b ? *lo + per : b;
}

// Lanes of the warp holding the same 8-bit digit d, within the lanes where
// `ok` holds (ALL: every lane): eight ballots, one per digit bit.  No shared
// memory, and the cost does not depend on how the digits repeat.
template <bool ALL>
__device__ __forceinline__ unsigned digit_peers(unsigned d, bool ok) {
  unsigned m = ALL ? 0xffffffffu : __ballot_sync(0xffffffffu, ok);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const bool bit = (d >> b) & 1u;
    const unsigned v = __ballot_sync(0xffffffffu, bit);
    m &= bit ? v : ~v;
  }
  return m;
}

// Stable rank of one row of 32 keys (one per lane) within a warp: the
// warp's count of digit d before this row (cnt[d], per warp, shared) plus
// the lanes below holding d.  The lowest lane of each digit group advances
// cnt[d].
template <bool ALL>
__device__ __forceinline__ unsigned rank_peers(unsigned short* cnt, unsigned d, bool ok, int lane, unsigned m) {
  const int leader = __ffs(m) - 1;
  unsigned b = 0;
  if (ok && lane == leader) {
    b = cnt[d];
    cnt[d] = (unsigned short)(b + (unsigned)__popc(m));
  }
  b = __shfl_sync(0xffffffffu, b, leader < 0 ? lane : leader);
  __syncwarp();
  return b + (unsigned)__popc(m & ((1u << lane) - 1u));
}
template <bool ALL>
__device__ __forceinline__ unsigned rank_row(unsigned short* cnt, unsigned d, bool ok, int lane) {
  return rank_peers<ALL>(cnt, d, ok, lane, digit_peers<ALL>(d, ok));
}
// The same with the peer set from one match.any over the digit.
template <bool ALL>
__device__ __forceinline__ unsigned rank_row_match(unsigned short* cnt, unsigned d, bool ok, int lane) {
  unsigned m = __match_any_sync(0xffffffffu, d);
  if (!ALL) m &= __ballot_sync(0xffffffffu, ok);
  return rank_peers<ALL>(cnt, d, ok, lane, m);
}

// The same rank from a per-warp array of 256 lane masks in shared memory
// (zero between rows): every lane ORs its bit into its digit's mask, reads
// the mask back as its peer set, and the group's lowest lane advances the
// count and clears the mask.  About a third of the instructions of the
// eight ballots; lanes sharing a digit serialise on its word, so the plan
// picks it only for passes where no digit value holds a large share of the
// keys.
template <bool ALL>
__device__ __forceinline__ unsigned rank_row_or(unsigned short* cnt, unsigned* masks, unsigned d, bool ok,
                                                int lane) {
  const unsigned bit = 1u << lane;
  if (ALL || ok) atomicOr(&masks[d], bit);
  __syncwarp();
  const unsigned m = (ALL || ok) ? masks[d] : 0u;
  __syncwarp();  // every lane has read its mask before the leader clears it
  const int leader = __ffs(m) - 1;
  unsigned b = 0;
  if ((ALL || ok) && lane == leader) {
    b = cnt[d];
    cnt[d] = (unsigned short)(b + (unsigned)__popc(m));
    masks[d] = 0u;
  }
  b = __shfl_sync(0xffffffffu, b, leader < 0 ? lane : leader);
  __syncwarp();
  return b + (unsigned)__popc(m & (bit - 1u));
}

// After a wait that gave up: wait (bounded) for the bulk copies still in
// flight into stages j in [from, to), so none lands after the CTA exits.
__device__ __forceinline__ void drain_stages(unsigned long long* bars, int stages, int64_t from, int64_t to,
                                             int64_t limit) {
  for (int64_t j = from; j < to; ++j) mbar_wait(&bars[j % stages], (unsigned)(j / stages) & 1u, limit);
}

// The sort's plan, built on the device from the digit histogram.
struct SortPlan {
  int active[8];   // the pass's digit differs between keys
  int src[8];      // 0: the pass reads the caller's buffers, 1: the temporaries
  int first[8];    // the first active pass (its per-chunk counts come from k_digit_hist)
  int rank[8];     // ranking of the pass's scatter: 0 ballots, 1 lane masks, 2 match.any (see k_sort_plan)
  int final_tmp;   // after the last active pass the data is in the temporaries
  int pad[3];
};

// ---- 1. all digit positions, whole array and per chunk ----------------------
// hist[p*256 + d] (u64) and ccounts[(p*nchunks + c)*256 + d] (u32), both
// zeroed by the caller.  Grid = nchunks * sub.
template <int DT, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_digit_hist(const typename Radix<DT>::K* __restrict__ keys, int64_t n, int64_t chunk_keys, int sub,
                 int nchunks, unsigned long long* __restrict__ hist, unsigned* __restrict__ ccounts) {
  using K = typename Radix<DT>::K;
  constexpr int KB = sizeof(K);
  constexpr int U = 4;  // keys per thread per step (loads in flight)
  __shared__ unsigned sh[KB * 256];
  for (int i = threadIdx.x; i < KB * 256; i += BLOCK) sh[i] = 0u;
  __syncthreads();
  const int c = blockIdx.x / sub;
  int64_t lo, hi;
  chunk_part(n, chunk_keys, c, blockIdx.x % sub, sub, &lo, &hi);
  for (int64_t base = lo; base < hi; base += (int64_t)BLOCK * U) {
    K img[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + u * BLOCK + threadIdx.x;
      ok[u] = i < hi;
      img[u] = ok[u] ? Radix<DT>::img(keys[i]) : K(0);
    }
    // Increments without a result: lanes of a warp on one counter are
    // combined by the shared-memory atomic unit, so skewed keys stay fast.
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (ok[u]) {
#pragma unroll
        for (int p = 0; p < KB; ++p) atomicAdd(sh + p * 256 + ((unsigned)(img[u] >> (8 * p)) & 255u), 1u);
      }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < KB * 256; i += BLOCK) {
    const unsigned v = sh[i];
    if (v) {
      atomicAdd(hist + i, (unsigned long long)v);
      atomicAdd(ccounts + ((int64_t)(i >> 8) * nchunks + c) * 256 + (i & 255), v);
    }
  }
}

// ---- 2a. per-chunk counts of one digit ----------------------------------------
constexpr int CNT_BLOCK = 256;
constexpr int CNT_STAGE_BYTES = 16384;
constexpr int CNT_STAGES = 4;
constexpr int CNT_SUB = 3;  // CTAs per chunk

// counts[c*256 + d] (u32, zeroed by the caller).  Grid = nchunks * CNT_SUB.
// TMA: keys 16-byte aligned, streamed through the ring; otherwise plain loads.
// The plan picks the buffer the pass reads (the caller's or the temporary);
// the first active pass and passes with a constant digit count nothing.
template <int DT, bool TMA>
__global__ void __launch_bounds__(CNT_BLOCK)
    k_chunk_count(const typename Radix<DT>::K* __restrict__ keys_user, const typename Radix<DT>::K* __restrict__ keys_tmp,
                  const SortPlan* __restrict__ plan, int pass, int64_t n, int64_t chunk_keys, int shift,
                  unsigned* __restrict__ counts, int* err, int64_t wait_limit) {
  using K = typename Radix<DT>::K;
  if (!plan->active[pass] || plan->first[pass]) return;
  const K* __restrict__ keys = plan->src[pass] ? keys_tmp : keys_user;
  constexpr int E = CNT_STAGE_BYTES / (int)sizeof(K);  // keys per stage
  constexpr int WARPS = CNT_BLOCK / 32;
  extern __shared__ __align__(128) unsigned char ring[];
  __shared__ __align__(8) unsigned long long s_bar[CNT_STAGES];
  __shared__ unsigned s_h[WARPS][256];
  const int warp = threadIdx.x >> 5;
  const int c = blockIdx.x / CNT_SUB;
  int64_t lo, hi;
  chunk_part(n, chunk_keys, c, blockIdx.x % CNT_SUB, CNT_SUB, &lo, &hi);
  const int64_t nst = (hi - lo + E - 1) / E;
  for (int i = threadIdx.x; i < WARPS * 256; i += CNT_BLOCK) (&s_h[0][0])[i] = 0u;
  // Thread 0 only: start the copy of the whole 4-key groups of stage j.
  auto fill = [&](int64_t j) {
    if (j >= nst) return;
    const int64_t s0 = lo + j * E;
    const int64_t cnt = hi - s0 < E ? hi - s0 : E;
    const unsigned bytes = (unsigned)((cnt & ~(int64_t)3) * (int64_t)sizeof(K));
    unsigned long long* bar = &s_bar[j % CNT_STAGES];
    mbar_arrive_expect_tx(bar, bytes);
    if (bytes) bulk_g2s(ring + (size_t)(j % CNT_STAGES) * CNT_STAGE_BYTES, keys + s0, bytes, bar);
  };
  if (TMA && threadIdx.x == 0) {
    for (int s = 0; s < CNT_STAGES; ++s) mbar_init(&s_bar[s], 1);
    fence_mbar_init();
    for (int s = 0; s < CNT_STAGES; ++s) fill(s);
  }
  __syncthreads();
  int64_t failed = -1;
  for (int64_t j = 0; j < nst; ++j) {
    const int64_t s0 = lo + j * E;
    const int cnt = (int)(hi - s0 < E ? hi - s0 : E);
    const int cv = TMA ? (cnt & ~3) : 0;
    const K* sk = reinterpret_cast<const K*>(ring + (size_t)(j % CNT_STAGES) * CNT_STAGE_BYTES);
    bool bad = false;
    if (TMA) bad = !mbar_wait(&s_bar[j % CNT_STAGES], (unsigned)(j / CNT_STAGES) & 1u, wait_limit);
    if (cv == E) {
#pragma unroll 4
      for (int idx = threadIdx.x; idx < E; idx += CNT_BLOCK)
        atomicAdd(&s_h[warp][(unsigned)(Radix<DT>::img(sk[idx]) >> shift) & 255u], 1u);
    } else {
      for (int idx = threadIdx.x; idx < cnt; idx += CNT_BLOCK) {
        const K key = idx < cv ? sk[idx] : keys[s0 + idx];
        atomicAdd(&s_h[warp][(unsigned)(Radix<DT>::img(key) >> shift) & 255u], 1u);
      }
    }
    if (TMA) {
      if (__syncthreads_or(bad)) {  // stage j fully read, or a copy never arrived
        failed = j;
        break;
      }
      if (threadIdx.x == 0) fill(j + CNT_STAGES);
    }
  }
  if (failed >= 0) {
    if (threadIdx.x == 0) {
      drain_stages(s_bar, CNT_STAGES, failed, failed + CNT_STAGES < nst ? failed + CNT_STAGES : nst, wait_limit);
      atomicOr(err, GBK_EBIT_TIMEOUT);
    }
    return;
  }
  __syncthreads();
  {
    const int d = threadIdx.x;  // CNT_BLOCK == 256: one digit per thread
    unsigned v = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) v += s_h[w][d];
    if (v) atomicAdd(counts + (int64_t)c * 256 + d, v);
  }
}

// ---- 2b. persistent in-order scatter of each chunk ------------------------------
// Launch shape: threads per CTA, keys per thread per tile (for 8- to 12-byte
// keys+values; doubled for 4-byte keys alone) and CTAs per SM.  Threads
// 0..255 also own one digit each.  The ring takes what shared memory is left
// per CTA, at most 6 stages.  Measured on 2^27 u64 keys + u32 values (8
// passes), uniform / low-entropy keys: 512 x 8, 1 CTA/SM: 10.3 / 6.8 ms;
// 512 x 4, 2/SM: 12.5 / 7.0; 256 x 8, 3/SM: 13.2 / 6.1; 256 x 8, 2/SM:
// 12.2 / 6.4; 1024 x 4, 1/SM: 11.2 / 7.4; 256 x 16, 2/SM: 9.8 / 6.0 (kept:
// a 4096-key tile, and two CTAs per SM whose rank, reorder and store phases
// overlap).
template <int VAR> struct ScVar;
template <> struct ScVar<0> { static constexpr int BLOCK = 256, KPT = 16, MINB = 2; };

template <int KB, int VB, int VAR> struct ScShape {
  static constexpr int BLOCK = ScVar<VAR>::BLOCK, MINB = ScVar<VAR>::MINB;
  static constexpr int WARPS = BLOCK / 32;
  static constexpr int STATIC_BYTES = WARPS * 256 * 6 + 256 * 8 + 256;  // counters, masks/offsets, bases, misc
  static constexpr int BUDGET = 233472 / MINB - 1024 - STATIC_BYTES;  // per CTA, 1 KiB reserved per CTA
  // keys per thread: doubled for 4-byte keys alone, halved when two stages
  // of the widest elements would not fit
  static constexpr int KPT0 = (KB + VB) <= 4 ? 2 * ScVar<VAR>::KPT : ScVar<VAR>::KPT;
  static constexpr int KPT = BUDGET / (BLOCK * KPT0 * (KB + VB)) >= 2 ? KPT0 : KPT0 / 2;
  static constexpr int TILE = BLOCK * KPT;
  static constexpr int KEY_BYTES = TILE * KB;
  static constexpr int STAGE_BYTES = TILE * (KB + VB);
  static constexpr int STAGES = BUDGET / STAGE_BYTES > 6 ? 6 : BUDGET / STAGE_BYTES;
  static_assert(STAGES >= 2, "at least one tile in flight beside the one being sorted");
  static_assert(KPT * 32 <= 65535 && TILE <= 65535, "16-bit tile offsets");
};

// Passes whose rows of 32 keys are expected to hold at most this many
// distinct digits rank with match.any.  Measured on 2^27 u64 keys + u32
// values: keys with 2 distinct digits per pass (8 random bits) sort in
// 4.24 ms with match.any, 5.53 with ballots and 6.03 with lane masks; uniform
// keys (30 distinct digits per row) in 11.47 / 9.79 / 9.68 ms; on 2^26 keys
// with 16-40 random bits (passes of 2 to 25 distinct digits per row) the
// crossing between match.any and the masks lies near 15.
constexpr float kMatchDistinct = 16.0f;

// One CTA of 256 threads (one per digit): digit starts of every pass and the
// plan.  A histogram whose counts do not add up to n (keys changed under the
// sort) marks every pass inactive and raises the bad-state status.
template <int KB>
__global__ void __launch_bounds__(256)
    k_sort_plan(const unsigned long long* __restrict__ hist, int64_t n, int64_t* __restrict__ off, SortPlan* plan,
                int* err) {
  __shared__ unsigned long long s_w[8];
  __shared__ int s_const[KB], s_hot[KB];
  __shared__ unsigned long long s_tot[KB];
  __shared__ float s_e[8], s_dist[KB];
  const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
  for (int p = 0; p < KB; ++p) {
    const unsigned long long v = hist[p * 256 + d];
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    unsigned long long pre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      if (w < warp) pre += s_w[w];
      tot += s_w[w];
    }
    off[p * 256 + d] = (int64_t)(pre + inc - v);
    // expected number of distinct digits among 32 keys: sum over d of
    // 1 - (1 - share_d)^32
    float q = 1.0f - (float)v / (float)(n > 0 ? n : 1);
#pragma unroll
    for (int k = 0; k < 5; ++k) q *= q;
    float e = 1.0f - q;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (lane == 0) s_e[warp] = e;
    const int c = __syncthreads_or((int64_t)v == n);
    const int hot = __syncthreads_or((int64_t)v * 8 > n);
    if (d == 0) {
      s_const[p] = c;
      s_hot[p] = hot;
      s_tot[p] = tot;
      float de = 0.0f;
      for (int w = 0; w < 8; ++w) de += s_e[w];
      s_dist[p] = de;
    }
    __syncthreads();
  }
  if (d == 0) {
    bool ok = true;
    for (int p = 0; p < KB; ++p) ok = ok && (int64_t)s_tot[p] == n;
    if (!ok) atomicOr(err, GBK_EBIT_BAD_STATE);
    int done = 0;
    for (int p = 0; p < 8; ++p) {
      const int act = ok && p < KB && !s_const[p];
      plan->active[p] = act;
      plan->src[p] = done & 1;
      plan->first[p] = act && done == 0;
      // A row of 32 keys with few distinct digits is ranked fastest by
      // match.any (its cost grows with the distinct values); with many, by
      // the lane masks, unless one digit holds over 1/8 of the keys (its
      // word then serialises the masks): the eight ballots.
      plan->rank[p] = p >= KB ? 0 : s_dist[p] <= kMatchDistinct ? 2 : !s_hot[p] ? 1 : 0;
      done += act;
    }
    plan->final_tmp = done & 1;
  }
}

struct ScatterArgs {
  const int64_t* digit_start;  // [256] global start of each digit in this pass
  const unsigned* counts;      // [nchunks][256] per-chunk digit counts (the non-first passes)
  const unsigned* first_counts;  // [nchunks][256] this pass's counts from k_digit_hist (the first active pass)
  const SortPlan* plan;
  int* err;
  int64_t tiles_per_chunk;
  int64_t wait_limit;
  int shift;
  int pass;
  int rank_mode;  // 0: the plan's choice, 1: lane masks, 2: ballots
};

// Grid = nchunks, MINB CTAs per SM.  TMA: kin/vin 16-byte aligned, tiles
// streamed through the ring; otherwise tiles are loaded with plain loads and
// stage 0 only holds the reorder.
// ku / vu: the caller's keys and values, kt / vt: the temporaries; the plan
// says which pair the pass reads (it writes the other).
template <int DT, int VB, bool TMA, int VAR>
__global__ void __launch_bounds__(ScVar<VAR>::BLOCK, ScVar<VAR>::MINB)
    k_chunk_scatter(typename Radix<DT>::K* ku, typename Radix<DT>::K* kt, typename ValT<VB>::T* vu,
                    typename ValT<VB>::T* vt, int64_t n, ScatterArgs A) {
  using K = typename Radix<DT>::K;
  using V = typename ValT<VB>::T;
  const SortPlan* plan = A.plan;
  if (!plan->active[A.pass]) return;
  const bool from_tmp = plan->src[A.pass] != 0;
  const K* __restrict__ kin = from_tmp ? kt : ku;
  K* __restrict__ kout = from_tmp ? ku : kt;
  const V* __restrict__ vin = from_tmp ? vt : vu;
  V* __restrict__ vout = from_tmp ? vu : vt;
  const unsigned* counts = plan->first[A.pass] ? A.first_counts : A.counts;
  // 1: lane masks, 2: match.any, 0: ballots
  const int rank_by = A.rank_mode == 1 ? 1 : A.rank_mode == 2 ? 0 : A.rank_mode == 3 ? 2 : plan->rank[A.pass];
  using Sh = ScShape<(int)sizeof(K), VB, VAR>;
  constexpr int BLOCK = Sh::BLOCK, KPT = Sh::KPT, TILE = Sh::TILE, STAGES = Sh::STAGES, WARPS = Sh::WARPS;
  extern __shared__ __align__(128) unsigned char ring[];
  __shared__ __align__(8) unsigned long long s_bar[STAGES];
  __shared__ unsigned short s_cnt[WARPS][256];  // per-warp digit counts of the tile (rank_row)
  // per-warp lane masks of rank_row_or while a tile is ranked; afterwards the
  // first half holds s_off: the tile-local slot of each warp's first key of
  // each digit
  __shared__ __align__(16) unsigned s_rk[WARPS * 256];
  unsigned short(*s_off)[256] = reinterpret_cast<unsigned short(*)[256]>(s_rk);
  __shared__ long long s_gb[256];               // global position of tile slot 0 of each digit
  __shared__ unsigned s_wsum[8];
  __shared__ int s_oob;  // a digit range of the current tile falls outside [0, n)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ntiles = (n + TILE - 1) / TILE;
  const int64_t t0 = (int64_t)blockIdx.x * A.tiles_per_chunk;
  const int64_t nt = (t0 + A.tiles_per_chunk < ntiles ? t0 + A.tiles_per_chunk : ntiles) - t0;
  // Thread 0 only: start the copies of the whole 4-key groups of tile j.
  auto fill = [&](int64_t j) {
    if (j >= nt) return;
    const int64_t base = (t0 + j) * TILE;
    const int64_t cnt = n - base < TILE ? n - base : TILE;
    const int64_t cv = cnt & ~(int64_t)3;
    unsigned char* st = ring + (size_t)(j % STAGES) * Sh::STAGE_BYTES;
    unsigned long long* bar = &s_bar[j % STAGES];
    mbar_arrive_expect_tx(bar, (unsigned)(cv * (int64_t)(sizeof(K) + VB)));
    if (cv) {
      bulk_g2s(st, kin + base, (unsigned)(cv * (int64_t)sizeof(K)), bar);
      if (VB) bulk_g2s(st + Sh::KEY_BYTES, vin + base, (unsigned)(cv * VB), bar);
    }
  };
  if (TMA && threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&s_bar[s], 1);
    fence_mbar_init();
    for (int s = 0; s < STAGES; ++s) fill(s);
  }
  // Running global offset of digit threadIdx.x: its start plus its counts in
  // the earlier chunks (loads batched 16 at a time).
  long long run = 0;
  if (threadIdx.x < 256) {
    long long r = A.digit_start[threadIdx.x];
    const unsigned* cp = counts + threadIdx.x;
    const int64_t nc = blockIdx.x;
    int64_t q = 0;
    for (; q + 16 <= nc; q += 16) {
      unsigned v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) v[u] = cp[(q + u) * 256];
#pragma unroll
      for (int u = 0; u < 16; ++u) r += v[u];
    }
    for (; q < nc; ++q) r += cp[q * 256];
    run = r;
  }
  for (int i = threadIdx.x; i < WARPS * 256; i += BLOCK) {
    (&s_cnt[0][0])[i] = 0;
    s_rk[i] = 0u;
  }
  if (threadIdx.x == 0) s_oob = 0;
  __syncthreads();
  const int wb = warp * 32 * KPT;  // the warp's first slot in the tile
  int64_t failed = -1;
  bool out_of_range = false;
  for (int64_t j = 0; j < nt; ++j) {
    const int64_t base = (t0 + j) * TILE;
    const int cnt = (int)(n - base < TILE ? n - base : TILE);
    const int cv = TMA ? (cnt & ~3) : 0;
    unsigned char* st = ring + (size_t)(TMA ? j % STAGES : 0) * Sh::STAGE_BYTES;
    K* s_keys = reinterpret_cast<K*>(st);
    V* s_vals = reinterpret_cast<V*>(st + Sh::KEY_BYTES);
    bool bad = false;
    if (TMA) bad = !mbar_wait(&s_bar[j % STAGES], (unsigned)(j / STAGES) & 1u, A.wait_limit);
    // ---- load (warp-contiguous slots) and rank within the warp -------------
    const bool full = cv == TILE;  // every tile but the array's last
    K key[KPT];
    V val[KPT];
    unsigned dig[KPT];
    unsigned rk[KPT];
    if (full) {  // every key of the tile present: no bounds, no validity ballot
#pragma unroll
      for (int k = 0; k < KPT; ++k) {
        const int slot = wb + k * 32 + lane;
        key[k] = s_keys[slot];
        if (VB) val[k] = s_vals[slot];
        dig[k] = (unsigned)(Radix<DT>::img(key[k]) >> A.shift) & 255u;
      }
      if (rank_by == 1) {
#pragma unroll
        for (int k = 0; k < KPT; ++k) rk[k] = rank_row_or<true>(s_cnt[warp], s_rk + warp * 256, dig[k], true, lane);
      } else if (rank_by == 2) {
#pragma unroll
        for (int k = 0; k < KPT; ++k) rk[k] = rank_row_match<true>(s_cnt[warp], dig[k], true, lane);
      } else {
#pragma unroll
        for (int k = 0; k < KPT; ++k) rk[k] = rank_row<true>(s_cnt[warp], dig[k], true, lane);
      }
    } else {
#pragma unroll
      for (int k = 0; k < KPT; ++k) {
        const int slot = wb + k * 32 + lane;
        const bool ok = slot < cnt;
        key[k] = slot < cv ? s_keys[slot] : (ok ? kin[base + slot] : K(0));
        if (VB) val[k] = slot < cv ? s_vals[slot] : (ok ? vin[base + slot] : V(0));
        dig[k] = (unsigned)(Radix<DT>::img(key[k]) >> A.shift) & 255u;
      }
      if (rank_by == 1) {
#pragma unroll
        for (int k = 0; k < KPT; ++k)
          rk[k] = rank_row_or<false>(s_cnt[warp], s_rk + warp * 256, dig[k], wb + k * 32 + lane < cnt, lane);
      } else if (rank_by == 2) {
#pragma unroll
        for (int k = 0; k < KPT; ++k) rk[k] = rank_row_match<false>(s_cnt[warp], dig[k], wb + k * 32 + lane < cnt, lane);
      } else {
#pragma unroll
        for (int k = 0; k < KPT; ++k) rk[k] = rank_row<false>(s_cnt[warp], dig[k], wb + k * 32 + lane < cnt, lane);
      }
    }
    if (__syncthreads_or(bad)) {  // counts complete and every key read, or a copy never arrived
      failed = j;
      break;
    }
    // ---- digit totals, tile-local starts, global positions ------------------
    if (threadIdx.x < 256) {
      const unsigned d = threadIdx.x;
      unsigned tot = 0;
      unsigned short wpre[WARPS];  // exclusive prefix over warps
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const unsigned c = s_cnt[w][d];
        s_cnt[w][d] = 0;  // ready for the next tile
        wpre[w] = (unsigned short)tot;
        tot += c;
      }
      unsigned inc = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      if (lane == 31) s_wsum[warp] = inc;
      bar_sync(1, 256);
      unsigned pre = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w)
        if (w < warp) pre += s_wsum[w];
      const unsigned start = pre + inc - tot;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) s_off[w][d] = (unsigned short)(start + wpre[w]);
      s_gb[d] = run - (long long)start;
      // this tile writes [run, run + tot) for digit d: inside [0, n) unless
      // the counts and the keys disagree (keys changed under the sort)
      if (tot && (run < 0 || run + (long long)tot > n)) s_oob = 1;
      run += tot;
    }
    __syncthreads();
    // ---- reorder the tile by digit, in place ---------------------------------
    if (full) {
#pragma unroll
      for (int k = 0; k < KPT; ++k) {
        const unsigned r = (unsigned)s_off[warp][dig[k]] + rk[k];
        s_keys[r] = key[k];
        if (VB) s_vals[r] = val[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < KPT; ++k) {
        if (wb + k * 32 + lane < cnt) {
          const unsigned r = (unsigned)s_off[warp][dig[k]] + rk[k];
          s_keys[r] = key[k];
          if (VB) s_vals[r] = val[k];
        }
      }
    }
    __syncthreads();
    if (rank_by == 1) {  // s_off is dead: clear the lane masks for the next tile (visible after the loop's barrier)
      uint4* z = reinterpret_cast<uint4*>(s_rk);
      for (int i = threadIdx.x; i < WARPS * 256 / 4; i += BLOCK) z[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    // ---- write the runs of equal digits ---------------------------------------
    auto emit = [&](int i) {
      const K kk = s_keys[i];
      const long long pos = s_gb[(unsigned)(Radix<DT>::img(kk) >> A.shift) & 255u] + i;
      kout[pos] = kk;
      if (VB) vout[pos] = s_vals[i];
    };
    if (s_oob) {
      out_of_range = true;  // write nothing of this tile
    } else if (full) {
#pragma unroll
      for (int q = 0; q < KPT; ++q) emit(q * BLOCK + threadIdx.x);
    } else {
      for (int i = threadIdx.x; i < cnt; i += BLOCK) emit(i);
    }
    if (TMA) fence_proxy_async_smem();  // generic writes of the stage before the next bulk copy into it
    __syncthreads();
    if (TMA && threadIdx.x == 0) fill(j + STAGES);
  }
  if (failed >= 0 && threadIdx.x == 0) {
    drain_stages(s_bar, STAGES, failed, failed + STAGES < nt ? failed + STAGES : nt, A.wait_limit);
    atomicOr(A.err, GBK_EBIT_TIMEOUT);
  }
  if (out_of_range) atomicOr(A.err, GBK_EBIT_BAD_STATE);
}

// ---- host driver ------------------------------------------------------------
constexpr int HIST_BLOCK = 512;
constexpr int HIST_SUB = 4;  // CTAs per chunk for the all-digit histogram

template <int DT, int VB, bool TMA, int VAR>
int launch_pass(typename Radix<DT>::K* ku, typename Radix<DT>::K* kt, typename ValT<VB>::T* vu,
                typename ValT<VB>::T* vt, int64_t n, int64_t nchunks, int64_t chunk_keys, const ScatterArgs& A,
                Workspace* w) {
  using K = typename Radix<DT>::K;
  using Sh = ScShape<(int)sizeof(K), VB, VAR>;
  cudaStream_t s = w->stream;
  auto cfn = k_chunk_count<DT, TMA>;
  constexpr size_t cdyn = TMA ? (size_t)CNT_STAGES * CNT_STAGE_BYTES : 0;
  static std::atomic<bool> cset{false};
  if (!cset && cdyn) {
    GBK_CUDA_TRY(cudaFuncSetAttribute(cfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cdyn));
    cset = true;
  }
  GBK_CUDA_TRY(cudaMemsetAsync((void*)A.counts, 0, (size_t)nchunks * 256 * 4, s));
  cfn<<<(unsigned)(nchunks * CNT_SUB), CNT_BLOCK, cdyn, s>>>(ku, kt, A.plan, A.pass, n, chunk_keys, A.shift,
                                                             (unsigned*)A.counts, w->err, A.wait_limit);
  note_launch();
  GBK_CUDA_TRY(cudaGetLastError());
  auto sfn = k_chunk_scatter<DT, VB, TMA, VAR>;
  constexpr size_t sdyn = (size_t)(TMA ? Sh::STAGES : 1) * Sh::STAGE_BYTES;
  static std::atomic<bool> sset{false};
  if (!sset) {
    GBK_CUDA_TRY(cudaFuncSetAttribute(sfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sdyn));
    sset = true;
  }
  sfn<<<(unsigned)nchunks, Sh::BLOCK, sdyn, s>>>(ku, kt, vu, vt, n, A);
  note_launch();
  return cuda_status(cudaGetLastError());
}

// After the passes: when an odd number of passes ran, the sorted data is in
// the temporaries and goes back to the caller's buffers.
template <class K, class V>
__global__ void k_sort_copy_back(const SortPlan* __restrict__ plan, const K* __restrict__ kt, K* __restrict__ ku,
                                 const V* __restrict__ vt, V* __restrict__ vu, int64_t n) {
  if (!plan->final_tmp) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    ku[i] = kt[i];
    if (vu) vu[i] = vt[i];
  }
}

// Ranking of the scatter passes: GBK_SORT_RANK=masks, =ballot or =match in
// the environment forces one method for every pass; otherwise the plan
// chooses per pass from the digit histogram.
int sort_rank_mode() {
  static std::atomic<int> mode{-1};
  if (mode < 0) {
    const char* e = getenv("GBK_SORT_RANK");
    mode = (e && !strcmp(e, "masks")) ? 1 : (e && !strcmp(e, "ballot")) ? 2 : (e && !strcmp(e, "match")) ? 3 : 0;
  }
  return mode;
}

template <int DT, int VB, int VAR>
int sort_var(void* keys, void* vals, int64_t n, Workspace* w) {
  using K = typename Radix<DT>::K;
  using V = typename ValT<VB>::T;
  using Sh = ScShape<(int)sizeof(K), VB, VAR>;
  constexpr int KB = sizeof(K), TILE = Sh::TILE;
  static_assert(CNT_BLOCK == 256, "one digit per counting thread");
  cudaStream_t s = w->stream;
  if (n <= 1) return GBK_OK;
  if (n >= ((int64_t)1 << 38)) return GBK_ERR_INVALID_ARGUMENT;  // per-chunk counts are u32
  const int64_t ntiles = (n + TILE - 1) / TILE;
  int64_t nchunks = std::min<int64_t>((int64_t)sm_count() * Sh::MINB, ntiles);
  const int64_t tpc = (ntiles + nchunks - 1) / nchunks;
  nchunks = (ntiles + tpc - 1) / tpc;  // every chunk non-empty
  const int64_t chunk_keys = tpc * TILE;
  // scratch: histogram | digit starts | plan | per-chunk counts of every
  // digit | per-chunk counts of one digit | key temp | value temp
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t hb = (size_t)KB * 256 * 8, ob = (size_t)KB * 256 * 8, pb = 256;
  const size_t ccb = up((size_t)KB * nchunks * 256 * 4), c1b = up((size_t)nchunks * 256 * 4);
  const size_t kb = up((size_t)n * sizeof(K)), vb = VB ? up((size_t)n * VB) : 0;
  int st = GBK_OK;
  char* scr = ws_scratch(w, hb + ob + pb + ccb + c1b + kb + vb, &st);
  if (!scr) return st;
  unsigned long long* d_hist = (unsigned long long*)scr;
  int64_t* d_off = (int64_t*)(scr + hb);
  SortPlan* d_plan = (SortPlan*)(scr + hb + ob);
  unsigned* d_cc = (unsigned*)(scr + hb + ob + pb);
  unsigned* d_c1 = (unsigned*)(scr + hb + ob + pb + ccb);
  K* ktmp = (K*)(scr + hb + ob + pb + ccb + c1b);
  V* vtmp = VB ? (V*)(scr + hb + ob + pb + ccb + c1b + kb) : nullptr;

  GBK_CUDA_TRY(cudaMemsetAsync(d_hist, 0, hb, s));
  GBK_CUDA_TRY(cudaMemsetAsync(d_cc, 0, ccb, s));
  k_digit_hist<DT, HIST_BLOCK><<<(unsigned)(nchunks * HIST_SUB), HIST_BLOCK, 0, s>>>(
      (const K*)keys, n, chunk_keys, HIST_SUB, (int)nchunks, d_hist, d_cc);
  k_sort_plan<KB><<<1, 256, 0, s>>>(d_hist, n, d_off, d_plan, w->err);
  note_launch(2);
  GBK_CUDA_TRY(cudaGetLastError());
  // Bulk copies want 16-byte aligned sources: the caller's buffers may not be
  // (the temporaries are); unaligned callers get the plain-load kernels.
  const bool user_aligned = (uintptr_t)keys % 16 == 0 && (!VB || (uintptr_t)vals % 16 == 0);
  const int rank_mode = sort_rank_mode();
  for (int p = 0; p < KB; ++p) {
    ScatterArgs A;
    A.digit_start = d_off + p * 256;
    A.counts = d_c1;
    A.first_counts = d_cc + (size_t)p * nchunks * 256;
    A.plan = d_plan;
    A.err = w->err;
    A.tiles_per_chunk = tpc;
    A.wait_limit = wait_limit();
    A.shift = 8 * p;
    A.pass = p;
    A.rank_mode = rank_mode;
    st = user_aligned
             ? launch_pass<DT, VB, true, VAR>((K*)keys, ktmp, (V*)vals, vtmp, n, nchunks, chunk_keys, A, w)
             : launch_pass<DT, VB, false, VAR>((K*)keys, ktmp, (V*)vals, vtmp, n, nchunks, chunk_keys, A, w);
    if (st) return st;
  }
  const unsigned cg = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 16);
  k_sort_copy_back<K, V><<<cg, 256, 0, s>>>(d_plan, ktmp, (K*)keys, vtmp, (V*)vals, n);
  note_launch();
  return cuda_status(cudaGetLastError());
}

template <int DT, int VB>
int sort_impl(void* keys, void* vals, int64_t n, Workspace* w) {
  return sort_var<DT, VB, 0>(keys, vals, n, w);
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
