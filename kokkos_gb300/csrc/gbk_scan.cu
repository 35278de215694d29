// Single-pass prefix scan with decoupled look-back (Merrill & Garland,
// "Single-pass Parallel Prefix Scan with Decoupled Look-back", NVIDIA
// NVR-2016-002).  Replaces the two-launch, two-read CUDA ParallelScan of
// core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:390-700 (and the
// ParallelScanWithTotal variant :704-1053): one read of x, one write of y.
//
// Persistent, warp-specialised CTAs on a cooperative (co-resident) grid of G
// CTAs: CTA b owns tiles b, b + G, b + 2G, ... of 256 * IPT 16-byte input
// vectors.  Every tile a look-back waits on belongs to a running CTA that
// handles its tiles in order, so the waits cannot deadlock; and the static
// order keeps aggregates appearing in tile order (tickets taken ahead of use
// let a CTA hold tiles whose aggregates come microseconds late, and every
// look-back behind them waits).  Per CTA:
//   * eight compute warps run a software pipeline over the CTA's tiles: the
//     tile-sum pass of tile i+AHEAD (its aggregate is published at once),
//     then the output pass of tile i, whose exclusive prefix is ready by then;
//   * NLB look-back warps resolve the prefixes, tile slots round-robin.
// Input tiles arrive in a shared-memory ring by 1-D bulk copies
// (TMA engine, mbarrier completion); output tiles are staged in shared
// memory and leave as coalesced 16-byte streaming stores.  (A bulk store
// would need a generic-to-async proxy fence per tile, and that fence waited
// for the ring's copies in flight: microseconds per tile.)
//
// Tile status lives in the look-back descriptors of gbk_lookback.cuh (tagged
// 64-bit word pairs, no fences, epoch-tagged so nothing is cleared per
// launch).  Every wait is bounded by the library's wait limit and sets the
// timeout bit of the stream's error word instead of hanging.
#include <algorithm>
#include <type_traits>

#include "gbk_lookback.cuh"

namespace gbk {
namespace {

constexpr int SCAN_COMPUTE = 256;  // compute threads per CTA
// Look-back warps: the CTA's tile slots go round-robin to them, so up to NLB
// look-backs of one CTA are in flight at once (a look-back needs only its
// predecessors' aggregates, not their prefixes).
constexpr int NLB = 4;
constexpr int SCAN_BLOCK = SCAN_COMPUTE + 32 * NLB;
// Named barriers: tile info handed to look-back warp k (id BAR_INFO + k),
// prefix handed back (BAR_PREFIX + k), compute warps only.
constexpr int BAR_INFO = 1, BAR_PREFIX = 1 + NLB, BAR_COMPUTE = 1 + 2 * NLB;
constexpr int BAR_HANDOFF = SCAN_COMPUTE + 32;  // threads in one hand-off
static_assert(BAR_COMPUTE <= 15, "named barrier ids");

template <class T> __device__ __forceinline__ T shup(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }

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

// FAST: x and y are 16-byte aligned; tiles move by bulk copies through
// shared memory.  Otherwise every element is loaded and stored directly with
// the same thread-to-element mapping (the path for unaligned views).
//
// Thread-sequential chunks: compute thread i owns input vectors
// i*IPT .. i*IPT+IPT-1 of a tile.  IPT is odd, so the 8 lanes of a
// quarter-warp touch 8 different bank groups at every step and shared-memory
// accesses need no swizzle.  A thread scans its IPT * VEC elements serially:
// one warp scan per thread and about two additions per element (the FP64
// pipe, not HBM, bounds the f64 scans).
//
// Pipeline: the tile-sum pass runs AHEAD tiles ahead of the output pass, so
// a look-back has AHEAD iterations to finish; STAGES >= AHEAD + 1 input
// stages (one more lets the next copy land a full iteration early).  The
// out tile goes out in ROUNDS rounds (1, or 2 for widening scans: half the
// threads each, and an out tile of one input tile's bytes).
template <class TI, class TO, bool INCL, bool FAST, int IPT, int STAGES, int AHEAD, int ROUNDS>
__global__ void __launch_bounds__(SCAN_BLOCK, 2)
    k_scan(const TI* __restrict__ x, TO* __restrict__ y, int64_t n, TO init, LbState S, TO* total) {
  constexpr int VEC = 16 / sizeof(TI);
  constexpr int WARPS = SCAN_COMPUTE / 32;
  constexpr int OVN = (int)(VEC * sizeof(TO) / 16);  // output vectors per input vector: 1 or 2
  constexpr int OV = 16 / sizeof(TO);                 // elements per output vector
  constexpr int64_t TILE = (int64_t)SCAN_COMPUTE * IPT * VEC;
  constexpr unsigned IN_BYTES = (unsigned)SCAN_COMPUTE * IPT * 16;
  constexpr int RT = SCAN_COMPUTE / ROUNDS;  // threads per output round
  constexpr int64_t RTILE = TILE / ROUNDS;    // elements per output round
  static_assert(IPT % 2 == 1, "an odd vector count per thread keeps shared-memory accesses conflict-free");
  static_assert(OVN == 1 || OVN == 2, "output at most twice the input width");
  static_assert(AHEAD >= 1 && STAGES >= AHEAD + 1 && AHEAD < NLB, "pipeline depth");
  static_assert(ROUNDS == 1 || ROUNDS == OVN, "output rounds");
  // FAST: STAGES input stages, then the out tile (IN_BYTES * OVN / ROUNDS)
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ __align__(8) unsigned long long s_bar[STAGES];
  __shared__ int64_t s_info_tile[NLB];  // tile handed to look-back warp k
  __shared__ TO s_info_agg[NLB];
  __shared__ TO s_excl[NLB];            // its exclusive prefix, handed back
  __shared__ TO s_warp[2][WARPS];
  __shared__ int s_bad;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nin = FAST ? n / VEC * VEC : 0;  // elements the bulk loads cover
  const int64_t nout = FAST ? n / OV * OV : 0;   // elements the bulk stores cover
  unsigned char* outt = dsm + (size_t)STAGES * IN_BYTES;
  // The CTA's j-th tile.
  auto tile_of = [&](int j) { return (int64_t)blockIdx.x + (int64_t)j * gridDim.x; };

  // Thread 0 only: start the copy of the CTA's j-th tile into its stage.
  auto fill = [&](int j) {
    const int64_t t = tile_of(j);
    if (FAST && t < S.ntiles) {
      const int s = j % STAGES;
      const int64_t e0 = t * TILE;
      const int64_t cnt = nin - e0 < TILE ? nin - e0 : TILE;
      const unsigned bytes = (unsigned)(cnt * (int64_t)sizeof(TI));
      mbar_arrive_expect_tx(&s_bar[s], bytes);
      if (bytes) bulk_g2s(dsm + (size_t)s * IN_BYTES, x + e0, bytes, &s_bar[s]);
    }
  };

  pdl_entry();  // nothing of the previous launch is read or written before this
  if (threadIdx.x == 0) {
    s_bad = 0;
#pragma unroll
    for (int s = 0; s < STAGES; ++s) mbar_init(&s_bar[s], 1);
    fence_mbar_init();
#pragma unroll
    for (int j = 0; j < STAGES; ++j) fill(j);
  }
  __syncthreads();
  bool bad = false;

  if (warp >= WARPS) {
    // ---- look-back warp k: the CTA's tile slots k, k + NLB, k + 2 NLB, ... --
    const int k = warp - WARPS;
    while (true) {
      bar_sync(BAR_INFO + k, BAR_HANDOFF);
      const int64_t tile = s_info_tile[k];
      if (tile >= S.ntiles) break;
      const TO agg = s_info_agg[k];
      const TO excl = tile == 0 ? TO(0) : look_back<TO, lb_k<TO>(), LbSum<TO>>(S, tile, agg, true, &bad);
      if (lane == 0) {
        s_excl[k] = excl;
        if (total && tile == S.ntiles - 1) *total = INCL ? excl + agg : init + (excl + agg);
      }
      bar_arrive(BAR_PREFIX + k, BAR_HANDOFF);
    }
  } else {
    // ---- compute warps ------------------------------------------------------
    // Vector jj of this thread in the tile held by stage s.
    auto load_vec = [&](int s, int64_t tbase, int jj, TI (&v)[VEC]) {
      const int64_t e0 = tbase + ((int64_t)threadIdx.x * IPT + jj) * VEC;
      const unsigned char* stg = dsm + (size_t)s * IN_BYTES;
      if (FAST && tbase + TILE <= nin) {
        Vec16<TI> u;
        u.u = reinterpret_cast<const uint4*>(stg)[threadIdx.x * IPT + jj];
#pragma unroll
        for (int q = 0; q < VEC; ++q) v[q] = u.v[q];
      } else if (FAST) {
        const TI* sv = reinterpret_cast<const TI*>(stg) + ((size_t)threadIdx.x * IPT + jj) * VEC;
#pragma unroll
        for (int q = 0; q < VEC; ++q) v[q] = e0 + q < nin ? sv[q] : (e0 + q < n ? x[e0 + q] : TI(0));
      } else {
#pragma unroll
        for (int q = 0; q < VEC; ++q) v[q] = e0 + q < n ? x[e0 + q] : TI(0);
      }
    };
    // Tile-sum pass of the CTA's j-th tile (stage j % STAGES): this thread's
    // exclusive prefix within its warp (tex) and its warp's within the tile
    // (wpre); thread 0 publishes the aggregate and fills the hand-off slot.
    auto tile_sums = [&](int j, int64_t tile, TO& tex, TO& wpre) {
      const int s = j % STAGES;
      if (FAST && !mbar_wait(&s_bar[s], (unsigned)(j / STAGES) & 1u, S.wait_limit)) bad = true;
      TO tsum = TO(0);
#pragma unroll
      for (int jj = 0; jj < IPT; ++jj) {
        TI v[VEC];
        load_vec(s, tile * TILE, jj, v);
#pragma unroll
        for (int q = 0; q < VEC; ++q) tsum = tsum + (TO)v[q];
      }
      const TO tinc = warp_iscan(tsum);
      tex = shup(tinc, 1);
      if (lane == 0) tex = TO(0);
      if (lane == 31) s_warp[j & 1][warp] = tinc;
      bar_sync(BAR_COMPUTE, SCAN_COMPUTE);
      TO agg = TO(0);
      wpre = TO(0);
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        if (w == warp) wpre = agg;
        agg = agg + s_warp[j & 1][w];
      }
      if (threadIdx.x == 0) {
        lb_publish(S, tile, tile == 0 ? LB_FLAG_P : LB_FLAG_A, agg);
        s_info_tile[j % NLB] = tile;
        s_info_agg[j % NLB] = agg;
      }
    };

    // Per-thread prefixes of the tiles summed but not yet written: entry a
    // belongs to the CTA's tile i + a.
    TO q_tex[AHEAD + 1], q_wpre[AHEAD + 1];
#pragma unroll
    for (int a = 0; a <= AHEAD; ++a) q_tex[a] = q_wpre[a] = TO(0);
    // Hand-offs go to the look-back warps for valid tiles only, in slot
    // order; after the last one every look-back warp gets one end mark.
    auto hand_off = [&](int j) { bar_arrive(BAR_INFO + j % NLB, BAR_HANDOFF); };
#pragma unroll
    for (int a = 0; a < AHEAD; ++a) {
      if (tile_of(a) < S.ntiles) {
        tile_sums(a, tile_of(a), q_tex[a], q_wpre[a]);
        hand_off(a);
      }
    }
    int i = 0;
    for (; tile_of(i) < S.ntiles; ++i) {
      // Tile sums AHEAD tiles ahead first: that aggregate goes out while this
      // tile's prefix is being resolved.
      if (tile_of(i + AHEAD) < S.ntiles) {
        tile_sums(i + AHEAD, tile_of(i + AHEAD), q_tex[AHEAD], q_wpre[AHEAD]);
        hand_off(i + AHEAD);
      }
      bar_sync(BAR_PREFIX + i % NLB, BAR_HANDOFF);
      const TO tile_pre = s_excl[i % NLB];

      // ---- output pass of the CTA's i-th tile (stage i % STAGES) -----------
      const int s = i % STAGES;
      const int64_t tbase = tile_of(i) * TILE;
      const bool out_full = FAST && tbase + TILE <= nout;
#pragma unroll
      for (int r = 0; r < ROUNDS; ++r) {
        if (FAST ? threadIdx.x / RT == r : r == 0) {
          const int lt = FAST ? threadIdx.x - r * RT : 0;  // index within the round
          const int64_t e_thr = tbase + (int64_t)threadIdx.x * IPT * VEC;
          TO run = (INCL ? tile_pre + q_wpre[0] : init + (tile_pre + q_wpre[0])) + q_tex[0];
#pragma unroll
          for (int jj = 0; jj < IPT; ++jj) {
            TI v[VEC];
            load_vec(s, tbase, jj, v);
            TO o[VEC];
#pragma unroll
            for (int q = 0; q < VEC; ++q) {
              if (INCL) {
                run = run + (TO)v[q];
                o[q] = run;
              } else {
                o[q] = run;
                run = run + (TO)v[q];
              }
            }
            if (FAST) {
              uint4* ov = reinterpret_cast<uint4*>(outt) + ((size_t)lt * IPT + jj) * OVN;
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
                // Past the last 16-byte boundary of y: direct stores.
#pragma unroll
                for (int q = 0; q < VEC; ++q) {
                  const int64_t e = e_thr + jj * VEC + q;
                  if (e >= nout && e < n) y[e] = o[q];
                }
              }
            } else {
#pragma unroll
              for (int q = 0; q < VEC; ++q) {
                const int64_t e = e_thr + jj * VEC + q;
                if (e < n) y[e] = o[q];
              }
            }
          }
        }
        // This round's part of the out tile is written (and, after the last
        // round, stage s has been read by every compute thread): stream it to
        // y in warp-striped order, 512 contiguous bytes per warp instruction,
        // and refill the stage (the barrier orders those reads before the
        // copy's writes).
        bar_sync(BAR_COMPUTE, SCAN_COMPUTE);
        if (r == ROUNDS - 1 && threadIdx.x == 0) fill(i + STAGES);
        if (FAST) {
          const int64_t rbase = tbase + (int64_t)r * RTILE;
          const uint4* ov = reinterpret_cast<const uint4*>(outt);
          uint4* yv = reinterpret_cast<uint4*>(y + rbase);
          const int64_t left = nout - rbase < RTILE ? nout - rbase : RTILE;
          const int64_t nvec = left > 0 ? left * (int64_t)sizeof(TO) / 16 : 0;
#pragma unroll
          for (int k = 0; k < IPT * OVN / ROUNDS; ++k) {
            const int q = k * SCAN_COMPUTE + threadIdx.x;
            if (out_full || q < nvec) __stcs(yv + q, ov[q]);
          }
          // The next round rewrites the out tile.  (The next tile's first
          // writes come after its prefix barrier.)
          if (r + 1 < ROUNDS) bar_sync(BAR_COMPUTE, SCAN_COMPUTE);
        }
      }
#pragma unroll
      for (int a = 0; a < AHEAD; ++a) {
        q_tex[a] = q_tex[a + 1];
        q_wpre[a] = q_wpre[a + 1];
      }
    }
    // i = the number of tiles this CTA handed off: one end mark per look-back
    // warp, in slot order.
    for (int j = i; j < i + NLB; ++j) {
      if (threadIdx.x == 0) s_info_tile[j % NLB] = S.ntiles;
      hand_off(j);
    }
  }

  if (bad) s_bad = 1;
  __syncthreads();
  if (threadIdx.x == 0 && s_bad) atomicOr(S.err, GBK_EBIT_TIMEOUT);
}

// Launch one instantiation as a cooperative grid (all CTAs co-resident, which
// the static tile order needs): min(tiles, resident CTAs), or ctas_per_sm x
// SMs when the tuning asks for fewer.
template <class TI, class TO, bool INCL, bool FAST, int IPT, int STAGES, int AHEAD, int ROUNDS>
int launch_k_scan(const TI* x, TO* y, int64_t n, TO init, const LbState& S, TO* total, int cps, cudaStream_t s) {
  auto kfn = k_scan<TI, TO, INCL, FAST, IPT, STAGES, AHEAD, ROUNDS>;
  constexpr size_t in_bytes = (size_t)SCAN_COMPUTE * IPT * 16;
  // stages + out tile
  const size_t dyn = FAST ? STAGES * in_bytes + in_bytes * (sizeof(TO) / sizeof(TI)) / ROUNDS : 0;
  static std::atomic<int> resident{0};  // CTAs per SM, per instantiation (set once, any host thread)
  if (!resident) {
    // Static + dynamic shared memory above 48 KiB needs the opt-in.
    if (dyn) GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int r = 0;
    GBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kfn, SCAN_BLOCK, dyn));
    if (r < 1) return GBK_ERR_UNSUPPORTED;
    resident = r;
  }
  const int per_sm = cps > 0 && cps < resident ? cps : resident.load();
  const int64_t grid = std::min<int64_t>(S.ntiles, (int64_t)per_sm * sm_count());
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(SCAN_BLOCK);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = s;
  // Cooperative, and scheduled while the previous launch on the stream runs
  // (programmatic dependent launch: the kernel waits for it on the device
  // before its first access).  A driver that refuses the pair for a
  // cooperative grid gets the plain cooperative launch from then on.
  static std::atomic<bool> pdl_ok{true};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_ok && pdl_enabled() ? 2 : 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, kfn, x, y, n, init, S, total);
  if (e != cudaSuccess && cfg.numAttrs == 2) {
    (void)cudaGetLastError();
    pdl_ok = false;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kfn, x, y, n, init, S, total);
  }
  return cuda_status(e);
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
  constexpr bool WIDE = sizeof(TO) > sizeof(TI);
  // Shapes (vectors per thread, stages, tiles ahead, output rounds), all two
  // CTAs per SM; bigger tiles mean fewer look-backs.  Measured on 2^24 and
  // 2^28 elements, the default is the fastest of the shapes tried:
  //   default  9, 2, 1, 1 (widening: 7, 2, 1, 1, its out tile is two input tiles)
  //   <= 8     7, 3, 1, 1 (widening: 5, 3, 2, 1)
  //   <= 4     3, 4, 2, 1 or 2 (small tiles)
  const bool fast = (uintptr_t)x % 16 == 0 && (uintptr_t)y % 16 == 0;
  constexpr int BIG = WIDE ? 7 : 9;
  const int want = t && t->items_per_thread > 0 ? t->items_per_thread : 9;
  const int ipt = !fast ? BIG : want <= 4 ? 3 : want <= 8 ? (WIDE ? 5 : 7) : BIG;
  const int shape = !fast ? 0 : want <= 4 ? 2 : want <= 8 ? 1 : 0;
  const int cps = t ? t->ctas_per_sm : 0;
  const int64_t tile = (int64_t)SCAN_COMPUTE * ipt * VEC;
  const int64_t ntiles = (n + tile - 1) / tile;
  if (ntiles >= (int64_t)0xFFFFFFFFu - (1 << 24)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  LbState S;
  S.desc = (TileDesc*)ws_flags(w, lb_flag_words(ntiles), &S.epoch, &st);
  if (!S.desc) return st;
  S.err = w->err;
  S.ntiles = ntiles;
  S.wait_limit = wait_limit();
  constexpr int OVN = sizeof(TO) / sizeof(TI);
  if (!fast)
    st = launch_k_scan<TI, TO, INCL, false, BIG, 2, 1, 1>(x, y, n, init, S, total, cps, s);
  else if (shape == 2)
    st = launch_k_scan<TI, TO, INCL, true, 3, 4, 2, OVN>(x, y, n, init, S, total, cps, s);
  else if (shape == 1)
    st = WIDE ? launch_k_scan<TI, TO, INCL, true, 5, 3, 2, 1>(x, y, n, init, S, total, cps, s)
              : launch_k_scan<TI, TO, INCL, true, 7, 3, 1, 1>(x, y, n, init, S, total, cps, s);
  else
    st = launch_k_scan<TI, TO, INCL, true, BIG, 2, 1, 1>(x, y, n, init, S, total, cps, s);
  if (st) return st;
  note_launch();
  return GBK_OK;
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
