// ScatterView contributions: histogram and general scatter-op.
//
// The reference's CUDA default is NonDuplicated + Atomic: one global
// atom.add per contribution (containers/src/Kokkos_ScatterView.hpp:152-165,
// :250-286 -> desul device_atomic_fetch_add).  Here the histogram instead
// privatises the bins in shared memory:
//   * CL = 1: each CTA holds all bins (u32 counters) and counts with
//     shared-memory atomics.
//   * CL > 1: the bins are split across the CL CTAs of a thread-block
//     cluster (bin b lives in CTA b % CL at slot b / CL); a key's count goes
//     to its owner's shared memory through distributed shared memory
//     (mapa + red.shared::cluster).  2^16 int64 bins need 256 KiB of u32
//     counters, more than one CTA has, but fit a 2-CTA cluster.
//   * AGG: warp aggregation first (match.any groups equal keys, the lowest
//     lane adds the group size), which removes same-address conflicts on the
//     hot bins of skewed (Zipf) keys.
// At the end every CTA adds its non-zero counters into the int64 bins with
// fire-and-forget red.global.add.u64.  Counts are exact integers, so the
// result is bit-exact whatever the order.  No CTA ever waits on another
// except at the cluster barriers, which the hardware co-schedules.
#include <cooperative_groups.h>

#include "gbk_internal.cuh"

namespace cg = cooperative_groups;

namespace gbk {
namespace {

__device__ __forceinline__ void dsmem_add(uint32_t local_addr, unsigned owner, unsigned v) {
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(local_addr), "r"(owner));
  asm volatile("red.shared::cluster.add.u32 [%0], %1;" ::"r"(ra), "r"(v) : "memory");
}

template <int CL, bool AGG>
__device__ __forceinline__ void count_key(int32_t k, int64_t nbins, unsigned* sh, uint32_t sh_base, bool& bad) {
  const bool ok = (uint32_t)k < (uint64_t)nbins;
  if (!ok) bad = true;
  unsigned add = 1;
  bool leader = ok;
  if (AGG) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, ok ? k : -1);
    leader = ok && ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1));
    add = __popc(peers);
  }
  if (!leader) return;
  if (CL == 1) {
    atomicAdd(sh + k, add);
  } else {
    const unsigned owner = (unsigned)k % CL;
    const unsigned slot = (unsigned)k / CL;
    dsmem_add(sh_base + 4u * slot, owner, add);
  }
}

template <int CL, int BLOCK, bool AGG>
__global__ void __launch_bounds__(BLOCK)
    k_hist_priv(const int32_t* __restrict__ keys, int64_t n, int64_t nbins, unsigned long long* bins, int* err) {
  extern __shared__ __align__(16) unsigned sh[];
  const int per = (int)((nbins + CL - 1) / CL);
  for (int i = threadIdx.x; i < per; i += BLOCK) sh[i] = 0u;
  unsigned rank = 0;
  if constexpr (CL > 1) {
    cg::cluster_group cl = cg::this_cluster();
    rank = cl.block_rank();
    cl.sync();
  } else {
    __syncthreads();
  }
  const uint32_t sh_base = (uint32_t)__cvta_generic_to_shared(sh);
  bool bad = false;
  const int64_t g = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * BLOCK;
  const uintptr_t a = (uintptr_t)keys;
  int64_t head = (int64_t)(((16 - (a & 15)) & 15) / 4);
  if (head > n) head = n;
  if (g < head) count_key<CL, AGG>(keys[g], nbins, sh, sh_base, bad);
  const int32_t* kb = keys + head;
  const int64_t nvec = (n - head) / 4;
  int64_t v = g;
  for (; v + stride < nvec; v += 2 * stride) {
    Vec16<int32_t> u0, u1;
    u0.u = ld_stream16(kb + 4 * v);
    u1.u = ld_stream16(kb + 4 * (v + stride));
#pragma unroll
    for (int j = 0; j < 4; ++j) count_key<CL, AGG>(u0.v[j], nbins, sh, sh_base, bad);
#pragma unroll
    for (int j = 0; j < 4; ++j) count_key<CL, AGG>(u1.v[j], nbins, sh, sh_base, bad);
  }
  for (; v < nvec; v += stride) {
    Vec16<int32_t> u0;
    u0.u = ld_stream16(kb + 4 * v);
#pragma unroll
    for (int j = 0; j < 4; ++j) count_key<CL, AGG>(u0.v[j], nbins, sh, sh_base, bad);
  }
  const int64_t t0 = head + nvec * 4;
  if (t0 + g < n) count_key<CL, AGG>(keys[t0 + g], nbins, sh, sh_base, bad);
  if constexpr (CL > 1) {
    cg::this_cluster().sync();
  } else {
    __syncthreads();
  }
  for (int i = threadIdx.x; i < per; i += BLOCK) {
    const unsigned c = sh[i];
    const int64_t b = (int64_t)i * CL + rank;
    if (c && b < nbins) red_add_u64(bins + b, (unsigned long long)c);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, GBK_EBIT_KEY_RANGE);
}

// One CTA per SM holding every bin as a 16-bit counter (two per 32-bit
// word, 2^16 bins in 128 KiB).  Word i holds bins i (low half) and
// i + nwords (high half): bins next to each other land in different words,
// so the few hot bins of a skewed key distribution (Zipf: bins 0, 1, 2, ...)
// do not also collide on one word with their neighbours.  The CTA walks its
// contiguous share of the keys in rounds of BLOCK*8 keys; keys for the next
// round are loaded before the current round is counted, so two rounds of
// loads are in flight.  Overflow handling, by MODE:
//
// MODE 0 (drains): after every DRAIN rounds (at most 32768 keys, so no
// half-word can pass 0xFFFF from below 0x8000) all threads sync and every
// half-word that reached 0x8000 gives 0x8000 to the global bin.  Overflow is
// therefore impossible and no carry ever reaches the neighbouring bin.
//
// MODE 1 (drain-free): each increment reads the counter's old value (the
// shared atomic returns it); the one increment that takes a 16-bit counter
// from 0x7FFF to 0x8000 moves 0x8000 to the global bin itself (a shared
// atomic subtract and a global red.add).  Until that subtract lands, other
// increments can raise the counter by less than the 0x7FFF headroom left
// (far fewer increments are in flight in one CTA), so no carry reaches the
// neighbouring bin.
//
// MODE 2 (drain-free, power-of-two bin counts): MODE 1 with the per-key
// arithmetic as multiplies (see the loop).  Measured on GB300 with ncu, the
// general form is bound by the ALU pipe (math-pipe-throttle stalls, about 27
// warp instructions per 32 keys, shared-memory wavefronts at half their
// peak); moving the work to the multiply pipe took 2^26 keys into 2^16 bins
// from 66.5 to 61.4 us (Zipf 1.1) and from 70.1 to 64.7 us (uniform).
template <int BLOCK, bool AGG, int MODE>
__global__ void __launch_bounds__(BLOCK, 1)
    k_hist16(const int32_t* __restrict__ keys, int64_t nvec, int64_t nbins, unsigned long long* bins, int* err,
             unsigned mulw, unsigned cffff, unsigned c7fff) {
  extern __shared__ __align__(16) unsigned sh[];
  constexpr int VPT = 2;                       // vectors (4 keys each) per thread per round (4: slower)
  constexpr int ROUND = BLOCK * VPT;           // vectors per round
  constexpr int DRAIN = 32768 / (ROUND * 4);   // rounds between drains
  static_assert(DRAIN >= 1, "round too large for 16-bit counters");
  constexpr bool NODRAIN = MODE == 1 || MODE == 2 || MODE == 4;
  const int nwords = (int)((nbins + 1) >> 1);
  for (int i = threadIdx.x; i <= nwords; i += BLOCK) sh[i] = 0u;  // the counters and the spare word
  pdl_entry();
  __syncthreads();
  bool bad = false;
  // Contiguous, balanced share of the vectors for this CTA.
  const int64_t per = nvec / gridDim.x, rem = nvec % gridDim.x;
  const int64_t v0 = blockIdx.x * per + (blockIdx.x < rem ? blockIdx.x : rem);
  const int64_t v1 = v0 + per + (blockIdx.x < rem ? 1 : 0);
  const unsigned nb32 = (unsigned)nbins, nw32 = (unsigned)nwords;  // nbins fits the 200 KiB of counters
  auto count = [&](int32_t k) {
    if (AGG) {
      const bool ok = (uint32_t)k < (uint64_t)nbins;
      if (!ok) bad = true;
      const unsigned act = __activemask();
      const unsigned peers = __match_any_sync(act, ok ? k : -1);
      const bool leader = ok && ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1));
      const unsigned add = __popc(peers);
      if (leader) {
        const bool hi = k >= nwords;
        atomicAdd(sh + (hi ? k - nwords : k), add << (hi ? 16 : 0));
      }
    } else {
      // Branch-free: a key outside the bins counts into the spare word
      // sh[nwords] (never drained nor flushed) and raises the error flag.
      const unsigned uk = (unsigned)k;
      const bool ok = uk < nb32;
      bad = bad || !ok;
      const unsigned hi = uk >= nw32 ? 1u : 0u;
      const unsigned word = ok ? uk - (hi ? nw32 : 0u) : nw32;
      const unsigned old = atomicAdd(sh + word, 1u << (hi << 4));
      if (NODRAIN && ok && ((old >> (hi << 4)) & 0xFFFFu) == 0x7FFFu) {
        atomicSub(sh + word, 0x8000u << (hi << 4));
        red_add_u64(bins + (hi ? nw32 + word : word), 0x8000ull);
      }
    }
  };
  auto drain_word = [&](int i, unsigned w) {
    const unsigned hi = w & 0x80008000u;
    if (hi) {
      sh[i] = w - hi;
      if (hi & 0x8000u) red_add_u64(bins + i, 0x8000ull);
      if (hi & 0x80000000u) red_add_u64(bins + nwords + i, 0x8000ull);
    }
  };
  // Every word is scanned once per drain (as many word reads as keys
  // between drains): 16-byte reads and one test per four words.
  auto drain = [&]() {
    __syncthreads();
    const int nq = nwords >> 2;
    const uint4* sq = reinterpret_cast<const uint4*>(sh);
    for (int i = threadIdx.x; i < nq; i += BLOCK) {
      const uint4 w = sq[i];
      if ((w.x | w.y | w.z | w.w) & 0x80008000u) {
        drain_word(4 * i, w.x);
        drain_word(4 * i + 1, w.y);
        drain_word(4 * i + 2, w.z);
        drain_word(4 * i + 3, w.w);
      }
    }
    for (int i = 4 * nq + threadIdx.x; i < nwords; i += BLOCK) drain_word(i, sh[i]);
    __syncthreads();
  };
  int64_t v = v0;
  if constexpr (MODE == 4) {
    // MODE 2's arithmetic with the round's eight atomics issued back to
    // back and one crossing test per round: t = (old ^ 0x7FFF<<half) &
    // 0xFFFF<<half is zero only for the increment that took its counter
    // from 0x7FFF to 0x8000, so the minimum of the eight t is zero when any
    // crossing happened; that rare round then finds its crossings one by
    // one.  The crossing thread subtracts once its round's eight atomics
    // have returned (a few hundred cycles); passing the 0x7FFF headroom
    // meanwhile would take 32,767 more increments of that one counter, which
    // shared memory applies one at a time.
    // Two register sets take turns (one is counted while the other loads),
    // and only a CTA's last, partial round checks bounds per vector.
    auto load = [&](Vec16<int32_t>* r, int64_t vb) {
#pragma unroll
      for (int j = 0; j < VPT; ++j) {
        const int64_t q = vb + (int64_t)j * BLOCK + threadIdx.x;
        r[j].u = q < v1 ? ld_stream16(keys + 4 * q) : make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
      }
    };
    auto count_round = [&](const Vec16<int32_t>* r, int64_t vb) {
      if (vb + ROUND <= v1) {
        unsigned mx = 0;
#pragma unroll
        for (int j = 0; j < VPT; ++j)
          mx = max(mx, max(__vimax3_u32((unsigned)r[j].v[0], (unsigned)r[j].v[1], (unsigned)r[j].v[2]),
                           (unsigned)r[j].v[3]));
        if (mx < nb32) {
          unsigned o[VPT * 4];
#pragma unroll
          for (int j = 0; j < VPT; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const unsigned uk = (unsigned)r[j].v[e];
              const unsigned hi = __umulhi(uk, mulw);
              o[j * 4 + e] = atomicAdd(sh + (uk - hi * nw32), 1u + hi * cffff);
            }
          unsigned t = 0xFFFFFFFFu;
#pragma unroll
          for (int j = 0; j < VPT; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const unsigned inc = 1u + __umulhi((unsigned)r[j].v[e], mulw) * cffff;
              t = min(t, (o[j * 4 + e] ^ (inc * c7fff)) & (inc * cffff));
            }
          if (t == 0u) {
#pragma unroll
            for (int j = 0; j < VPT; ++j)
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const unsigned uk = (unsigned)r[j].v[e];
                const unsigned hi = __umulhi(uk, mulw);
                const unsigned word = uk - hi * nw32;
                const unsigned inc = 1u + hi * cffff;
                if (((o[j * 4 + e] ^ (inc * c7fff)) & (inc * cffff)) == 0u) {
                  atomicSub(sh + word, inc << 15);
                  red_add_u64(bins + word + hi * nw32, 0x8000ull);
                }
              }
          }
        } else {
#pragma unroll
          for (int j = 0; j < VPT; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) count(r[j].v[e]);
        }
      } else {
#pragma unroll
        for (int j = 0; j < VPT; ++j) {
          const int64_t q = vb + (int64_t)j * BLOCK + threadIdx.x;
          if (q < v1) {
#pragma unroll
            for (int e = 0; e < 4; ++e) count(r[j].v[e]);
          }
        }
      }
    };
    Vec16<int32_t> ra[VPT], rb[VPT];
    load(ra, v);
    while (v < v1) {
      load(rb, v + ROUND);
      count_round(ra, v);
      v += ROUND;
      if (v >= v1) break;
      load(ra, v + ROUND);
      count_round(rb, v);
      v += ROUND;
    }
  } else {
  Vec16<int32_t> cur[VPT], nxt[VPT];
#pragma unroll
  for (int j = 0; j < VPT; ++j) {
    const int64_t q = v + (int64_t)j * BLOCK + threadIdx.x;
    cur[j].u = q < v1 ? ld_stream16(keys + 4 * q) : make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
  }
  int since = 0;
  while (v < v1) {
    const int64_t vn = v + ROUND;
#pragma unroll
    for (int j = 0; j < VPT; ++j) {
      const int64_t q = vn + (int64_t)j * BLOCK + threadIdx.x;
      nxt[j].u = q < v1 ? ld_stream16(keys + 4 * q) : make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    }
    if constexpr (MODE == 2 && !AGG) {
      // Power-of-two bins: the word, the half and the increment come from
      // multiplies (hi = key >> log2(nwords) as a high multiply by mulw; word
      // = key - hi * nwords; increment 1 or 0x10000 = 1 + hi * 0xFFFF) and the
      // crossing test is one masked compare, so a key costs few ALU-pipe
      // instructions (the ALU pipe bounds the general form).  The constants
      // arrive as kernel arguments so that they stay multiplies.  A vector
      // with any key outside the bins takes the general path.
#pragma unroll
      for (int j = 0; j < VPT; ++j) {
        const int64_t q = v + (int64_t)j * BLOCK + threadIdx.x;
        if (q < v1) {
          const unsigned k0 = (unsigned)cur[j].v[0], k1 = (unsigned)cur[j].v[1];
          const unsigned k2 = (unsigned)cur[j].v[2], k3 = (unsigned)cur[j].v[3];
          const unsigned mx = max(__vimax3_u32(k0, k1, k2), k3);
          if (mx < nb32) {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const unsigned uk = (unsigned)cur[j].v[e];
              const unsigned hi = __umulhi(uk, mulw);
              const unsigned word = uk - hi * nw32;
              const unsigned inc = 1u + hi * cffff;
              const unsigned old = atomicAdd(sh + word, inc);
              if (((old & (inc * cffff)) ^ (inc * c7fff)) == 0u) {
                atomicSub(sh + word, inc << 15);
                red_add_u64(bins + word + hi * nw32, 0x8000ull);
              }
            }
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) count(cur[j].v[e]);
          }
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < VPT; ++j) {
        const int64_t q = v + (int64_t)j * BLOCK + threadIdx.x;
        if (q < v1) {
#pragma unroll
          for (int e = 0; e < 4; ++e) count(cur[j].v[e]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < VPT; ++j) cur[j] = nxt[j];
    v = vn;
    if (!NODRAIN && ++since == DRAIN) {
      since = 0;
      drain();
    }
  }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nwords; i += BLOCK) {
    const unsigned w = sh[i];
    if (w & 0xFFFFu) red_add_u64(bins + i, (unsigned long long)(w & 0xFFFFu));
    if ((w >> 16) && nwords + i < nbins) red_add_u64(bins + nwords + i, (unsigned long long)(w >> 16));
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, GBK_EBIT_KEY_RANGE);
}

// Keys that are not part of a whole 16-byte vector (unaligned head, tail).
__global__ void k_hist_edges(const int32_t* __restrict__ keys, int64_t head, int64_t tail0, int64_t n, int64_t nbins,
                             unsigned long long* bins, int* err) {
  const int64_t i = threadIdx.x;
  int64_t idx = -1;
  if (i < head) idx = i;
  else if (i - head < n - tail0) idx = tail0 + (i - head);
  if (idx < 0) return;
  const int32_t k = keys[idx];
  if ((uint32_t)k < (uint64_t)nbins) red_add_u64(bins + k, 1ull);
  else atomicOr(err, GBK_EBIT_KEY_RANGE);
}

template <bool AGG, int MODE>
int launch_hist16(const int32_t* keys, int64_t n, int64_t nbins, int64_t* bins, Workspace* w) {
  constexpr int BLOCK = 1024;
  const size_t smem = (size_t)((nbins + 1) >> 1) * 4 + 16;  // counters, then the spare word for keys outside the bins
  auto kfn = k_hist16<BLOCK, AGG, MODE>;
  GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uintptr_t a = (uintptr_t)keys;
  int64_t head = (int64_t)(((16 - (a & 15)) & 15) / 4);
  if (head > n) head = n;
  const int64_t nvec = (n - head) / 4;
  const int64_t tail0 = head + nvec * 4;
  if (head || tail0 < n) {
    k_hist_edges<<<1, 32, 0, w->stream>>>(keys, head, tail0, n, nbins, (unsigned long long*)bins, w->err);
    note_launch();
  }
  if (nvec > 0) {
    int64_t grid = sm_count();
    const int64_t need = (nvec + BLOCK * 2 - 1) / (BLOCK * 2);
    if (grid > need) grid = need;
    // MODEs 2 and 4 need a power-of-two bin count of at least 4 (mulw = 2^32 / nwords)
    const unsigned mulw = MODE == 2 || MODE == 4 ? (unsigned)((1ull << 32) / (uint64_t)((nbins + 1) >> 1)) : 0u;
    GBK_CUDA_TRY(launch_pdl(kfn, dim3((unsigned)grid), dim3(BLOCK), smem, w->stream, keys + head, nvec, nbins,
                            (unsigned long long*)bins, w->err, mulw, 0xFFFFu, 0x7FFFu));
    note_launch();
  }
  return cuda_status(cudaGetLastError());
}

// No privatisation (bins too many for shared memory): warp-aggregated
// global reductions.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_hist_global(const int32_t* __restrict__ keys, int64_t n, int64_t nbins, unsigned long long* bins, int* err) {
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (int64_t)gridDim.x * BLOCK) {
    const int32_t k = keys[i];
    const bool ok = (uint32_t)k < (uint64_t)nbins;
    if (!ok) bad = true;
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, ok ? k : -1);
    if (ok && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) red_add_u64(bins + k, (unsigned long long)__popc(peers));
  }
  if (bad) atomicOr(err, GBK_EBIT_KEY_RANGE);
}

template <int CL, int BLOCK, bool AGG>
int launch_priv(const int32_t* keys, int64_t n, int64_t nbins, int64_t* bins, Workspace* w, int ctas_per_sm) {
  const size_t smem = (size_t)((nbins + CL - 1) / CL) * 4;
  auto kfn = k_hist_priv<CL, BLOCK, AGG>;
  GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 1) GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(BLOCK);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = w->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // One wave of co-resident clusters (the count the hardware can place at
  // once), capped by ctas_per_sm and by the work.
  int64_t grid = (int64_t)sm_count() * (ctas_per_sm > 0 ? ctas_per_sm : 1);
  cfg.gridDim = dim3((unsigned)grid);
  int ncl = 0;
  if (cudaOccupancyMaxActiveClusters(&ncl, kfn, &cfg) == cudaSuccess && ncl > 0 && (int64_t)ncl * CL < grid)
    grid = (int64_t)ncl * CL;
  const int64_t need = (n + (int64_t)BLOCK * 8 - 1) / ((int64_t)BLOCK * 8);
  if (grid > need) grid = need;
  if (grid < CL) grid = CL;
  grid = grid / CL * CL;
  // Each cluster counts in u32: keep keys per cluster below 2^32.
  while (n / (grid / CL) >= (int64_t)0xFFFFFFFFLL) grid += CL;
  cfg.gridDim = dim3((unsigned)grid);
  GBK_CUDA_TRY(cudaLaunchKernelEx(&cfg, kfn, keys, n, nbins, (unsigned long long*)bins, w->err));
  note_launch();
  return GBK_OK;
}

int hist_launch(const int32_t* keys, int64_t n, int64_t* bins, int64_t nbins, Workspace* w, const gbk_tuning_t* t) {
  if (n == 0) return GBK_OK;
  // variant bits: 0x0F cluster size of the 32-bit privatised kernel (1, 2,
  // 4, 8); 0x10 warp aggregation; 0x20 the 16-bit one-CTA-per-SM kernel;
  // 0x40 no privatisation; 0x80 the 16-bit kernel without drains; 0x100
  // the same in its multiply form for power-of-two bin counts; 0x200 the
  // multiply form with one crossing test per round.
  // 0 = automatic choice.
  const int var = t ? t->variant : 0;
  int cl = var & 0xF;
  bool agg = (var & 0x10) != 0;
  const int cps = t && t->ctas_per_sm ? t->ctas_per_sm : 1;
  const int64_t max_smem = 200 * 1024;
  bool use16 = (var & 0x20) != 0;
  const bool force_global = (var & 0x40) != 0;
  if (var == 0) {
    if (nbins * 4 <= 96 * 1024) cl = 1;
    else if ((nbins + 1) / 2 * 4 <= max_smem) {
      const bool pow2 = (nbins & (nbins - 1)) == 0;  // nbins > 24576 here
      return pow2 ? launch_hist16<false, 2>(keys, n, nbins, bins, w) : launch_hist16<false, 1>(keys, n, nbins, bins, w);
    }
    else { cl = 2; while (cl <= 8 && (nbins + cl - 1) / cl * 4 > max_smem) cl *= 2; }
  }
  if ((var & 0x200) && (nbins + 1) / 2 * 4 <= max_smem) {
    const bool pow2 = nbins >= 4 && (nbins & (nbins - 1)) == 0;
    return pow2 ? launch_hist16<false, 4>(keys, n, nbins, bins, w) : launch_hist16<false, 1>(keys, n, nbins, bins, w);
  }
  if ((var & 0x100) && (nbins + 1) / 2 * 4 <= max_smem) {
    const bool pow2 = nbins >= 4 && (nbins & (nbins - 1)) == 0;
    return pow2 ? launch_hist16<false, 2>(keys, n, nbins, bins, w) : launch_hist16<false, 1>(keys, n, nbins, bins, w);
  }
  if ((var & 0x80) && (nbins + 1) / 2 * 4 <= max_smem) return launch_hist16<false, 1>(keys, n, nbins, bins, w);
  if (use16 && !force_global && (nbins + 1) / 2 * 4 <= max_smem) {
    return agg ? launch_hist16<true, 0>(keys, n, nbins, bins, w) : launch_hist16<false, 0>(keys, n, nbins, bins, w);
  }
  if (cl == 0) cl = 1;
  if (force_global || (nbins + cl - 1) / cl * 4 > max_smem || cl > 8) {
    int64_t grid = (int64_t)sm_count() * 8;
    k_hist_global<256><<<(unsigned)grid, 256, 0, w->stream>>>(keys, n, nbins, (unsigned long long*)bins, w->err);
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  // Two 1024-thread CTAs per SM when the private table is small enough.
  const int cps2 = (t && t->ctas_per_sm) ? cps : ((nbins + cl - 1) / cl * 4 <= 100 * 1024 ? 2 : 1);
#define GBK_HL(C, A) return launch_priv<C, 1024, A>(keys, n, nbins, bins, w, cps2)
  switch (cl) {
    case 1: if (agg) GBK_HL(1, true); else GBK_HL(1, false);
    case 2: if (agg) GBK_HL(2, true); else GBK_HL(2, false);
    case 4: if (agg) GBK_HL(4, true); else GBK_HL(4, false);
    case 8: if (agg) GBK_HL(8, true); else GBK_HL(8, false);
  }
#undef GBK_HL
  return GBK_ERR_INVALID_ARGUMENT;
}

// ---- general scatter -------------------------------------------------------
template <class T> struct AtomOps;
template <> struct AtomOps<int32_t> {
  __device__ static void add(int32_t* p, int32_t v) { atomicAdd(p, v); }
  __device__ static void mn(int32_t* p, int32_t v) { atomicMin(p, v); }
  __device__ static void mx(int32_t* p, int32_t v) { atomicMax(p, v); }
};
template <> struct AtomOps<uint32_t> {
  __device__ static void add(uint32_t* p, uint32_t v) { atomicAdd(p, v); }
  __device__ static void mn(uint32_t* p, uint32_t v) { atomicMin(p, v); }
  __device__ static void mx(uint32_t* p, uint32_t v) { atomicMax(p, v); }
};
template <> struct AtomOps<int64_t> {
  __device__ static void add(int64_t* p, int64_t v) { atomicAdd((unsigned long long*)p, (unsigned long long)v); }
  __device__ static void mn(int64_t* p, int64_t v) { atomicMin((long long*)p, (long long)v); }
  __device__ static void mx(int64_t* p, int64_t v) { atomicMax((long long*)p, (long long)v); }
};
template <> struct AtomOps<uint64_t> {
  __device__ static void add(uint64_t* p, uint64_t v) { atomicAdd((unsigned long long*)p, (unsigned long long)v); }
  __device__ static void mn(uint64_t* p, uint64_t v) { atomicMin((unsigned long long*)p, (unsigned long long)v); }
  __device__ static void mx(uint64_t* p, uint64_t v) { atomicMax((unsigned long long*)p, (unsigned long long)v); }
};
template <class T, class F>
__device__ void cas_loop(T* p, F f) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "size");
  using U = typename std::conditional<sizeof(T) == 4, unsigned, unsigned long long>::type;
  U* up = reinterpret_cast<U*>(p);
  U old = *reinterpret_cast<volatile U*>(up), assumed;
  do {
    assumed = old;
    T cur;
    memcpy(&cur, &assumed, sizeof(T));
    const T nv = f(cur);
    U nu;
    memcpy(&nu, &nv, sizeof(T));
    if (nu == assumed) return;
    old = atomicCAS(up, assumed, nu);
  } while (old != assumed);
}
template <> struct AtomOps<float> {
  __device__ static void add(float* p, float v) { atomicAdd(p, v); }
  __device__ static void mn(float* p, float v) { cas_loop(p, [v](float c) { return v < c ? v : c; }); }
  __device__ static void mx(float* p, float v) { cas_loop(p, [v](float c) { return v > c ? v : c; }); }
};
template <> struct AtomOps<double> {
  __device__ static void add(double* p, double v) { atomicAdd(p, v); }
  __device__ static void mn(double* p, double v) { cas_loop(p, [v](double c) { return v < c ? v : c; }); }
  __device__ static void mx(double* p, double v) { cas_loop(p, [v](double c) { return v > c ? v : c; }); }
};

template <class T, int OP>
__global__ void k_scatter(const int32_t* __restrict__ idx, const T* __restrict__ vals, int64_t n, T* dest,
                          int64_t ndest, int* err) {
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = idx[i];
    if ((uint32_t)k >= (uint64_t)ndest) { bad = true; continue; }
    const T v = vals[i];
    if (OP == GBK_SUM) AtomOps<T>::add(dest + k, v);
    else if (OP == GBK_MIN) AtomOps<T>::mn(dest + k, v);
    else if (OP == GBK_MAX) AtomOps<T>::mx(dest + k, v);
    else cas_loop(dest + k, [v](T c) { return c * v; });
  }
  if (bad) atomicOr(err, GBK_EBIT_KEY_RANGE);
}

template <class T>
int scatter_t(int op, const int32_t* idx, const void* vals, int64_t n, void* dest, int64_t nd, Workspace* w) {
  if (n == 0) return GBK_OK;
  int64_t grid = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (grid > cap) grid = cap;
  const T* v = (const T*)vals;
  T* d = (T*)dest;
  switch (op) {
    case GBK_SUM: k_scatter<T, GBK_SUM><<<(unsigned)grid, 256, 0, w->stream>>>(idx, v, n, d, nd, w->err); break;
    case GBK_PROD: k_scatter<T, GBK_PROD><<<(unsigned)grid, 256, 0, w->stream>>>(idx, v, n, d, nd, w->err); break;
    case GBK_MIN: k_scatter<T, GBK_MIN><<<(unsigned)grid, 256, 0, w->stream>>>(idx, v, n, d, nd, w->err); break;
    case GBK_MAX: k_scatter<T, GBK_MAX><<<(unsigned)grid, 256, 0, w->stream>>>(idx, v, n, d, nd, w->err); break;
    default: return GBK_ERR_UNSUPPORTED;
  }
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_histogram_i32_i64(const int32_t* keys, int64_t n, int64_t* bins, int64_t nbins, gbk_stream_t stream,
                          const gbk_tuning_t* tune) {
  if (n < 0 || nbins <= 0 || nbins > 0x7FFFFFFF || !bins || (n > 0 && !keys)) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)keys % 4 || (uintptr_t)bins % 8) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  gbk_tuning_t tt;
  if (!tune) {
    int lb = 0;
    while (((int64_t)1 << lb) < nbins) ++lb;
    tune = tuned_config(TUNE_HIST, 0, GBK_I32, n, lb * 8, &tt);
  }
  std::lock_guard<std::mutex> lk(w->mu);
  return hist_launch(keys, n, bins, nbins, w, tune);
}

int gbk_histogram_i32_i64_host(const int32_t* hkeys, int64_t n, int64_t* hbins, int64_t nbins, gbk_stream_t stream,
                               const gbk_tuning_t* tune) {
  if (n < 0 || nbins <= 0 || nbins > 0x7FFFFFFF || !hbins || (n > 0 && !hkeys)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Workspace* w = ws_get(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  const size_t kb = ((size_t)n * 4 + 255) / 256 * 256;
  char* d = ws_stage(w, kb + (size_t)nbins * 8 + 256, &st);
  if (!d) return st;
  int64_t* db = (int64_t*)(d + kb);
  if (n) GBK_CUDA_TRY(cudaMemcpyAsync(d, hkeys, (size_t)n * 4, cudaMemcpyHostToDevice, s));
  GBK_CUDA_TRY(cudaMemcpyAsync(db, hbins, (size_t)nbins * 8, cudaMemcpyHostToDevice, s));
  st = hist_launch((const int32_t*)d, n, db, nbins, w, tune);
  if (st) return st;
  GBK_CUDA_TRY(cudaMemcpyAsync(hbins, db, (size_t)nbins * 8, cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  return GBK_OK;
}

int gbk_scatter(gbk_reducer_t op, gbk_dtype_t dt, const int32_t* idx, const void* vals, int64_t n, void* dest,
                int64_t nd, gbk_stream_t stream) {
  if (n < 0 || nd < 0 || (n > 0 && (!idx || !vals || !dest))) return GBK_ERR_INVALID_ARGUMENT;
  if (op != GBK_SUM && op != GBK_PROD && op != GBK_MIN && op != GBK_MAX) return GBK_ERR_UNSUPPORTED;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  switch (dt) {
    case GBK_I32: return scatter_t<int32_t>(op, idx, vals, n, dest, nd, w);
    case GBK_I64: return scatter_t<int64_t>(op, idx, vals, n, dest, nd, w);
    case GBK_U32: return scatter_t<uint32_t>(op, idx, vals, n, dest, nd, w);
    case GBK_U64: return scatter_t<uint64_t>(op, idx, vals, n, dest, nd, w);
    case GBK_F32: return scatter_t<float>(op, idx, vals, n, dest, nd, w);
    case GBK_F64: return scatter_t<double>(op, idx, vals, n, dest, nd, w);
  }
  return GBK_ERR_UNSUPPORTED;
}

}  // extern "C"
