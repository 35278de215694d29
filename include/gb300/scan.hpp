// parallel_scan over a RangePolicy for user functors f(i, update, final)
// (core/src/Kokkos_Parallel.hpp:351-458; the reference's CUDA
// ParallelScan[WithTotal] is core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:390-1053,
// two launches), and parallel_scan over a TeamThreadRange
// (core/src/Cuda/Kokkos_Cuda_Team.hpp:231-270, 721-790).
//
// One launch: each CTA takes a tile index from a ticket (tiles it waits on
// belong to running CTAs), each thread calls the functor with final = false
// over its ITEMS consecutive indices to form its partial, the CTA scans the
// partials, warp 0 looks back over the predecessor tiles' status words (a
// 32-tile window per step, every wait bounded), and each thread calls the
// functor again with final = true starting from its exclusive prefix.  The
// status words are cleared with a memset before the launch.
#pragma once

#include "parallel.hpp"

namespace gb300k {
namespace Impl {

constexpr int kSlotScan = 33;

template <class F> struct scan_value;
// (top-level const of a parameter is not part of the function type)
template <class C, class I, class T> struct scan_value<void (C::*)(I, T&, bool) const> { using type = T; };
template <class C, class I, class T> struct scan_value<void (C::*)(const I&, T&, bool) const> { using type = T; };
template <class F> using scan_value_t = typename scan_value<decltype(&F::operator())>::type;

template <class V>
struct HdrScan {
  unsigned* flags;  // 1 = aggregate, 2 = inclusive prefix; cleared per launch
  V* agg;
  V* incl;
  unsigned* ticket;
  int* err;
  int64_t ntiles;
  int64_t wait_limit;
};

template <class V>
__device__ __forceinline__ V ld_volatile(const V* p) {
  V r;
  const volatile unsigned* s = reinterpret_cast<const volatile unsigned*>(p);
  unsigned* d = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(V) / 4); ++i) d[i] = s[i];
  return r;
}

template <class V>
__device__ V warp_excl_scan(V v, V* total) {
  const int lane = threadIdx.x & 31;
  V inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    V o;
    const unsigned* s = reinterpret_cast<const unsigned*>(&inc);
    unsigned* dd = reinterpret_cast<unsigned*>(&o);
#pragma unroll
    for (int w = 0; w < (int)(sizeof(V) / 4); ++w) dd[w] = __shfl_up_sync(0xffffffffu, s[w], d);
    if (lane >= d) inc = o + inc;
  }
  V t;
  {
    const unsigned* s = reinterpret_cast<const unsigned*>(&inc);
    unsigned* dd = reinterpret_cast<unsigned*>(&t);
#pragma unroll
    for (int w = 0; w < (int)(sizeof(V) / 4); ++w) dd[w] = __shfl_sync(0xffffffffu, s[w], 31);
  }
  *total = t;
  return inc - v;
}

// The scan's join: zero() and add(a, b) with a before b in index order
// (no commutativity assumed).  PlusJ is the functor-update default.
template <class V>
struct PlusJ {
  __device__ V zero() const { return V(0); }
  __device__ V add(const V& a, const V& b) const { return a + b; }
};

template <class V>
__device__ __forceinline__ V shfl_up_any(const V& v, int d) {
  V o;
  const unsigned* s = reinterpret_cast<const unsigned*>(&v);
  unsigned* dd = reinterpret_cast<unsigned*>(&o);
#pragma unroll
  for (int w = 0; w < (int)(sizeof(V) / 4); ++w) dd[w] = __shfl_up_sync(0xffffffffu, s[w], d);
  return o;
}
template <class V>
__device__ __forceinline__ V shfl_down_any(const V& v, int d) {
  V o;
  const unsigned* s = reinterpret_cast<const unsigned*>(&v);
  unsigned* dd = reinterpret_cast<unsigned*>(&o);
#pragma unroll
  for (int w = 0; w < (int)(sizeof(V) / 4); ++w) dd[w] = __shfl_down_sync(0xffffffffu, s[w], d);
  return o;
}
template <class V>
__device__ __forceinline__ V shfl_idx_any(const V& v, int l) {
  V o;
  const unsigned* s = reinterpret_cast<const unsigned*>(&v);
  unsigned* dd = reinterpret_cast<unsigned*>(&o);
#pragma unroll
  for (int w = 0; w < (int)(sizeof(V) / 4); ++w) dd[w] = __shfl_sync(0xffffffffu, s[w], l);
  return o;
}
// Ordered warp scan: exclusive prefix of v over lower lanes, warp total.
template <class V, class J>
__device__ V warp_excl_scan_j(const J& j, V v, V* total) {
  const int lane = threadIdx.x & 31;
  V inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const V o = shfl_up_any(inc, d);
    if (lane >= d) inc = j.add(o, inc);
  }
  *total = shfl_idx_any(inc, 31);
  const V ex = shfl_up_any(inc, 1);
  return lane == 0 ? j.zero() : ex;
}

template <class F, class V, int ITEMS, class J>
__global__ void __launch_bounds__(kBlock) k_range_scan(F f, J j, int64_t b, int64_t n, HdrScan<V> S, V* total) {
  constexpr int TILE = kBlock * ITEMS;
  constexpr int WARPS = kBlock / 32;
  __shared__ int64_t s_tile;
  __shared__ V s_w[WARPS];
  __shared__ V s_pre;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(S.ticket, 1u);
    if ((int64_t)t == S.ntiles - 1) *S.ticket = 0u;
    s_tile = t;
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t i0 = tile * TILE + (int64_t)threadIdx.x * ITEMS;
  const int64_t i1 = i0 + ITEMS < n ? i0 + ITEMS : n;
  V part = j.zero();
  for (int64_t i = i0; i < i1; ++i) f(b + i, part, false);
  V wtot;
  const V wex = warp_excl_scan_j(j, part, &wtot);
  if (lane == 0) s_w[warp] = wtot;
  __syncthreads();
  V wpre = j.zero(), agg = j.zero();
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    if (w == warp) wpre = agg;
    agg = j.add(agg, s_w[w]);
  }
  if (warp == 0) {
    V excl = j.zero();
    if (tile == 0) {
      if (lane == 0) {
        S.incl[0] = agg;
        gbk::st_release_u32(S.flags, 2u);
      }
    } else {
      if (lane == 0) {
        S.agg[tile] = agg;
        gbk::st_release_u32(S.flags + tile, 1u);
      }
      int64_t pt0 = tile - 1;
      bool gave_up = false;
      while (true) {
        const int64_t pt = pt0 - lane;
        unsigned fl = 2u;
        V val = j.zero();
        if (pt >= 0) {
          int64_t polls = 0;
          while ((fl = gbk::ld_acquire_u32(S.flags + pt)) == 0u) {
            if (++polls > S.wait_limit || gave_up) { fl = 2u; gave_up = true; break; }
            if (polls > 8) __nanosleep(128);
          }
          if (!gave_up) val = (fl == 2u) ? ld_volatile(S.incl + pt) : ld_volatile(S.agg + pt);
        }
        gave_up = __any_sync(0xffffffffu, gave_up);
        const unsigned pm = __ballot_sync(0xffffffffu, fl == 2u);
        const int last = pm ? __ffs(pm) - 1 : 31;
        // lane l holds tile pt0 - l: fold from the farthest tile to the
        // nearest (lane 0 ends with the window's ordered total)
        V c = lane <= last ? val : j.zero();
#pragma unroll
        for (int m = 1; m < 32; m <<= 1) {
          const V o = shfl_down_any(c, m);
          if (lane + m < 32) c = j.add(o, c);
        }
        excl = j.add(c, excl);
        if (pm) break;
        pt0 -= 32;
      }
      if (lane == 0) {
        if (gave_up) atomicOr(S.err, 1);
        S.incl[tile] = j.add(excl, agg);
        gbk::st_release_u32(S.flags + tile, 2u);
      }
    }
    if (lane == 0) s_pre = excl;
  }
  __syncthreads();
  const V tpre = s_pre;
  if (total && tile == S.ntiles - 1 && threadIdx.x == 0) *total = j.add(tpre, agg);
  V up = j.add(j.add(tpre, wpre), wex);
  for (int64_t i = i0; i < i1; ++i) f(b + i, up, true);
}

}  // namespace Impl

template <class V, class P, class F, class J = Impl::PlusJ<V>>
void parallel_scan_impl(const P& p, const F& f, V* host_total, J j = J()) {
  Tools::Impl::Region<F> tool_region(Tools::Impl::kScan, p.space().stream());
  static_assert(sizeof(V) % 4 == 0, "scan value size must be a multiple of 4 bytes");
  constexpr int ITEMS = 8;
  constexpr int64_t TILE = Impl::kBlock * ITEMS;
  const int64_t n = p.end() - p.begin();
  cudaStream_t s = p.space().stream();
  if (n <= 0) {
    if (host_total) *host_total = V{};
    return;
  }
  const int64_t nt = (n + TILE - 1) / TILE;
  const size_t fb = ((size_t)nt * 4 + 255) / 256 * 256, vb = ((size_t)nt * sizeof(V) + 255) / 256 * 256;
  Impl::Scratch sc = Impl::acquire(s, 256 + fb + 2 * vb);
  Impl::HdrScan<V> S;
  S.flags = reinterpret_cast<unsigned*>(sc.base + 256);
  S.agg = reinterpret_cast<V*>(sc.base + 256 + fb);
  S.incl = reinterpret_cast<V*>(sc.base + 256 + fb + vb);
  S.ticket = sc.counters + Impl::kSlotScan;
  S.err = sc.err;
  S.ntiles = nt;
  S.wait_limit = int64_t(1) << 22;
  check_cuda(cudaMemsetAsync(S.flags, 0, (size_t)nt * 4, s), "parallel_scan");
  V* dtot = host_total ? reinterpret_cast<V*>(sc.base) : nullptr;
  Impl::k_range_scan<F, V, ITEMS, J><<<(unsigned)nt, Impl::kBlock, 0, s>>>(f, j, p.begin(), n, S, dtot);
  Impl::launched(cudaGetLastError(), "parallel_scan");
  if (host_total) {
    check_cuda(cudaMemcpyAsync(host_total, dtot, sizeof(V), cudaMemcpyDeviceToHost, s), "parallel_scan");
    check(gbk_stream_check((gbk_stream_t)s), "parallel_scan");
  }
}

template <class E, class... R, class F>
void parallel_scan(const RangePolicy<E, R...>& p, const F& f) {
  parallel_scan_impl<Impl::scan_value_t<F>>(p, f, nullptr);
}
// With the total (ParallelScanWithTotal): the call fences to return it.
template <class E, class... R, class F, class V>
void parallel_scan(const RangePolicy<E, R...>& p, const F& f, V& total) {
  parallel_scan_impl<V>(p, f, &total);
}
template <class F>
void parallel_scan(int64_t n, const F& f) {
  parallel_scan(RangePolicy<>(0, n), f);
}
template <class P, class F>
void parallel_scan(const std::string& label, const P& p, const F& f) {
  Tools::Impl::LabelScope ls(label);
  parallel_scan(p, f);
}
template <class P, class F, class V>
void parallel_scan(const std::string& label, const P& p, const F& f, V& total) {
  Tools::Impl::LabelScope ls(label);
  parallel_scan(p, f, total);
}

// Team-level scan over a TeamThreadRange: each team thread takes a
// consecutive block of the range, the team scans the block totals in
// shared memory, then every thread replays its block with final = true.
template <class F>
KOKKOS_INLINE_FUNCTION void parallel_scan(const TeamThreadRangeBoundaries<>& r, const F& f) {
#ifndef __CUDA_ARCH__
  (void)r;
  (void)f;
#else
  using T = Impl::scan_value_t<F>;
  __shared__ __align__(16) unsigned char raw[33 * sizeof(T)];
  T* sm = reinterpret_cast<T*>(raw);
  const int ts = r.member.team_size(), tr = r.member.team_rank();
  const int64_t n = r.end - r.begin;
  const int64_t chunk = (n + ts - 1) / ts;
  const int64_t a = r.begin + tr * chunk;
  const int64_t e = a + chunk < r.end ? a + chunk : r.end;
  T part = T(0);
  for (int64_t i = a; i < e; ++i) f(i, part, false);
  T wtot;
  const T wex = Impl::warp_excl_scan(part, &wtot);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (ts + 31) >> 5;
  if (lane == 0) sm[warp] = wtot;
  __syncthreads();
  T wpre = T(0);
  for (int w = 0; w < nw; ++w)
    if (w < warp) wpre = wpre + sm[w];
  __syncthreads();
  T up = wpre + wex;
  for (int64_t i = a; i < e; ++i) f(i, up, true);
#endif
}

// Scan over a ThreadVectorRange: vector length 1, so the thread calls the
// functor in index order with final = true.
template <class F>
KOKKOS_INLINE_FUNCTION void parallel_scan(const ThreadVectorRangeBoundaries& r, const F& f) {
  using T = Impl::scan_value_t<F>;
  T v = T(0);
  for (int64_t i = r.begin; i < r.end; ++i) f(i, v, true);
}

namespace Impl {
template <class T>
__device__ T atomic_add_old(T* p, T v) {
  if constexpr (std::is_integral<T>::value && sizeof(T) == 8)
    return (T)atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  else if constexpr (std::is_integral<T>::value && sizeof(T) == 4)
    return (T)atomicAdd(reinterpret_cast<unsigned*>(p), (unsigned)v);
  else
    return atomicAdd(p, v);  // float, double
}
// TeamMember::team_scan: exclusive prefix sum in team_rank order, offset by
// the old *global_accum when given (the last thread adds the team total).
template <class T>
__device__ T team_exclusive_sum(const T& v, T* global_accum) {
  __shared__ __align__(16) unsigned char raw[33 * sizeof(T)];
  T* sm = reinterpret_cast<T*>(raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  T wtot;
  const T wex = warp_excl_scan(v, &wtot);
  __syncthreads();  // earlier readers of sm are done
  if (lane == 0) sm[warp] = wtot;
  __syncthreads();
  T wpre = T(0), tot = T(0);
  for (int w = 0; w < nw; ++w) {
    if (w < warp) wpre = wpre + sm[w];
    tot = tot + sm[w];
  }
  T base = T(0);
  if (global_accum) {
    if ((int)threadIdx.x == (int)blockDim.x - 1) sm[32] = atomic_add_old(global_accum, tot);
    __syncthreads();
    base = sm[32];
  }
  return base + wpre + wex;
}
}  // namespace Impl

}  // namespace gb300k
