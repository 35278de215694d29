// Kernel skeletons of the GB300 execution space: parallel_for, parallel_reduce
// and parallel_scan over a flat index space, for any closure.
//
// These kernels know nothing of Kokkos' types.  A closure (built by the
// pattern specialisations in Kokkos_GB300_Parallel_*.hpp from a Kokkos functor
// and its FunctorAnalysis reducer) supplies the work and the value algebra:
//
//   for:     __device__ void exec(int64_t i) const;
//   reduce:  __device__ void init(void* v) const;           // reducer.init
//            __device__ void join(void* dst, const void* src) const;
//            __device__ void exec(int64_t i, void* v) const; // functor(i, update)
//            __device__ void final_(void* v) const;         // reducer.final
//   scan:    the reduce members, with exec(i, v, bool final_pass).
//
// The value is VB bytes (the reducer's value_size rounded up to 16; at most
// kMaxValueBytes), held per thread in registers or local memory and moved
// between lanes as 32-bit words.  Scratch (per-CTA partials, look-back
// descriptors) and the ticket counters come from the library workspace of the
// stream (gbk_workspace_acquire), so nothing here allocates.
//
// Shapes (the library's flat-kernel design, see gbk_reduce_impl.cuh):
//   * for / reduce: a grid of at most SMs x 8 CTAs of 256 threads; CTA b owns
//     one contiguous, equal share of [0, n) and its threads stride by 256
//     through it (coalesced for functors that read x(i)); each thread works
//     kUnroll indices per step, so kUnroll independent loads are in flight
//     per thread even though the functor updates one value;
//   * reduce finish: a warp butterfly and a CTA tree of the closure's join,
//     then the last CTA to take a ticket joins the per-CTA partials in CTA
//     order, applies final_ and stores the result: one launch;
//   * scan: decoupled look-back (Merrill & Garland 2016): each CTA takes a
//     tile index from a ticket (every tile it waits on belongs to a CTA that
//     is already running), calls the functor with final_pass = false over
//     its kItems consecutive indices per thread, publishes the tile's
//     aggregate, warp 0 folds the predecessors' aggregates / inclusive
//     prefixes 32 tiles per step (every wait bounded, a give-up is reported
//     in the stream's error word), and every thread runs its indices again
//     with final_pass = true from its exclusive prefix.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <type_traits>

#include "../../gbk.h"

namespace gbk_skel {

constexpr int kBlock = 256;
constexpr int kUnroll = 4;
constexpr int kItems = 8;
constexpr int kMaxValueBytes = 256;
// Ticket slots of the stream workspace used by these kernels (slots 32..63
// are free for kernels instantiated outside the library; each kernel resets
// its slot before it exits).
constexpr int kSlotReduce = 40;
constexpr int kSlotScan = 41;
// Bit of the stream's error word (gbk_stream_check -> GBK_ERR_DEVICE_ABORT)
// that a kernel sets when code it ran asked for an abort.
constexpr int kErrBitAbort = 8;

// Device-side abort request (Kokkos::abort called in device code): the first
// request of this translation unit prints its message, a flag of the unit is
// set, which every skeleton kernel of the unit folds into its stream's error
// word when it finishes (so the next fence raises it), and the calling thread
// ends (PTX exit: no trap, the context stays usable).  The flag stays set for
// the rest of the process, as a device-side assertion would leave a CUDA
// context unusable.  Correct programs never reach this path.
static __device__ int g_abort_requested = 0;
__device__ inline void request_abort(const char* msg) {
  if (atomicExch(&g_abort_requested, 1) == 0) printf("Kokkos::abort on the GB300 device: %s\n", msg);
  __threadfence();
  asm volatile("exit;");
}
__device__ __forceinline__ void report_abort(int* err) {
  if (threadIdx.x == 0 && err && *(volatile int*)&g_abort_requested) atomicOr(err, kErrBitAbort);
}

template <int VB>
struct alignas(16) Val {
  unsigned w[VB / 4];
};

constexpr int value_bytes(size_t value_size) { return (int)((value_size + 15) / 16 * 16); }

// ---- lane exchange of an opaque value ------------------------------------
template <int VB>
__device__ __forceinline__ Val<VB> shfl_xor(const Val<VB>& v, int m) {
  Val<VB> o;
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) o.w[i] = __shfl_xor_sync(0xffffffffu, v.w[i], m);
  return o;
}
template <int VB>
__device__ __forceinline__ Val<VB> shfl_up(const Val<VB>& v, int d) {
  Val<VB> o;
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) o.w[i] = __shfl_up_sync(0xffffffffu, v.w[i], d);
  return o;
}
template <int VB>
__device__ __forceinline__ Val<VB> shfl_down(const Val<VB>& v, int d) {
  Val<VB> o;
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) o.w[i] = __shfl_down_sync(0xffffffffu, v.w[i], d);
  return o;
}
template <int VB>
__device__ __forceinline__ Val<VB> shfl_idx(const Val<VB>& v, int l) {
  Val<VB> o;
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) o.w[i] = __shfl_sync(0xffffffffu, v.w[i], l);
  return o;
}
template <int VB>
__device__ __forceinline__ Val<VB> ld_cg(const Val<VB>* p) {
  Val<VB> r;
  const unsigned* s = reinterpret_cast<const unsigned*>(p);
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) r.w[i] = __ldcg(s + i);
  return r;
}
template <int VB>
__device__ __forceinline__ Val<VB> ld_volatile(const Val<VB>* p) {
  Val<VB> r;
  const volatile unsigned* s = reinterpret_cast<const volatile unsigned*>(p);
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) r.w[i] = s[i];
  return r;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// A CTA's contiguous share of [0, n).
__device__ __forceinline__ void cta_share(int64_t n, int64_t* c0, int64_t* c1) {
  const int64_t per = n / gridDim.x, rem = n % gridDim.x, b = blockIdx.x;
  *c0 = b * per + (b < rem ? b : rem);
  *c1 = *c0 + per + (b < rem ? 1 : 0);
}

// Join of every thread's value; the CTA's total ends in thread 0.
template <int VB, class C>
__device__ Val<VB> cta_reduce(const C& c, Val<VB> v) {
  __shared__ Val<VB> sm[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    const Val<VB> o = shfl_xor(v, m);
    c.join(&v, &o);
  }
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    if (lane < nw) v = sm[lane];
    else c.init(&v);
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      const Val<VB> o = shfl_xor(v, m);
      c.join(&v, &o);
    }
  }
  __syncthreads();
  return v;
}


// The same for any CTA size (a team need not be a multiple of 32 threads):
// shifts down within each warp's active lanes, lane 0 of the CTA ends with
// the total, joined in thread order.
template <int VB>
__device__ __forceinline__ Val<VB> shfl_down_m(const Val<VB>& v, int d, unsigned mask) {
  Val<VB> o;
#pragma unroll
  for (int i = 0; i < VB / 4; ++i) o.w[i] = __shfl_down_sync(mask, v.w[i], d);
  return o;
}
__device__ __forceinline__ unsigned warp_mask_of(int count) {
  return count >= 32 ? 0xffffffffu : ((1u << count) - 1u);
}
template <int VB, class C>
__device__ Val<VB> cta_reduce_any(const C& c, Val<VB> v) {
  __shared__ Val<VB> sm[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const int cnt = min(32, (int)blockDim.x - warp * 32);
  const unsigned mask = warp_mask_of(cnt);
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const Val<VB> o = shfl_down_m(v, d, mask);
    if (lane + d < cnt) c.join(&v, &o);
  }
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    if (lane < nw) v = sm[lane];
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      const Val<VB> o = shfl_down_m(v, d, mask);
      if (lane + d < nw) c.join(&v, &o);
    }
  }
  __syncthreads();
  return v;
}

// ---- parallel_for ---------------------------------------------------------
// A closure may walk its index space itself: with a nested walk_state type it
// provides walk_start(state, flat), walk_exec(state[, value]) and
// walk_next(state), the last stepping by kBlock flat indices; the loops
// below then use those instead of exec(flat) (the MDRange closures keep
// their multi-index instead of dividing for every element).
template <class C, class = void>
struct has_walk : std::false_type {};
template <class C>
struct has_walk<C, std::void_t<typename C::walk_state>> : std::true_type {};

template <class C>
__global__ void __launch_bounds__(kBlock) k_for(const C c, int64_t begin, int64_t n, int* err) {
  int64_t c0, c1;
  cta_share(n, &c0, &c1);
  int64_t i = c0 + threadIdx.x;
  if constexpr (has_walk<C>::value) {
    if (i < c1) {
      typename C::walk_state w;
      c.walk_start(w, begin + i);
      for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
          c.walk_exec(w);
          c.walk_next(w);
        }
      }
      for (; i < c1; i += kBlock) {
        c.walk_exec(w);
        c.walk_next(w);
      }
    }
  } else {
    for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) c.exec(begin + i + u * kBlock);
    }
    for (; i < c1; i += kBlock) c.exec(begin + i);
  }
  report_abort(err);
}

// ---- parallel_reduce ------------------------------------------------------
// partials: gridDim.x values; counter: a zeroed ticket the kernel leaves at
// zero; out: where the final value goes (device memory).
template <int VB, class C>
__global__ void __launch_bounds__(kBlock)
    k_reduce(const C c, int64_t begin, int64_t n, Val<VB>* partials, unsigned* counter, Val<VB>* out, int* err) {
  Val<VB> v;
  c.init(&v);
  int64_t c0, c1;
  cta_share(n, &c0, &c1);
  int64_t i = c0 + threadIdx.x;
  if constexpr (has_walk<C>::value) {
    if (i < c1) {
      typename C::walk_state w;
      c.walk_start(w, begin + i);
      for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
          c.walk_exec(w, &v);
          c.walk_next(w);
        }
      }
      for (; i < c1; i += kBlock) {
        c.walk_exec(w, &v);
        c.walk_next(w);
      }
    }
  } else {
    for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) c.exec(begin + i + u * kBlock, &v);
    }
    for (; i < c1; i += kBlock) c.exec(begin + i, &v);
  }
  v = cta_reduce<VB>(c, v);
  report_abort(err);
  __shared__ unsigned s_ticket;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = v;
    __threadfence();
    s_ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (s_ticket != gridDim.x - 1) return;
  __threadfence();
  Val<VB> a;
  c.init(&a);
  // per-thread partials in CTA order, then the tree: the join is assumed
  // associative (as every Kokkos reducer is)
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    const Val<VB> p = ld_cg(partials + b);
    c.join(&a, &p);
  }
  a = cta_reduce<VB>(c, a);
  if (threadIdx.x == 0) {
    c.final_(&a);
    *out = a;
    *counter = 0u;
  }
}

// ---- parallel_scan --------------------------------------------------------
template <int VB>
struct ScanState {
  unsigned* flags;  // per tile: 0 = none, 1 = aggregate, 2 = inclusive prefix (cleared before the launch)
  Val<VB>* agg;
  Val<VB>* incl;
  unsigned* ticket;
  int* err;
  int64_t ntiles;
  int64_t wait_limit;
};

// Exclusive prefix of v over the lower lanes (in lane order), warp total.
template <int VB, class C>
__device__ Val<VB> warp_excl_scan(const C& c, Val<VB> v, Val<VB>* total) {
  const int lane = threadIdx.x & 31;
  Val<VB> inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    Val<VB> o = shfl_up(inc, d);
    if (lane >= d) {
      c.join(&o, &inc);  // o = o (earlier) + inc (later)
      inc = o;
    }
  }
  *total = shfl_idx(inc, 31);
  Val<VB> ex = shfl_up(inc, 1);
  if (lane == 0) c.init(&ex);
  return ex;
}

// total: where the grand total goes when non-null (ParallelScanWithTotal).
template <int VB, class C>
__global__ void __launch_bounds__(kBlock) k_scan(const C c, int64_t begin, int64_t n, ScanState<VB> S, Val<VB>* total) {
  constexpr int TILE = kBlock * kItems;
  constexpr int WARPS = kBlock / 32;
  __shared__ int64_t s_tile;
  __shared__ Val<VB> s_w[WARPS];
  __shared__ Val<VB> s_pre;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(S.ticket, 1u);
    if ((int64_t)t == S.ntiles - 1) *S.ticket = 0u;
    s_tile = t;
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t i0 = tile * TILE + (int64_t)threadIdx.x * kItems;
  const int64_t i1 = i0 + kItems < n ? i0 + kItems : n;
  Val<VB> part;
  c.init(&part);
  for (int64_t i = i0; i < i1; ++i) c.exec(begin + i, &part, false);
  Val<VB> wtot;
  const Val<VB> wex = warp_excl_scan<VB>(c, part, &wtot);
  if (lane == 0) s_w[warp] = wtot;
  __syncthreads();
  Val<VB> wpre, agg;
  c.init(&wpre);
  c.init(&agg);
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    if (w == warp) wpre = agg;
    c.join(&agg, &s_w[w]);
  }
  if (warp == 0) {
    Val<VB> excl;
    c.init(&excl);
    if (tile == 0) {
      if (lane == 0) {
        S.incl[0] = agg;
        __threadfence();
        st_release(S.flags, 2u);
      }
    } else {
      if (lane == 0) {
        S.agg[tile] = agg;
        __threadfence();
        st_release(S.flags + tile, 1u);
      }
      int64_t pt0 = tile - 1;
      bool gave_up = false;
      while (true) {
        const int64_t pt = pt0 - lane;
        unsigned fl = 2u;
        Val<VB> val;
        c.init(&val);
        if (pt >= 0) {
          int64_t polls = 0;
          while ((fl = ld_acquire(S.flags + pt)) == 0u) {
            if (++polls > S.wait_limit || gave_up) {
              fl = 2u;
              gave_up = true;
              break;
            }
            if (polls > 8) __nanosleep(128);
          }
          if (!gave_up) val = (fl == 2u) ? ld_volatile(S.incl + pt) : ld_volatile(S.agg + pt);
        }
        gave_up = __any_sync(0xffffffffu, gave_up);
        const unsigned pm = __ballot_sync(0xffffffffu, fl == 2u);
        const int last = pm ? __ffs(pm) - 1 : 31;
        // lane l holds tile pt0 - l: fold from the farthest to the nearest,
        // so lane 0 ends with the window's ordered total
        Val<VB> acc = val;
        if (lane > last) c.init(&acc);
#pragma unroll
        for (int m = 1; m < 32; m <<= 1) {
          Val<VB> o = shfl_down(acc, m);
          if (lane + m < 32) {
            c.join(&o, &acc);  // o (earlier tiles) + acc (later tiles)
            acc = o;
          }
        }
        c.join(&acc, &excl);  // the window precedes what was folded so far
        excl = acc;
        if (pm) break;
        pt0 -= 32;
      }
      if (lane == 0) {
        if (gave_up) atomicOr(S.err, 1);
        Val<VB> inc = excl;
        c.join(&inc, &agg);
        S.incl[tile] = inc;
        __threadfence();
        st_release(S.flags + tile, 2u);
      }
    }
    if (lane == 0) s_pre = excl;
  }
  __syncthreads();
  // this thread's exclusive prefix: tile prefix + earlier warps + earlier lanes
  Val<VB> pre = s_pre;
  if (total && tile == S.ntiles - 1 && threadIdx.x == 0) {
    Val<VB> t = pre;
    c.join(&t, &agg);
    *total = t;
  }
  c.join(&pre, &wpre);
  c.join(&pre, &wex);
  for (int64_t i = i0; i < i1; ++i) c.exec(begin + i, &pre, true);
  report_abort(S.err);
}

// ---- TeamPolicy: one CTA per team, league ranks strided over the grid ------
// The closure runs one team: exec_team(league_rank, league_size, shmem)
// (and an opaque value for the reduce).  shmem is the CTA's dynamic shared
// memory (the team's level-0 scratch).
template <class C>
__global__ void k_team_for(const C c, int64_t league, int* err) {
  extern __shared__ __align__(16) unsigned char team_shmem[];
  for (int64_t lr = blockIdx.x; lr < league; lr += gridDim.x) {
    c.exec_team(lr, league, team_shmem);
    __syncthreads();
  }
  report_abort(err);
}

template <int VB, class C>
__global__ void k_team_reduce(const C c, int64_t league, Val<VB>* partials, unsigned* counter, Val<VB>* out,
                              int* err) {
  extern __shared__ __align__(16) unsigned char team_shmem[];
  Val<VB> v;
  c.init(&v);
  for (int64_t lr = blockIdx.x; lr < league; lr += gridDim.x) {
    c.exec_team(lr, league, team_shmem, &v);
    __syncthreads();
  }
  v = cta_reduce_any<VB>(c, v);
  report_abort(err);
  __shared__ unsigned s_ticket;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = v;
    __threadfence();
    s_ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (s_ticket != gridDim.x - 1) return;
  __threadfence();
  Val<VB> a;
  c.init(&a);
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    const Val<VB> p = ld_cg(partials + b);
    c.join(&a, &p);
  }
  a = cta_reduce_any<VB>(c, a);
  if (threadIdx.x == 0) {
    c.final_(&a);
    *out = a;
    *counter = 0u;
  }
}

}  // namespace gbk_skel
