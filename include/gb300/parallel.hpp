// parallel_for / parallel_reduce over RangePolicy, MDRangePolicy and
// TeamPolicy for user functors, plus the nested TeamThreadRange /
// ThreadVectorRange patterns (core/src/Kokkos_Parallel.hpp,
// core/src/Kokkos_Parallel_Reduce.hpp:1684-1790; the reference's CUDA
// versions are core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp,
// Kokkos_Cuda_Parallel_MDRange.hpp, Kokkos_Cuda_Parallel_Team.hpp,
// Kokkos_Cuda_Team.hpp:517-810).
//
// Kernel shape (the library's flat-reduce skeleton, instantiated for the
// user's functor): a grid of at most SMs x 8 CTAs of 256 threads, each CTA
// owning one contiguous, equal share of the index space with its threads
// striding by 256 (coalesced for functors that read x(i)); a warp butterfly
// and a CTA tree of the reducer's join; the last CTA to take a ticket
// combines the per-CTA partials in CTA order — one launch, deterministic for
// a given device.  A host-scalar result is copied back and the space fenced
// (the reference's fence rule, Kokkos_Parallel_Reduce.hpp:1581-1640); a View
// result is written on the device without a fence.
#pragma once

#include <string>
#include <utility>

#include "reducers.hpp"

namespace gb300k {
namespace Impl {

constexpr int kBlock = 256;
constexpr int kSlotReduce = 32;  // library ticket slot used by header reduces

struct Scratch {
  char* base;
  unsigned* counters;
  int* err;
};
inline Scratch acquire(cudaStream_t s, size_t bytes) {
  void* p = nullptr;
  unsigned* c = nullptr;
  int* e = nullptr;
  check(gbk_workspace_acquire((gbk_stream_t)s, (int64_t)bytes, &p, &c, &e), "workspace");
  return {(char*)p, c, e};
}
inline int num_sms() {
  static int sm = 0;
  if (!sm) gbk_device_info(&sm, nullptr, nullptr, nullptr);
  return sm > 0 ? sm : 1;
}
inline void launched(cudaError_t e, const char* what) {
  check_cuda(e, what);
  gbk_note_launches(1);
}

template <class V>
__device__ V ld_cg(const V* p) {
  V r;
  const unsigned* s = reinterpret_cast<const unsigned*>(p);
  unsigned* d = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(V) / 4); ++i) d[i] = __ldcg(s + i);
  return r;
}

template <class Red, class V>
__device__ void grid_finish_obj(const Red& red, V acc, V* partials, unsigned* counter, V* out) {
  __shared__ __align__(16) unsigned char smraw[32 * sizeof(V)];
  __shared__ unsigned s_ticket;
  V* sm = reinterpret_cast<V*>(smraw);
  acc = block_reduce_obj(red, acc, sm);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    __threadfence();
    s_ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (s_ticket != gridDim.x - 1) return;
  __threadfence();
  V a;
  red.init(a);
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    V p = ld_cg(partials + i);
    red.join(a, p);
  }
  a = block_reduce_obj(red, a, sm);
  if (threadIdx.x == 0) {
    *out = a;
    *counter = 0u;
  }
}

__device__ inline void cta_share(int64_t n, int64_t* c0, int64_t* c1) {
  const int64_t per = n / gridDim.x, rem = n % gridDim.x, b = blockIdx.x;
  *c0 = b * per + (b < rem ? b : rem);
  *c1 = *c0 + per + (b < rem ? 1 : 0);
}

// ---- RangePolicy ------------------------------------------------------------
// Each thread takes kUnroll indices per step (kBlock apart), so that many
// independent loads of the functor are in flight per thread although the
// functor folds into one value.
constexpr int kUnroll = 4;
template <class F>
__global__ void __launch_bounds__(kBlock) k_range_for(F f, int64_t b, int64_t n) {
  int64_t c0, c1;
  cta_share(n, &c0, &c1);
  int64_t i = c0 + threadIdx.x;
  for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) f(b + i + u * kBlock);
  }
  for (; i < c1; i += kBlock) f(b + i);
}

template <class F, class Red, class V>
__global__ void __launch_bounds__(kBlock)
    k_range_reduce(F f, Red red, int64_t b, int64_t n, V* partials, unsigned* counter, V* out) {
  V v;
  red.init(v);
  int64_t c0, c1;
  cta_share(n, &c0, &c1);
  int64_t i = c0 + threadIdx.x;
  for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) f(b + i + u * kBlock, v);
  }
  for (; i < c1; i += kBlock) f(b + i, v);
  grid_finish_obj(red, v, partials, counter, out);
}

// ---- MDRangePolicy -------------------------------------------------------------
// The box is walked as one flat index space in which walk dimension 0 (the
// policy's inner direction: dimension 0 for Iterate::Left, the last for
// Right) varies fastest between consecutive threads, so a functor reading
// x(i0, ...) of a matching layout reads coalesced.  Each thread turns its
// first flat index into walk-order digits once (divisions) and then steps by
// the CTA width with a mixed-radix add of the step's digits (an add, a
// compare and a conditional subtract per dimension, no division per
// element).  The digit-to-argument order is fixed at compile time (LEFT).
struct MDArgs {
  int64_t lo[6];    // lower bounds, policy order
  int64_t ext[6];   // extents, walk order
  int64_t step[6];  // kBlock in the mixed radix of ext (walk order)
  bool fits32;      // every flat index below 2^31
};
template <class Tag, class F, class... A>
__device__ __forceinline__ void tag_call(const F& f, A&&... a) {
  if constexpr (std::is_void<Tag>::value) f(static_cast<A&&>(a)...);
  else f(Tag(), static_cast<A&&>(a)...);
}
template <int R, class IT>
struct MDWalk {
  IT d[R];  // walk-order digits of the current flat index
  __device__ __forceinline__ void start(const MDArgs& m, int64_t flat) {
    IT r = (IT)flat;
#pragma unroll
    for (int k = 0; k < R - 1; ++k) {
      const IT e = (IT)m.ext[k];
      d[k] = r % e;
      r /= e;
    }
    d[R - 1] = r;
  }
  __device__ __forceinline__ void advance(const MDArgs& m) {
    IT carry = 0;
#pragma unroll
    for (int k = 0; k < R - 1; ++k) {
      const IT v = d[k] + (IT)m.step[k] + carry;
      const IT e = (IT)m.ext[k];
      carry = v >= e ? IT(1) : IT(0);
      d[k] = carry ? v - e : v;
    }
    d[R - 1] += (IT)m.step[R - 1] + carry;
  }
  // policy-order argument p from the walk digits
  template <bool LEFT, int P>
  __device__ __forceinline__ int64_t arg(const MDArgs& m) const {
    return m.lo[P] + (int64_t)d[LEFT ? P : R - 1 - P];
  }
};
template <int R, bool LEFT, class Tag, class IT, class F, class... A>
__device__ __forceinline__ void md_call(const F& f, const MDArgs& m, const MDWalk<R, IT>& w, A&... a) {
  if constexpr (R == 2) tag_call<Tag>(f, w.template arg<LEFT, 0>(m), w.template arg<LEFT, 1>(m), a...);
  else if constexpr (R == 3)
    tag_call<Tag>(f, w.template arg<LEFT, 0>(m), w.template arg<LEFT, 1>(m), w.template arg<LEFT, 2>(m), a...);
  else if constexpr (R == 4)
    tag_call<Tag>(f, w.template arg<LEFT, 0>(m), w.template arg<LEFT, 1>(m), w.template arg<LEFT, 2>(m),
                  w.template arg<LEFT, 3>(m), a...);
  else if constexpr (R == 5)
    tag_call<Tag>(f, w.template arg<LEFT, 0>(m), w.template arg<LEFT, 1>(m), w.template arg<LEFT, 2>(m),
                  w.template arg<LEFT, 3>(m), w.template arg<LEFT, 4>(m), a...);
  else
    tag_call<Tag>(f, w.template arg<LEFT, 0>(m), w.template arg<LEFT, 1>(m), w.template arg<LEFT, 2>(m),
                  w.template arg<LEFT, 3>(m), w.template arg<LEFT, 4>(m), w.template arg<LEFT, 5>(m), a...);
}
// Walk [c0, c1) of the flat space in steps of kBlock from c0 + threadIdx.x,
// kUnroll steps per loop trip (their loads independent of one another).
template <int R, bool LEFT, class Tag, class IT, class F, class... A>
__device__ __forceinline__ void md_walk(const F& f, const MDArgs& m, int64_t c0, int64_t c1, A&... a) {
  int64_t i = c0 + threadIdx.x;
  if (i >= c1) return;
  MDWalk<R, IT> w;
  w.start(m, i);
  for (; i + (kUnroll - 1) * kBlock < c1; i += kUnroll * kBlock) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      md_call<R, LEFT, Tag>(f, m, w, a...);
      w.advance(m);
    }
  }
  for (; i < c1; i += kBlock) {
    md_call<R, LEFT, Tag>(f, m, w, a...);
    w.advance(m);
  }
}
template <int R, bool LEFT, class Tag, class IT, class F>
__global__ void __launch_bounds__(kBlock) k_md_for(F f, MDArgs m, int64_t n) {
  int64_t c0, c1;
  cta_share(n, &c0, &c1);
  md_walk<R, LEFT, Tag, IT>(f, m, c0, c1);
}
template <int R, bool LEFT, class Tag, class IT, class F, class Red, class V>
__global__ void __launch_bounds__(kBlock)
    k_md_reduce(F f, Red red, MDArgs m, int64_t n, V* partials, unsigned* counter, V* out) {
  V v;
  red.init(v);
  int64_t c0, c1;
  cta_share(n, &c0, &c1);
  md_walk<R, LEFT, Tag, IT>(f, m, c0, c1, v);
  grid_finish_obj(red, v, partials, counter, out);
}
template <class P>
MDArgs md_args(const P& p, int64_t* total) {
  constexpr int R = P::rank;
  constexpr bool left = P::inner_direction == Iterate::Left;
  MDArgs m{};
  int64_t n = 1;
  for (int d = 0; d < R; ++d) {
    const int pd = left ? d : R - 1 - d;
    m.lo[d] = p.lower(d);
    m.ext[d] = p.upper(pd) - p.lower(pd);
    n *= m.ext[d] > 0 ? m.ext[d] : 0;
  }
  // kBlock written in the mixed radix of the walk extents
  int64_t r = kBlock;
  for (int d = 0; d < R - 1; ++d) {
    const int64_t e = m.ext[d] > 0 ? m.ext[d] : 1;
    m.step[d] = r % e;
    r /= e;
  }
  m.step[R - 1] = r;
  m.fits32 = n + 2 * kUnroll * kBlock < (int64_t(1) << 31);
  *total = n;
  return m;
}

// ---- TeamPolicy: one CTA per team, league ranks strided over the grid ----------
constexpr int64_t kTeamGridMax = int64_t(1) << 20;
constexpr int64_t kTeamReduceGridMax = int64_t(1) << 16;
template <class F>
__global__ void k_team_for(F f, int64_t league) {
  for (int64_t lr = blockIdx.x; lr < league; lr += gridDim.x) {
    TeamMember m(lr, league);
    f(m);
    __syncthreads();
  }
}
template <class F, class Red, class V>
__global__ void k_team_reduce(F f, Red red, int64_t league, V* partials, unsigned* counter, V* out) {
  V v;
  red.init(v);
  for (int64_t lr = blockIdx.x; lr < league; lr += gridDim.x) {
    TeamMember m(lr, league);
    f(m, v);
    __syncthreads();
  }
  grid_finish_obj(red, v, partials, counter, out);
}

// Run a reduce kernel and deliver the result.
template <class Red, class Launch>
void run_reduce(cudaStream_t s, int64_t grid, const Red& red, Launch launch) {
  using V = typename Red::value_type;
  Scratch sc = acquire(s, 256 + (size_t)grid * sizeof(V) + 256);
  V* dev_out = red.res.device ? red.res.ptr : reinterpret_cast<V*>(sc.base);
  V* partials = reinterpret_cast<V*>(sc.base + 256);
  launched(launch(partials, sc.counters + kSlotReduce, dev_out), "parallel_reduce");
  if (!red.res.device) {
    if (sizeof(V) <= 256) {  // through the workspace's pinned slot: one synchronisation
      check(gbk_fence_read((gbk_stream_t)s, dev_out, red.res.ptr, (int64_t)sizeof(V)), "parallel_reduce");
    } else {
      check_cuda(cudaMemcpyAsync(red.res.ptr, dev_out, sizeof(V), cudaMemcpyDeviceToHost, s), "parallel_reduce");
      check(gbk_stream_check((gbk_stream_t)s), "parallel_reduce");
    }
  }
}

inline int64_t grid_for(int64_t n) {
  int64_t g = (n + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (g > cap) g = cap;
  return g < 1 ? 1 : g;
}

template <class T>
struct AsReducer {
  using type = Sum<T>;
  static Sum<T> make(T& r) { return Sum<T>(r); }
};

}  // namespace Impl

// ---- parallel_for ------------------------------------------------------------
template <class E, class... R, class F>
void parallel_for(const RangePolicy<E, R...>& p, const F& f) {
  Tools::Impl::Region<F> tool_region(Tools::Impl::kFor, p.space().stream());
  const int64_t n = p.end() - p.begin();
  if (n <= 0) return;
  const int64_t g = Impl::grid_for(n);
  Impl::k_range_for<<<(unsigned)g, Impl::kBlock, 0, p.space().stream()>>>(f, p.begin(), n);
  Impl::launched(cudaGetLastError(), "parallel_for");
}
template <class F>
void parallel_for(int64_t n, const F& f) {
  parallel_for(RangePolicy<>(0, n), f);
}
template <class... PP, class F>
void parallel_for(const MDRangePolicy<PP...>& p, const F& f) {
  using P = MDRangePolicy<PP...>;
  Tools::Impl::Region<F> tool_region(Tools::Impl::kFor, p.space().stream());
  int64_t n = 0;
  const Impl::MDArgs m = Impl::md_args(p, &n);
  if (n <= 0) return;
  constexpr bool left = P::inner_direction == Iterate::Left;
  const unsigned g = (unsigned)Impl::grid_for(n);
  if (m.fits32)
    Impl::k_md_for<P::rank, left, typename P::work_tag, int32_t><<<g, Impl::kBlock, 0, p.space().stream()>>>(f, m, n);
  else
    Impl::k_md_for<P::rank, left, typename P::work_tag, int64_t><<<g, Impl::kBlock, 0, p.space().stream()>>>(f, m, n);
  Impl::launched(cudaGetLastError(), "parallel_for(MDRange)");
}
template <class E, class... R, class F>
void parallel_for(const TeamPolicy<E, R...>& p, const F& f) {
  Tools::Impl::Region<F> tool_region(Tools::Impl::kFor, p.space().stream());
  if (p.league_size() <= 0) return;
  // One CTA per league rank (up to 2^20 CTAs, then each strides): the block
  // scheduler hands the next team to whichever SM frees up first, so a long
  // team does not hold back the teams that would have followed it on its CTA.
  int64_t g = p.league_size();
  if (g > Impl::kTeamGridMax) g = Impl::kTeamGridMax;
  Impl::k_team_for<<<(unsigned)g, p.team_size(), 0, p.space().stream()>>>(f, p.league_size());
  Impl::launched(cudaGetLastError(), "parallel_for(TeamPolicy)");
}
template <class P, class F>
void parallel_for(const std::string& label, const P& p, const F& f) {
  Tools::Impl::LabelScope ls(label);
  parallel_for(p, f);
}

// ---- parallel_reduce -----------------------------------------------------------
template <class E, class... R, class F, class Red,
          std::enable_if_t<Impl::is_reducer<Red>::value, bool> = true>
void parallel_reduce(const RangePolicy<E, R...>& p, const F& f, const Red& red) {
  Tools::Impl::Region<F> tool_region(Tools::Impl::kReduce, p.space().stream());
  using V = typename Red::value_type;
  const int64_t n = p.end() - p.begin();
  const int64_t g = Impl::grid_for(n);
  cudaStream_t s = p.space().stream();
  const int64_t b = p.begin();
  Impl::run_reduce(s, g, red, [&](V* part, unsigned* ctr, V* out) {
    Impl::k_range_reduce<<<(unsigned)g, Impl::kBlock, 0, s>>>(f, red, b, n, part, ctr, out);
    return cudaGetLastError();
  });
}
template <class... PP, class F, class Red, std::enable_if_t<Impl::is_reducer<Red>::value, bool> = true>
void parallel_reduce(const MDRangePolicy<PP...>& p, const F& f, const Red& red) {
  using P = MDRangePolicy<PP...>;
  Tools::Impl::Region<F> tool_region(Tools::Impl::kReduce, p.space().stream());
  using V = typename Red::value_type;
  int64_t n = 0;
  const Impl::MDArgs m = Impl::md_args(p, &n);
  const int64_t g = Impl::grid_for(n);
  cudaStream_t s = p.space().stream();
  constexpr bool left = P::inner_direction == Iterate::Left;
  Impl::run_reduce(s, g, red, [&](V* part, unsigned* ctr, V* out) {
    if (m.fits32)
      Impl::k_md_reduce<P::rank, left, typename P::work_tag, int32_t>
          <<<(unsigned)g, Impl::kBlock, 0, s>>>(f, red, m, n, part, ctr, out);
    else
      Impl::k_md_reduce<P::rank, left, typename P::work_tag, int64_t>
          <<<(unsigned)g, Impl::kBlock, 0, s>>>(f, red, m, n, part, ctr, out);
    return cudaGetLastError();
  });
}
template <class E, class... R, class F, class Red, std::enable_if_t<Impl::is_reducer<Red>::value, bool> = true>
void parallel_reduce(const TeamPolicy<E, R...>& p, const F& f, const Red& red) {
  Tools::Impl::Region<F> tool_region(Tools::Impl::kReduce, p.space().stream());
  using V = typename Red::value_type;
  // one CTA per league rank, as parallel_for; at most 2^16 per-CTA partials
  int64_t g = p.league_size();
  if (g > Impl::kTeamReduceGridMax) g = Impl::kTeamReduceGridMax;
  if (g < 1) g = 1;
  cudaStream_t s = p.space().stream();
  const int64_t league = p.league_size();
  const int ts = p.team_size();
  Impl::run_reduce(s, g, red, [&](V* part, unsigned* ctr, V* out) {
    Impl::k_team_reduce<<<(unsigned)g, ts, 0, s>>>(f, red, league, part, ctr, out);
    return cudaGetLastError();
  });
}
namespace Impl {
template <class P> struct is_policy : std::false_type {};
template <class E, class... R> struct is_policy<RangePolicy<E, R...>> : std::true_type {};
template <class... PP> struct is_policy<MDRangePolicy<PP...>> : std::true_type {};
template <class E, class... R> struct is_policy<TeamPolicy<E, R...>> : std::true_type {};
}  // namespace Impl

// Scalar result: a Sum into a host variable.
template <class P, class F, class T,
          std::enable_if_t<std::is_arithmetic<T>::value && Impl::is_policy<P>::value, bool> = true>
void parallel_reduce(const P& p, const F& f, T& result) {
  parallel_reduce(p, f, Sum<T>(result));
}
template <class F, class T, std::enable_if_t<std::is_arithmetic<T>::value, bool> = true>
void parallel_reduce(int64_t n, const F& f, T& result) {
  parallel_reduce(RangePolicy<>(0, n), f, Sum<T>(result));
}
template <class F, class Red, std::enable_if_t<Impl::is_reducer<Red>::value, bool> = true>
void parallel_reduce(int64_t n, const F& f, const Red& red) {
  parallel_reduce(RangePolicy<>(0, n), f, red);
}
template <class P, class F, class T>
void parallel_reduce(const std::string& label, const P& p, const F& f, T&& result) {
  Tools::Impl::LabelScope ls(label);
  parallel_reduce(p, f, std::forward<T>(result));
}

// ---- several reducers in one pass ----------------------------------------------
// parallel_reduce(policy, f, r0, r1, ...) (core/src/impl/Kokkos_Combined_Reducer.hpp:
// 533-620): the functor takes one value per reducer, f(i..., v0, v1, ...), and
// every result is delivered to its own reducer's target; a plain arithmetic
// result stands for a Sum into it.  The values travel through the kernels as
// one packed value, joined component-wise.
namespace Impl {
template <class... V> struct VPack;
template <class V0> struct VPack<V0> { V0 head; };
template <class V0, class V1, class... Vs> struct VPack<V0, V1, Vs...> {
  V0 head;
  VPack<V1, Vs...> tail;
};
template <size_t K> struct PackGet {
  template <class P> __host__ __device__ static auto& get(P& p) { return PackGet<K - 1>::get(p.tail); }
};
template <> struct PackGet<0> {
  template <class P> __host__ __device__ static auto& get(P& p) { return p.head; }
};

template <class... R> struct RPack;
template <class R0> struct RPack<R0> {
  R0 head;
  using value_type = VPack<typename R0::value_type>;
  __device__ void init(value_type& v) const { head.init(v.head); }
  __device__ void join(value_type& a, const value_type& b) const { head.join(a.head, b.head); }
};
template <class R0, class R1, class... Rs> struct RPack<R0, R1, Rs...> {
  R0 head;
  RPack<R1, Rs...> tail;
  using value_type = VPack<typename R0::value_type, typename R1::value_type, typename Rs::value_type...>;
  __device__ void init(value_type& v) const {
    head.init(v.head);
    tail.init(v.tail);
  }
  __device__ void join(value_type& a, const value_type& b) const {
    head.join(a.head, b.head);
    tail.join(a.tail, b.tail);
  }
};
template <class R0> RPack<R0> make_rpack(const R0& r0) { return RPack<R0>{r0}; }
template <class R0, class R1, class... Rs>
RPack<R0, R1, Rs...> make_rpack(const R0& r0, const R1& r1, const Rs&... rs) {
  return RPack<R0, R1, Rs...>{r0, make_rpack(r1, rs...)};
}

template <class... Rs>
struct CombinedReducer {
  using reducer = CombinedReducer;
  using value_type = VPack<typename Rs::value_type...>;
  RPack<Rs...> reds;
  ResultRef<value_type> res;
  __device__ void init(value_type& v) const { reds.init(v); }
  __device__ void join(value_type& a, const value_type& b) const { reds.join(a, b); }
};

// The user functor seen through the packed value: one overload per policy kind.
template <class F, class VP, size_t... Is>
struct CombinedFunctor {
  F f;
  __device__ void operator()(int64_t i, VP& v) const { f(i, PackGet<Is>::get(v)...); }
  __device__ void operator()(int64_t i, int64_t j, VP& v) const { f(i, j, PackGet<Is>::get(v)...); }
  __device__ void operator()(int64_t i, int64_t j, int64_t k, VP& v) const { f(i, j, k, PackGet<Is>::get(v)...); }
  __device__ void operator()(int64_t i, int64_t j, int64_t k, int64_t l, VP& v) const {
    f(i, j, k, l, PackGet<Is>::get(v)...);
  }
  __device__ void operator()(int64_t i, int64_t j, int64_t k, int64_t l, int64_t m, VP& v) const {
    f(i, j, k, l, m, PackGet<Is>::get(v)...);
  }
  __device__ void operator()(int64_t i, int64_t j, int64_t k, int64_t l, int64_t m, int64_t q, VP& v) const {
    f(i, j, k, l, m, q, PackGet<Is>::get(v)...);
  }
  __device__ void operator()(const TeamMember& m, VP& v) const { f(m, PackGet<Is>::get(v)...); }
};

template <class A, std::enable_if_t<is_reducer<std::decay_t<A>>::value, bool> = true>
std::decay_t<A> as_reducer(A&& a) {
  return a;
}
template <class T, std::enable_if_t<std::is_arithmetic<T>::value, bool> = true>
Sum<T> as_reducer(T& a) {
  return Sum<T>(a);
}
template <class D, class... P>
Sum<typename View<D, P...>::non_const_value_type> as_reducer(const View<D, P...>& v) {  // a View result: its first element
  return Sum<typename View<D, P...>::non_const_value_type>(v);
}

template <class R>
void deliver(const R& r, const typename R::value_type& v, cudaStream_t s) {
  if (r.res.device) {
    check_cuda(cudaMemcpyAsync(r.res.ptr, &v, sizeof(v), cudaMemcpyHostToDevice, s), "parallel_reduce");
    check_cuda(cudaStreamSynchronize(s), "parallel_reduce");
  } else {
    *r.res.ptr = v;
  }
}

template <class P, class F, size_t... Is, class... Rs>
void combined_reduce(const P& p, const F& f, std::index_sequence<Is...>, const Rs&... rs) {
  using VP = VPack<typename Rs::value_type...>;
  VP host_val{};
  CombinedReducer<Rs...> cr{make_rpack(rs...), ResultRef<VP>{&host_val, false}};
  parallel_reduce(p, CombinedFunctor<F, VP, Is...>{f}, cr);
  (deliver(rs, PackGet<Is>::get(host_val), p.space().stream()), ...);
}
}  // namespace Impl

template <class P, class F, class A0, class A1, class... As, std::enable_if_t<Impl::is_policy<P>::value, bool> = true>
void parallel_reduce(const P& p, const F& f, A0&& a0, A1&& a1, As&&... as) {
  Impl::combined_reduce(p, f, std::make_index_sequence<2 + sizeof...(As)>{}, Impl::as_reducer(a0),
                        Impl::as_reducer(a1), Impl::as_reducer(as)...);
}
template <class P, class F, class A0, class A1, class... As, std::enable_if_t<Impl::is_policy<P>::value, bool> = true>
void parallel_reduce(const std::string& label, const P& p, const F& f, A0&& a0, A1&& a1, As&&... as) {
  Tools::Impl::LabelScope ls(label);
  parallel_reduce(p, f, std::forward<A0>(a0), std::forward<A1>(a1), std::forward<As>(as)...);
}
// ... and over [0, n) (Kokkos_Combined_Reducer.hpp:597-620)
template <class N, class F, class A0, class A1, class... As, std::enable_if_t<std::is_integral<N>::value, bool> = true>
void parallel_reduce(N n, const F& f, A0&& a0, A1&& a1, As&&... as) {
  parallel_reduce(RangePolicy<>(0, (int64_t)n), f, std::forward<A0>(a0), std::forward<A1>(a1), std::forward<As>(as)...);
}
template <class N, class F, class A0, class A1, class... As, std::enable_if_t<std::is_integral<N>::value, bool> = true>
void parallel_reduce(const std::string& label, N n, const F& f, A0&& a0, A1&& a1, As&&... as) {
  Tools::Impl::LabelScope ls(label);
  parallel_reduce(RangePolicy<>(0, (int64_t)n), f, std::forward<A0>(a0), std::forward<A1>(a1), std::forward<As>(as)...);
}

// ---- nested patterns inside a TeamPolicy functor ---------------------------------
// (host-device because they are called from KOKKOS_LAMBDA bodies; they only
// do work in device code)
// A team thread takes indices team_rank, team_rank + team_size, ... of the
// range, 32 of them per loop trip while that many remain, then 8, then one
// at a time, so that up to 32 loads of the functor are in flight (calls
// stay in increasing index order per thread).  One team per league rank
// makes the longest range the league's tail: one CTA streams it alone, and
// its rate is the bytes it keeps in flight.
template <int U, class F, class... A>
__device__ __forceinline__ void team_range_steps(int64_t& i, int64_t e, int64_t step, const F& f, A&... a) {
  for (; i + (U - 1) * step < e; i += U * step) {
#pragma unroll
    for (int u = 0; u < U; ++u) f(i + u * step, a...);
  }
}
template <class F, class... A>
__device__ __forceinline__ void team_range_walk(int64_t b, int64_t e, int64_t step, const F& f, A&... a) {
  int64_t i = b;
  team_range_steps<32>(i, e, step, f, a...);
  team_range_steps<8>(i, e, step, f, a...);
  for (; i < e; i += step) f(i, a...);
}
template <class F>
KOKKOS_INLINE_FUNCTION void parallel_for(const TeamThreadRangeBoundaries<>& r, const F& f) {
#ifdef __CUDA_ARCH__
  team_range_walk(r.begin + r.member.team_rank(), r.end, (int64_t)r.member.team_size(), f);
#endif
}

namespace Impl {
// Team-wide join of every thread's value; the result reaches all threads.
template <class Red, class V>
__device__ V team_allreduce(const Red& red, V v) {
  __shared__ __align__(16) unsigned char raw[33 * sizeof(V)];
  V* sm = reinterpret_cast<V*>(raw);
  v = block_reduce_obj(red, v, sm);
  if (threadIdx.x == 0) sm[32] = v;
  __syncthreads();
  v = sm[32];
  __syncthreads();
  return v;
}
// Every thread receives the root thread's value.
template <class T>
__device__ void team_bcast(T& v, int root) {
  __shared__ __align__(16) unsigned char raw[sizeof(T)];
  __syncthreads();  // earlier readers of raw are done
  if ((int)threadIdx.x == root) *reinterpret_cast<T*>(raw) = v;
  __syncthreads();
  v = *reinterpret_cast<T*>(raw);
}
template <class T>
struct DevSum {
  using value_type = T;
  __device__ void init(T& v) const { v = T(0); }
  __device__ void join(T& a, const T& b) const { a += b; }
};
}  // namespace Impl

template <class F, class T, std::enable_if_t<std::is_arithmetic<T>::value, bool> = true>
KOKKOS_INLINE_FUNCTION void parallel_reduce(const TeamThreadRangeBoundaries<>& r, const F& f, T& result) {
#ifdef __CUDA_ARCH__
  T v = T(0);
  team_range_walk(r.begin + r.member.team_rank(), r.end, (int64_t)r.member.team_size(), f, v);
  result = Impl::team_allreduce(Impl::DevSum<T>{}, v);
#endif
}
template <class F, class Red, std::enable_if_t<Impl::is_reducer<Red>::value, bool> = true>
KOKKOS_INLINE_FUNCTION void parallel_reduce(const TeamThreadRangeBoundaries<>& r, const F& f, const Red& red) {
#ifdef __CUDA_ARCH__
  typename Red::value_type v;
  red.init(v);
  team_range_walk(r.begin + r.member.team_rank(), r.end, (int64_t)r.member.team_size(), f, v);
  red.reference() = Impl::team_allreduce(red, v);
#endif
}

// ThreadVectorRange: vector length 1 in this mapping (a team thread runs the
// range itself).
struct ThreadVectorRangeBoundaries {
  int64_t begin, end;
};
KOKKOS_INLINE_FUNCTION ThreadVectorRangeBoundaries ThreadVectorRange(const TeamMember&, int64_t n) { return {0, n}; }
KOKKOS_INLINE_FUNCTION ThreadVectorRangeBoundaries ThreadVectorRange(const TeamMember&, int64_t b, int64_t e) {
  return {b, e};
}
template <class F>
KOKKOS_INLINE_FUNCTION void parallel_for(const ThreadVectorRangeBoundaries& r, const F& f) {
  for (int64_t i = r.begin; i < r.end; ++i) f(i);
}
template <class F, class T, std::enable_if_t<!Impl::is_reducer<T>::value, bool> = true>
KOKKOS_INLINE_FUNCTION void parallel_reduce(const ThreadVectorRangeBoundaries& r, const F& f, T& result) {
  T v = T(0);
  for (int64_t i = r.begin; i < r.end; ++i) f(i, v);
  result = v;
}
template <class F, class Red, std::enable_if_t<Impl::is_reducer<Red>::value, bool> = true>
KOKKOS_INLINE_FUNCTION void parallel_reduce(const ThreadVectorRangeBoundaries& r, const F& f, const Red& red) {
#ifdef __CUDA_ARCH__
  typename Red::value_type v;
  red.init(v);
  for (int64_t i = r.begin; i < r.end; ++i) f(i, v);
  red.reference() = v;
#endif
}

}  // namespace gb300k
