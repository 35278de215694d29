// ParallelFor / ParallelReduce over an MDRangePolicy on the GB300 space
// (the CUDA space's versions: core/src/Cuda/Kokkos_Cuda_Parallel_MDRange.hpp:
// 45-497 with impl/KokkosExp_IterateTileGPU.hpp, one element per thread per
// tile and a grid of at most the block size in CTAs).
//
// Here the box [lower, upper) of rank 1..6 is walked as one flat index space
// on the skeleton kernels of Kokkos_GB300_Skeletons.hpp (through their walk
// protocol: each thread keeps its multi-index and steps it): the policy's inner
// iteration direction is the fastest-varying dimension across consecutive
// threads (Iterate::Left, the default on this space as on the CUDA space:
// dimension 0 fastest, which coalesces LayoutLeft views; Iterate::Right:
// the last dimension fastest, for LayoutRight views), the outer direction
// orders the remaining dimensions the same way.  The policy's tile sizes are
// accepted and checked by the policy itself; they do not change this walk
// (every tile shape covers the same elements, and a flat walk keeps each
// warp on consecutive addresses of the fastest dimension).
#ifndef KOKKOS_GB300_PARALLEL_MDRANGE_HPP_
#define KOKKOS_GB300_PARALLEL_MDRANGE_HPP_

#include <Kokkos_Macros.hpp>
#if defined(KOKKOS_ENABLE_GB300)

#include <KokkosExp_MDRangePolicy.hpp>

#include <GB300/Kokkos_GB300_Parallel_Range.hpp>

namespace Kokkos {

template <>
struct default_outer_direction<Kokkos::Experimental::GB300> {
  using type = Iterate;
  static constexpr Iterate value = Iterate::Left;
};
template <>
struct default_inner_direction<Kokkos::Experimental::GB300> {
  using type = Iterate;
  static constexpr Iterate value = Iterate::Left;
};

namespace Impl {

template <>
inline TileSizeProperties get_tile_size_properties<Kokkos::Experimental::GB300>(const Kokkos::Experimental::GB300&) {
  TileSizeProperties p;
  p.max_threads = 1024;
  p.default_largest_tile_size = 16;
  p.default_tile_size = 2;
  p.max_total_tile_size = 1024;
  return p;
}

// The box of an MDRangePolicy as the kernels see it: lower bounds in policy
// order, extents in walk order (walk dimension 0 fastest), and the CTA width
// (kBlock) written in the mixed radix of the extents.  A thread turns its
// first flat index into walk digits once (divisions), then steps by kBlock
// with a mixed-radix add (an add, a compare and a conditional subtract per
// dimension) instead of dividing for every element.
template <int R>
struct GB300Box {
  int64_t lo[R];
  int64_t ext[R];
  int64_t step[R];
  bool fits32;  // every flat index (and the walk's overshoot) below 2^31
};

// Walk digits; LEFT: walk dimension d is policy dimension d, else R - 1 - d.
template <int R, bool LEFT, class IT>
struct GB300Walk {
  IT d[R];
  __device__ __forceinline__ void start(const GB300Box<R>& b, int64_t flat) {
    IT r = (IT)flat;
#pragma unroll
    for (int k = 0; k < R - 1; ++k) {
      const IT e = (IT)b.ext[k];
      d[k] = r % e;
      r /= e;
    }
    d[R - 1] = r;
  }
  __device__ __forceinline__ void next(const GB300Box<R>& b) {
    IT carry = 0;
#pragma unroll
    for (int k = 0; k < R - 1; ++k) {
      const IT v = d[k] + (IT)b.step[k] + carry;
      const IT e = (IT)b.ext[k];
      carry = v >= e ? IT(1) : IT(0);
      d[k] = carry ? v - e : v;
    }
    d[R - 1] += (IT)b.step[R - 1] + carry;
  }
  template <class Index>
  __device__ __forceinline__ void point(const GB300Box<R>& b, Index (&i)[R]) const {
#pragma unroll
    for (int p = 0; p < R; ++p) i[p] = (Index)(b.lo[p] + (int64_t)d[LEFT ? p : R - 1 - p]);
  }
};

template <class MDPolicy, int R = MDPolicy::rank>
GB300Box<R> gb300_box(const MDPolicy& p, int64_t* total) {
  // Left: dimension 0 fastest; Right: dimension R-1 fastest.  The outer
  // direction of the reference orders tiles, which a flat walk does not have;
  // the inner direction alone sets the element order here.
  constexpr bool left = MDPolicy::inner_direction == Iterate::Left;
  GB300Box<R> b{};
  int64_t n = 1;
  for (int d = 0; d < R; ++d) {
    const int pd = left ? d : R - 1 - d;
    b.lo[d] = (int64_t)p.m_lower[d];
    const int64_t e = (int64_t)p.m_upper[pd] - (int64_t)p.m_lower[pd];
    b.ext[d] = e > 0 ? e : 0;
    n *= (e > 0 ? e : 0);
  }
  int64_t r = gbk_skel::kBlock;
  for (int d = 0; d < R - 1; ++d) {
    const int64_t e = b.ext[d] > 0 ? b.ext[d] : 1;
    b.step[d] = r % e;
    r /= e;
  }
  b.step[R - 1] = r;
  b.fits32 = n + 2 * gbk_skel::kUnroll * gbk_skel::kBlock < (int64_t(1) << 31);
  *total = n;
  return b;
}

// functor(i0, ..., iR-1 [, update]) with an optional work tag
template <class WorkTag, int R, class F, class Index, class... U>
__device__ __forceinline__ void gb300_md_call(const F& f, const Index (&i)[R], U&&... u) {
  if constexpr (R == 1) gb300_call<WorkTag>(f, i[0], static_cast<U&&>(u)...);
  else if constexpr (R == 2) gb300_call<WorkTag>(f, i[0], i[1], static_cast<U&&>(u)...);
  else if constexpr (R == 3) gb300_call<WorkTag>(f, i[0], i[1], i[2], static_cast<U&&>(u)...);
  else if constexpr (R == 4) gb300_call<WorkTag>(f, i[0], i[1], i[2], i[3], static_cast<U&&>(u)...);
  else if constexpr (R == 5) gb300_call<WorkTag>(f, i[0], i[1], i[2], i[3], i[4], static_cast<U&&>(u)...);
  else gb300_call<WorkTag>(f, i[0], i[1], i[2], i[3], i[4], i[5], static_cast<U&&>(u)...);
}

template <class FunctorType, class... Traits>
class ParallelFor<FunctorType, Kokkos::MDRangePolicy<Traits...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::MDRangePolicy<Traits...>;
  using functor_type = FunctorType;

 private:
  using WorkTag = typename Policy::work_tag;
  using Index = typename Policy::index_type;
  static constexpr int R = Policy::rank;
  const FunctorType m_functor;
  const Policy m_policy;

 public:
  static constexpr bool kLeft = Policy::inner_direction == Iterate::Left;
  template <class IT>
  struct Closure {
    FunctorType f;
    GB300Box<R> box;
    using walk_state = GB300Walk<R, kLeft, IT>;
    __device__ void walk_start(walk_state& w, int64_t flat) const { w.start(box, flat); }
    __device__ void walk_next(walk_state& w) const { w.next(box); }
    __device__ void walk_exec(const walk_state& w) const {
      Index i[R];
      w.point(box, i);
      gb300_md_call<WorkTag, R>(f, i);
    }
  };

  Policy const& get_policy() const { return m_policy; }
  ParallelFor(const FunctorType& arg_functor, const Policy& arg_policy)
      : m_functor(arg_functor), m_policy(arg_policy) {}

  template <typename P, typename F>
  static int max_tile_size_product(const P&, const F&) {
    return 1024;
  }

  void execute() const {
    int64_t n = 0;
    const auto box = gb300_box<Policy>(m_policy, &n);
    if (n <= 0) return;
    const auto& exec = m_policy.space();
    const int64_t g = gb300_grid(exec, n);
    int* err = gb300_scratch(exec, 0).err;
    if (box.fits32)
      gbk_skel::k_for<Closure<int32_t>>
          <<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(Closure<int32_t>{m_functor, box}, 0, n, err);
    else
      gbk_skel::k_for<Closure<int64_t>>
          <<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(Closure<int64_t>{m_functor, box}, 0, n, err);
    gb300_launched("parallel_for(MDRangePolicy)");
  }
};

template <class CombinedFunctorReducerType, class... Traits>
class ParallelReduce<CombinedFunctorReducerType, Kokkos::MDRangePolicy<Traits...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::MDRangePolicy<Traits...>;
  using FunctorType = typename CombinedFunctorReducerType::functor_type;
  using ReducerType = typename CombinedFunctorReducerType::reducer_type;
  using pointer_type = typename ReducerType::pointer_type;
  using value_type = typename ReducerType::value_type;
  using reference_type = typename ReducerType::reference_type;
  using functor_type = FunctorType;
  using reducer_type = ReducerType;

 private:
  using WorkTag = typename Policy::work_tag;
  using Index = typename Policy::index_type;
  static constexpr int R = Policy::rank;
  const CombinedFunctorReducerType m_functor_reducer;
  const Policy m_policy;
  const pointer_type m_result_ptr;
  const bool m_result_ptr_device_accessible;

 public:
  static constexpr bool kLeft = Policy::inner_direction == Iterate::Left;
  template <class IT>
  struct Closure : GB300ValueOps<ReducerType> {
    FunctorType f;
    GB300Box<R> box;
    using walk_state = GB300Walk<R, kLeft, IT>;
    __device__ void walk_start(walk_state& w, int64_t flat) const { w.start(box, flat); }
    __device__ void walk_next(walk_state& w) const { w.next(box); }
    __device__ void walk_exec(const walk_state& w, void* v) const {
      Index i[R];
      w.point(box, i);
      gb300_md_call<WorkTag, R>(f, i, this->r.reference(static_cast<pointer_type>(v)));
    }
  };

  Policy const& get_policy() const { return m_policy; }

  template <class ViewType>
  ParallelReduce(const CombinedFunctorReducerType& arg_functor_reducer, const Policy& arg_policy,
                 const ViewType& arg_result)
      : m_functor_reducer(arg_functor_reducer),
        m_policy(arg_policy),
        m_result_ptr(arg_result.data()),
        m_result_ptr_device_accessible(
            MemorySpaceAccess<Kokkos::Experimental::GB300Space, typename ViewType::memory_space>::accessible) {}

  template <typename P, typename F>
  static int max_tile_size_product(const P&, const F&) {
    return 1024;
  }

  void execute() const {
    constexpr int VB = gb300_value_bytes<ReducerType>();
    int64_t n = 0;
    const auto box = gb300_box<Policy>(m_policy, &n);
    const auto& exec = m_policy.space();
    const int64_t g = gb300_grid(exec, n > 0 ? n : 1);
    gb300_run_reduce<VB>(exec, m_functor_reducer.get_reducer(), g, m_result_ptr, m_result_ptr_device_accessible,
                         [&](gbk_skel::Val<VB>* part, unsigned* ctr, gbk_skel::Val<VB>* out, int* err) {
                           if (box.fits32) {
                             Closure<int32_t> c{{m_functor_reducer.get_reducer()}, m_functor_reducer.get_functor(),
                                                box};
                             gbk_skel::k_reduce<VB, Closure<int32_t>>
                                 <<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(c, 0, n > 0 ? n : 0, part,
                                                                                       ctr, out, err);
                           } else {
                             Closure<int64_t> c{{m_functor_reducer.get_reducer()}, m_functor_reducer.get_functor(),
                                                box};
                             gbk_skel::k_reduce<VB, Closure<int64_t>>
                                 <<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(c, 0, n > 0 ? n : 0, part,
                                                                                       ctr, out, err);
                           }
                         });
  }
};

}  // namespace Impl
}  // namespace Kokkos

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_PARALLEL_MDRANGE_HPP_
