// ParallelFor / ParallelReduce over an MDRangePolicy on the GB300 space
// (the CUDA space's versions: core/src/Cuda/Kokkos_Cuda_Parallel_MDRange.hpp:
// 45-497 with impl/KokkosExp_IterateTileGPU.hpp, one element per thread per
// tile and a grid of at most the block size in CTAs).
//
// Here the box [lower, upper) of rank 1..6 is walked as one flat index space
// on the skeleton kernels of Kokkos_GB300_Skeletons.hpp: the policy's inner
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

// The box of an MDRangePolicy as the kernels see it: extents in walk order
// (walk dimension 0 fastest) and, per walk dimension, the policy dimension it
// stands for.
template <int R, class Index>
struct GB300Box {
  Index lo[R];
  Index ext[R];
  int dim[R];  // walk order -> policy dimension
  bool fits32;

  // index of the element at flat position f, in policy dimension order
  __device__ __forceinline__ void point(int64_t f, Index (&i)[R]) const {
    if (fits32) {
      uint32_t r = (uint32_t)f;
#pragma unroll
      for (int d = 0; d < R - 1; ++d) {
        const uint32_t e = (uint32_t)ext[d];
        i[dim[d]] = lo[dim[d]] + (Index)(r % e);
        r /= e;
      }
      i[dim[R - 1]] = lo[dim[R - 1]] + (Index)r;
    } else {
      int64_t r = f;
#pragma unroll
      for (int d = 0; d < R - 1; ++d) {
        const int64_t e = (int64_t)ext[d];
        i[dim[d]] = lo[dim[d]] + (Index)(r % e);
        r /= e;
      }
      i[dim[R - 1]] = lo[dim[R - 1]] + (Index)r;
    }
  }
};

template <class MDPolicy, int R = MDPolicy::rank>
GB300Box<R, typename MDPolicy::index_type> gb300_box(const MDPolicy& p, int64_t* total) {
  using Index = typename MDPolicy::index_type;
  GB300Box<R, Index> b{};
  // Left: dimension 0 fastest; Right: dimension R-1 fastest.  The outer
  // direction of the reference orders tiles, which a flat walk does not have;
  // the inner direction alone sets the element order here.
  const bool left = MDPolicy::inner_direction == Iterate::Left;
  int64_t n = 1;
  for (int d = 0; d < R; ++d) {
    const int pd = left ? d : R - 1 - d;
    b.dim[d] = pd;
    b.lo[pd] = (Index)p.m_lower[pd];
    const int64_t e = (int64_t)p.m_upper[pd] - (int64_t)p.m_lower[pd];
    b.ext[d] = (Index)(e > 0 ? e : 0);
    n *= (e > 0 ? e : 0);
  }
  b.fits32 = n < (int64_t(1) << 31);
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
  struct Closure {
    FunctorType f;
    GB300Box<R, Index> box;
    __device__ void exec(int64_t flat) const {
      Index i[R];
      box.point(flat, i);
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
    gbk_skel::k_for<Closure><<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(Closure{m_functor, box}, 0, n,
                                                                                   err);
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
  struct Closure : GB300ValueOps<ReducerType> {
    FunctorType f;
    GB300Box<R, Index> box;
    __device__ void exec(int64_t flat, void* v) const {
      Index i[R];
      box.point(flat, i);
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
    Closure c{{m_functor_reducer.get_reducer()}, m_functor_reducer.get_functor(), box};
    gb300_run_reduce<VB>(exec, m_functor_reducer.get_reducer(), g, m_result_ptr, m_result_ptr_device_accessible,
                         [&](gbk_skel::Val<VB>* part, unsigned* ctr, gbk_skel::Val<VB>* out, int* err) {
                           gbk_skel::k_reduce<VB, Closure><<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(
                               c, 0, n > 0 ? n : 0, part, ctr, out, err);
                         });
  }
};

}  // namespace Impl
}  // namespace Kokkos

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_PARALLEL_MDRANGE_HPP_
