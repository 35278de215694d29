// ParallelFor / ParallelReduce / ParallelScan / ParallelScanWithTotal over a
// RangePolicy on the GB300 space: the Impl:: pattern classes Kokkos' generic
// dispatch constructs (core/src/Kokkos_Parallel.hpp:130-146,351-420,
// Kokkos_Parallel_Reduce.hpp:1508-1545) and calls execute() on.  Each adapts
// the Kokkos functor (and its FunctorAnalysis reducer) to a closure and
// launches one of the skeleton kernels of Kokkos_GB300_Skeletons.hpp; the CUDA
// space's versions (core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:38-1053) use
// two launches per scan and a grid capped at concurrency / block size, these
// use one launch each and a persistent grid.
#ifndef KOKKOS_GB300_PARALLEL_RANGE_HPP_
#define KOKKOS_GB300_PARALLEL_RANGE_HPP_

#include <Kokkos_Macros.hpp>
#if defined(KOKKOS_ENABLE_GB300)

#include <type_traits>

#include <Kokkos_Parallel.hpp>
#include <impl/Kokkos_FunctorAnalysis.hpp>

#include <GB300/Kokkos_GB300.hpp>
#include <GB300/Kokkos_GB300_Skeletons.hpp>

namespace Kokkos {
namespace Impl {

// ---- launch helpers ---------------------------------------------------------
struct GB300Scratch {
  char* base;
  unsigned* counters;
  int* err;
};
inline GB300Scratch gb300_scratch(const Kokkos::Experimental::GB300& exec, size_t bytes) {
  void* p = nullptr;
  unsigned* c = nullptr;
  int* e = nullptr;
  gb300_check(gbk_workspace_acquire((gbk_stream_t)exec.stream(), (int64_t)bytes, &p, &c, &e), "GB300 workspace");
  return {(char*)p, c, e};
}
inline void gb300_launched(const char* what) {
  gb300_check_cuda(cudaGetLastError(), what);
  gbk_note_launches(1);
}
inline int64_t gb300_grid(const Kokkos::Experimental::GB300& exec, int64_t n) {
  int64_t g = (n + gbk_skel::kBlock - 1) / gbk_skel::kBlock;
  const int64_t cap = (int64_t)exec.sm_count() * 8;
  if (g > cap) g = cap;
  return g < 1 ? 1 : g;
}

// Calls functor(i) or functor(Tag(), i).
template <class WorkTag, class F, class... A>
__device__ __forceinline__ void gb300_call(const F& f, A&&... a) {
  if constexpr (std::is_void_v<WorkTag>) f(static_cast<A&&>(a)...);
  else f(WorkTag{}, static_cast<A&&>(a)...);
}

// The reducer's algebra on opaque values (the skeletons' closure interface).
template <class ReducerType>
struct GB300ValueOps {
  ReducerType r;
  using pointer_type = typename ReducerType::pointer_type;
  using value_type = typename ReducerType::value_type;
  __device__ void init(void* v) const { r.init(static_cast<pointer_type>(v)); }
  __device__ void join(void* d, const void* s) const {
    r.join(static_cast<pointer_type>(d), static_cast<const value_type*>(s));
  }
  __device__ void final_(void* v) const { r.final(static_cast<pointer_type>(v)); }
};

// Value bytes of a reducer: compile-time when the value type is fixed, the
// skeletons' maximum when it is a runtime-length array.
template <class ReducerType>
constexpr int gb300_value_bytes() {
  return ReducerType::static_value_size() ? gbk_skel::value_bytes(ReducerType::static_value_size())
                                          : gbk_skel::kMaxValueBytes;
}

// Runs a reduce skeleton and delivers the value: to a device-accessible
// result in place, to a host result by a copy and a fence (the reference's
// rule, Kokkos_Cuda_Parallel_Range.hpp:343-367).
// `extra` bytes of the workspace after the partials (256-byte aligned) go to
// a launch that takes them as a fifth argument.
template <int VB, class ReducerType, class Launch>
void gb300_run_reduce(const Kokkos::Experimental::GB300& exec, const ReducerType& reducer, int64_t grid,
                      typename ReducerType::pointer_type result, bool result_on_device, Launch&& launch,
                      size_t extra = 0) {
  using V = gbk_skel::Val<VB>;
  const size_t vsize = reducer.value_size();
  if (vsize > (size_t)VB)
    gb300_check(GBK_ERR_UNSUPPORTED, "parallel_reduce on GB300: reduction value larger than 256 bytes");
  const size_t head = (256 + (size_t)(grid + 1) * sizeof(V) + 255) / 256 * 256;
  GB300Scratch sc = gb300_scratch(exec, head + extra);
  V* dev_out = reinterpret_cast<V*>(sc.base + 256);
  V* partials = dev_out + 1;
  if constexpr (std::is_invocable_v<Launch, V*, unsigned*, V*, int*, char*>)
    launch(partials, sc.counters + gbk_skel::kSlotReduce, dev_out, sc.err, sc.base + head);
  else
    launch(partials, sc.counters + gbk_skel::kSlotReduce, dev_out, sc.err);
  gb300_launched("parallel_reduce");
  if (!result) return;
  if (result_on_device) {
    gb300_check_cuda(cudaMemcpyAsync(result, dev_out, vsize, cudaMemcpyDeviceToDevice, exec.stream()),
                     "parallel_reduce");
  } else {
    // value sizes are at most VB = 256 bytes (checked above)
    exec.impl_fence_read("Kokkos::Impl::ParallelReduce<GB300>: result not device accessible", dev_out, result,
                         vsize);
  }
}

// ---- ParallelFor<RangePolicy> ----------------------------------------------
template <class FunctorType, class... Traits>
class ParallelFor<FunctorType, Kokkos::RangePolicy<Traits...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::RangePolicy<Traits...>;
  using functor_type = FunctorType;

 private:
  using Member = typename Policy::member_type;
  using WorkTag = typename Policy::work_tag;
  const FunctorType m_functor;
  const Policy m_policy;

 public:
  // the kernel's closure (public: a kernel template argument must be)
  struct Closure {
    FunctorType f;
    __device__ void exec(int64_t i) const { gb300_call<WorkTag>(f, static_cast<Member>(i)); }
  };

  Policy const& get_policy() const { return m_policy; }
  ParallelFor(const FunctorType& arg_functor, const Policy& arg_policy)
      : m_functor(arg_functor), m_policy(arg_policy) {}

  void execute() const {
    const int64_t n = (int64_t)m_policy.end() - (int64_t)m_policy.begin();
    if (n <= 0) return;
    const auto& exec = m_policy.space();
    const int64_t g = gb300_grid(exec, n);
    int* err = gb300_scratch(exec, 0).err;
    gbk_skel::k_for<Closure><<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(Closure{m_functor},
                                                                                   (int64_t)m_policy.begin(), n, err);
    gb300_launched("parallel_for");
  }
};

// ---- ParallelReduce<RangePolicy> -------------------------------------------
template <class CombinedFunctorReducerType, class... Traits>
class ParallelReduce<CombinedFunctorReducerType, Kokkos::RangePolicy<Traits...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::RangePolicy<Traits...>;
  using FunctorType = typename CombinedFunctorReducerType::functor_type;
  using ReducerType = typename CombinedFunctorReducerType::reducer_type;
  using pointer_type = typename ReducerType::pointer_type;
  using value_type = typename ReducerType::value_type;
  using reference_type = typename ReducerType::reference_type;
  using functor_type = FunctorType;
  using reducer_type = ReducerType;

 private:
  using Member = typename Policy::member_type;
  using WorkTag = typename Policy::work_tag;
  const CombinedFunctorReducerType m_functor_reducer;
  const Policy m_policy;
  const pointer_type m_result_ptr;
  const bool m_result_ptr_device_accessible;

 public:
  struct Closure : GB300ValueOps<ReducerType> {
    FunctorType f;
    __device__ void exec(int64_t i, void* v) const {
      gb300_call<WorkTag>(f, static_cast<Member>(i), this->r.reference(static_cast<pointer_type>(v)));
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

  void execute() const {
    constexpr int VB = gb300_value_bytes<ReducerType>();
    const int64_t n = (int64_t)m_policy.end() - (int64_t)m_policy.begin();
    const auto& exec = m_policy.space();
    const int64_t g = gb300_grid(exec, n > 0 ? n : 1);
    const int64_t b = (int64_t)m_policy.begin();
    Closure c{{m_functor_reducer.get_reducer()}, m_functor_reducer.get_functor()};
    gb300_run_reduce<VB>(exec, m_functor_reducer.get_reducer(), g, m_result_ptr, m_result_ptr_device_accessible,
                         [&](gbk_skel::Val<VB>* part, unsigned* ctr, gbk_skel::Val<VB>* out, int* err) {
                           gbk_skel::k_reduce<VB, Closure><<<(unsigned)g, gbk_skel::kBlock, 0, exec.stream()>>>(
                               c, b, n > 0 ? n : 0, part, ctr, out, err);
                         });
  }
};

// ---- ParallelScan / ParallelScanWithTotal<RangePolicy> ---------------------
template <class FunctorType, class ReducerType, class Member, class WorkTag>
struct GB300ScanClosure : GB300ValueOps<ReducerType> {
  FunctorType f;
  using pointer_type = typename ReducerType::pointer_type;
  __device__ void exec(int64_t i, void* v, bool final_pass) const {
    gb300_call<WorkTag>(f, static_cast<Member>(i), this->r.reference(static_cast<pointer_type>(v)), final_pass);
  }
};

// A closure with no work and no final step: a reduce over it yields the
// reducer's identity (the total of an empty scan).
template <class ReducerType>
struct GB300IdentityClosure : GB300ValueOps<ReducerType> {
  __device__ void exec(int64_t, void*) const {}
  __device__ void final_(void*) const {}
};

// One look-back scan launch; the total (if asked for) lands in *dev_total.
template <int VB, class Closure>
void gb300_run_scan(const Kokkos::Experimental::GB300& exec, const Closure& c, int64_t begin, int64_t n,
                    size_t vsize, gbk_skel::Val<VB>** dev_total) {
  using V = gbk_skel::Val<VB>;
  if (vsize > (size_t)VB) gb300_check(GBK_ERR_UNSUPPORTED, "parallel_scan on GB300: value larger than 256 bytes");
  constexpr int64_t TILE = (int64_t)gbk_skel::kBlock * gbk_skel::kItems;
  const int64_t nt = (n + TILE - 1) / TILE;
  const size_t fb = ((size_t)nt * 4 + 255) / 256 * 256, vb = ((size_t)nt * sizeof(V) + 255) / 256 * 256;
  GB300Scratch sc = gb300_scratch(exec, 256 + fb + 2 * vb);
  gbk_skel::ScanState<VB> S;
  S.flags = reinterpret_cast<unsigned*>(sc.base + 256);
  S.agg = reinterpret_cast<V*>(sc.base + 256 + fb);
  S.incl = reinterpret_cast<V*>(sc.base + 256 + fb + vb);
  S.ticket = sc.counters + gbk_skel::kSlotScan;
  S.err = sc.err;
  S.ntiles = nt;
  S.wait_limit = gbk_wait_limit();
  V* tot = reinterpret_cast<V*>(sc.base);
  if (dev_total) *dev_total = tot;
  gb300_check_cuda(cudaMemsetAsync(S.flags, 0, (size_t)nt * 4, exec.stream()), "parallel_scan");
  gbk_skel::k_scan<VB, Closure><<<(unsigned)nt, gbk_skel::kBlock, 0, exec.stream()>>>(c, begin, n, S,
                                                                                       dev_total ? tot : nullptr);
  gb300_launched("parallel_scan");
}

template <class FunctorType, class... Traits>
class ParallelScan<FunctorType, Kokkos::RangePolicy<Traits...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::RangePolicy<Traits...>;
  using functor_type = FunctorType;

 private:
  using Member = typename Policy::member_type;
  using WorkTag = typename Policy::work_tag;
  using Analysis = Kokkos::Impl::FunctorAnalysis<FunctorPatternInterface::SCAN, Policy, FunctorType, void>;
  using ReducerType = typename Analysis::Reducer;
  const CombinedFunctorReducer<FunctorType, ReducerType> m_functor_reducer;
  const Policy m_policy;

 public:
  Policy const& get_policy() const { return m_policy; }
  ParallelScan(const FunctorType& arg_functor, const Policy& arg_policy)
      : m_functor_reducer(arg_functor, ReducerType{arg_functor}), m_policy(arg_policy) {}

  void execute() const {
    constexpr int VB = gb300_value_bytes<ReducerType>();
    const int64_t n = (int64_t)m_policy.end() - (int64_t)m_policy.begin();
    if (n <= 0) return;
    using C = GB300ScanClosure<FunctorType, ReducerType, Member, WorkTag>;
    C c{{m_functor_reducer.get_reducer()}, m_functor_reducer.get_functor()};
    gb300_run_scan<VB>(m_policy.space(), c, (int64_t)m_policy.begin(), n, m_functor_reducer.get_reducer().value_size(),
                       nullptr);
  }
};

template <class FunctorType, class ReturnType, class... Traits>
class ParallelScanWithTotal<FunctorType, Kokkos::RangePolicy<Traits...>, ReturnType, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::RangePolicy<Traits...>;
  using functor_type = FunctorType;

 private:
  using Member = typename Policy::member_type;
  using WorkTag = typename Policy::work_tag;
  using Analysis = Kokkos::Impl::FunctorAnalysis<FunctorPatternInterface::SCAN, Policy, FunctorType, ReturnType>;
  using ReducerType = typename Analysis::Reducer;
  using pointer_type = typename Analysis::pointer_type;
  const CombinedFunctorReducer<FunctorType, ReducerType> m_functor_reducer;
  const Policy m_policy;
  const pointer_type m_result_ptr;
  const bool m_result_ptr_device_accessible;

 public:
  Policy const& get_policy() const { return m_policy; }
  template <class ViewType>
  ParallelScanWithTotal(const FunctorType& arg_functor, const Policy& arg_policy, const ViewType& arg_result_view)
      : m_functor_reducer(arg_functor, ReducerType{arg_functor}),
        m_policy(arg_policy),
        m_result_ptr(arg_result_view.data()),
        m_result_ptr_device_accessible(
            MemorySpaceAccess<Kokkos::Experimental::GB300Space, typename ViewType::memory_space>::accessible) {}

  void execute() const {
    constexpr int VB = gb300_value_bytes<ReducerType>();
    const auto& exec = m_policy.space();
    const auto& reducer = m_functor_reducer.get_reducer();
    const size_t vsize = reducer.value_size();
    const int64_t n = (int64_t)m_policy.end() - (int64_t)m_policy.begin();
    if (n <= 0) {
      // the total of an empty range is the reducer's identity
      if (m_result_ptr) {
        if (m_result_ptr_device_accessible) {
          gb300_run_reduce<VB>(exec, reducer, 1, m_result_ptr, true,
                               [&](gbk_skel::Val<VB>* part, unsigned* ctr, gbk_skel::Val<VB>* out, int* err) {
                                 gbk_skel::k_reduce<VB, GB300IdentityClosure<ReducerType>>
                                     <<<1, gbk_skel::kBlock, 0, exec.stream()>>>(
                                         GB300IdentityClosure<ReducerType>{{reducer}}, 0, 0, part, ctr, out, err);
                               });
        } else {
          reducer.init(m_result_ptr);
        }
      }
      return;
    }
    using C = GB300ScanClosure<FunctorType, ReducerType, Member, WorkTag>;
    C c{{reducer}, m_functor_reducer.get_functor()};
    gbk_skel::Val<VB>* tot = nullptr;
    gb300_run_scan<VB>(exec, c, (int64_t)m_policy.begin(), n, vsize, &tot);
    if (m_result_ptr) {
      gb300_check_cuda(cudaMemcpyAsync(m_result_ptr, tot, vsize,
                                       m_result_ptr_device_accessible ? cudaMemcpyDeviceToDevice
                                                                      : cudaMemcpyDeviceToHost,
                                       exec.stream()),
                       "parallel_scan total");
    }
  }
};

}  // namespace Impl
}  // namespace Kokkos

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_PARALLEL_RANGE_HPP_
