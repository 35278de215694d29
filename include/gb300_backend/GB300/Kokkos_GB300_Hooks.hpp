// The GB300 space's hooks in Kokkos' containers and algorithms, declared
// ahead of the headers that use them (Kokkos_Core.hpp includes this through
// the backend declarations, before Kokkos_ScatterView.hpp and Kokkos_Sort.hpp
// are read):
//
//   * ScatterView defaults (containers/src/Kokkos_ScatterView.hpp:59-198):
//     NonDuplicated + Atomic, as for the CUDA space; and the atomic Sum
//     contribution on this space is warp-aggregated: the lanes of a warp that
//     add to the same element combine their values first and one lane issues
//     the atomic (hot keys of a skewed histogram serialise 32x less);
//   * sort_device_view_without_comparator / sort_by_key_device_view_without_
//     comparator overloads (algorithms/src/sorting/impl/Kokkos_SortImpl.hpp:
//     347-396, impl/Kokkos_SortByKeyImpl.hpp:356-409): Kokkos::sort and
//     Experimental::sort_by_key on a contiguous GB300 View of 4- or 8-byte
//     keys run the library's stable radix sort (gbk_sort / gbk_sort_by_key)
//     where the CUDA space calls thrust.
#ifndef KOKKOS_GB300_HOOKS_HPP_
#define KOKKOS_GB300_HOOKS_HPP_

#include <Kokkos_Macros.hpp>
#if defined(KOKKOS_ENABLE_GB300)

#include <algorithm>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

#include <Kokkos_Atomic.hpp>

#include <GB300/Kokkos_GB300.hpp>

// ---- ScatterView ----------------------------------------------------------------
namespace Kokkos {
namespace Experimental {
struct ScatterSum;
struct ScatterNonDuplicated;
struct ScatterDuplicated;
struct ScatterAtomic;
}  // namespace Experimental
namespace Impl {
namespace Experimental {
template <typename ExecSpace>
struct DefaultDuplication;
template <typename ExecSpace, typename Duplication>
struct DefaultContribution;
template <typename ValueType, typename Op, typename DeviceType, typename Contribution>
struct ScatterValue;

template <>
struct DefaultDuplication<Kokkos::Experimental::GB300> {
  using type = Kokkos::Experimental::ScatterNonDuplicated;
};
template <>
struct DefaultContribution<Kokkos::Experimental::GB300, Kokkos::Experimental::ScatterNonDuplicated> {
  using type = Kokkos::Experimental::ScatterAtomic;
};
template <>
struct DefaultContribution<Kokkos::Experimental::GB300, Kokkos::Experimental::ScatterDuplicated> {
  using type = Kokkos::Experimental::ScatterAtomic;
};

// Native atomic add for the arithmetic types (64-bit integers as unsigned
// long long: two's complement addition is the same operation); others go
// through Kokkos::atomic_add.
template <class T>
__device__ __forceinline__ void gb300_atomic_add(T* dest, T v) {
  if constexpr (std::is_integral_v<T> && sizeof(T) == 8)
    atomicAdd(reinterpret_cast<unsigned long long*>(dest), (unsigned long long)v);
  else if constexpr (std::is_integral_v<T> && sizeof(T) == 4)
    atomicAdd(reinterpret_cast<unsigned*>(dest), (unsigned)v);
  else if constexpr (std::is_same_v<T, float> || std::is_same_v<T, double>)
    atomicAdd(dest, v);
  else
    Kokkos::atomic_add(dest, v);
}

// Warp-aggregated atomic add: lanes adding to the same element sum their
// values and the group's lowest lane adds the sum.  Lanes are grouped by
// element index: a 32-bit match on its low bits when every active lane's
// index agrees above them (one shuffle and a vote decide), else a 64-bit
// match.  Measured on GB300, 2^26 additions of 1 into 2^16 int64 elements
// from a user kernel: uniform indices 0.50 ms with the 32-bit match (plain
// atomics 0.38-0.41, the 64-bit match 1.42), Zipf(1.1) indices 8.3 ms (plain
// atomics 14.1: the hot elements serialise at L2).
template <class T>
__device__ __forceinline__ void gb300_aggregated_add(T* dest, T v) {
  if constexpr (std::is_arithmetic_v<T> && (sizeof(T) == 4 || sizeof(T) == 8)) {
    const unsigned active = __activemask();
    const uint64_t a = (uint64_t)(uintptr_t)dest / sizeof(T);
    const unsigned hi = (unsigned)(a >> 32);
    const unsigned peers = __all_sync(active, __shfl_sync(active, hi, __ffs(active) - 1) == hi)
                               ? __match_any_sync(active, (unsigned)a)
                               : __match_any_sync(active, (unsigned long long)a);
    const int leader = __ffs(peers) - 1;
    T sum;
    if constexpr (std::is_integral_v<T> && sizeof(T) == 4) {
      sum = (T)__reduce_add_sync(peers, (unsigned)v);
    } else {
      sum = T(0);
      for (unsigned m = peers; m; m &= m - 1) sum += __shfl_sync(peers, v, __ffs(m) - 1);
    }
    unsigned lane;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    if ((int)lane == leader) gb300_atomic_add(dest, sum);
  } else {
    Kokkos::atomic_add(dest, v);
  }
}

template <typename ValueType>
struct ScatterValue<ValueType, Kokkos::Experimental::ScatterSum,
                    Kokkos::Device<Kokkos::Experimental::GB300, Kokkos::Experimental::GB300Space>,
                    Kokkos::Experimental::ScatterAtomic> {
  ValueType& value;

 public:
  KOKKOS_FORCEINLINE_FUNCTION ScatterValue(ValueType& value_in) : value(value_in) {}
  KOKKOS_FORCEINLINE_FUNCTION void operator+=(ValueType const& rhs) { this->join(value, rhs); }
  KOKKOS_FORCEINLINE_FUNCTION void operator++() { this->join(value, ValueType(1)); }
  KOKKOS_FORCEINLINE_FUNCTION void operator++(int) { this->join(value, ValueType(1)); }
  KOKKOS_FORCEINLINE_FUNCTION void operator-=(ValueType const& rhs) { this->join(value, ValueType(-rhs)); }
  KOKKOS_FORCEINLINE_FUNCTION void operator--() { this->join(value, ValueType(-1)); }
  KOKKOS_FORCEINLINE_FUNCTION void operator--(int) { this->join(value, ValueType(-1)); }
  KOKKOS_INLINE_FUNCTION void join(ValueType& dest, const ValueType& src) const {
    KOKKOS_IF_ON_DEVICE((gb300_aggregated_add(&dest, src);))
    KOKKOS_IF_ON_HOST((Kokkos::atomic_add(&dest, src);))
  }
  KOKKOS_FORCEINLINE_FUNCTION void update(ValueType const& rhs) { this->join(value, rhs); }
  KOKKOS_FORCEINLINE_FUNCTION void reset() { value = ValueType(); }
};

}  // namespace Experimental

// ---- sort ----------------------------------------------------------------------------
template <class T>
constexpr int gb300_sort_dtype() {
  if constexpr (std::is_same_v<T, int32_t>) return GBK_I32;
  else if constexpr (std::is_same_v<T, int64_t>) return GBK_I64;
  else if constexpr (std::is_same_v<T, uint32_t>) return GBK_U32;
  else if constexpr (std::is_same_v<T, uint64_t>) return GBK_U64;
  else if constexpr (std::is_same_v<T, float>) return GBK_F32;
  else if constexpr (std::is_same_v<T, double>) return GBK_F64;
  else if constexpr (std::is_integral_v<T> && sizeof(T) == 8)
    return std::is_signed_v<T> ? GBK_I64 : GBK_U64;  // long long / unsigned long long
  else return -1;
}

// A strided (non-contiguous) View is sorted in a contiguous copy; values of
// a size the library does not move (not 4 or 8 bytes) follow the keys through
// a sorted index permutation and one gather.  The copies are small kernels of
// their own (this header is read before Kokkos' deep_copy and parallel_for).
template <class T>
using GB300SortTemp = Kokkos::View<T*, Kokkos::Experimental::GB300Space>;
template <class T>
GB300SortTemp<T> gb300_sort_temp(const Kokkos::Experimental::GB300& exec, const char* label, int64_t n) {
  return GB300SortTemp<T>(Kokkos::view_alloc(exec, Kokkos::WithoutInitializing, std::string(label)), n);
}
template <class Dst, class Src>
__global__ void k_gb300_copy_view(Dst dst, Src src, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst(i) = src(i);
}
template <class P>
__global__ void k_gb300_iota(P* p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (P)i;
}
template <class Dst, class Src, class P>
__global__ void k_gb300_gather(Dst dst, Src src, const P* perm, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst(i) = src(perm[i]);
}
inline unsigned gb300_copy_grid(const Kokkos::Experimental::GB300& exec, int64_t n) {
  int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)exec.sm_count() * 8;
  return (unsigned)(g < 1 ? 1 : g > cap ? cap : g);
}
template <class Dst, class Src>
void gb300_copy_view(const Kokkos::Experimental::GB300& exec, const Dst& dst, const Src& src, int64_t n) {
  k_gb300_copy_view<<<gb300_copy_grid(exec, n), 256, 0, exec.stream()>>>(dst, src, n);
  gb300_check_cuda(cudaGetLastError(), "Kokkos::sort on GB300: copy");
  gbk_note_launches(1);
}

template <class DataType, class... Properties>
void sort_device_view_without_comparator(const Kokkos::Experimental::GB300& exec,
                                         const Kokkos::View<DataType, Properties...>& view) {
  using ViewType = Kokkos::View<DataType, Properties...>;
  using T = typename ViewType::non_const_value_type;
  static_assert(ViewType::rank == 1, "Kokkos::sort: currently only supports rank-1 Views.");
  constexpr int dt = gb300_sort_dtype<T>();
  static_assert(dt >= 0, "Kokkos::sort on GB300: keys must be 4- or 8-byte integers or floating point");
  const int64_t n = (int64_t)view.extent(0);
  if (n <= 1) return;
  if (view.span_is_contiguous()) {
    gb300_check(gbk_sort((gbk_dtype_t)dt, (void*)view.data(), n, (gbk_stream_t)exec.stream()), "sort");
    return;
  }
  auto kt = gb300_sort_temp<T>(exec, "Kokkos::sort keys", n);
  gb300_copy_view(exec, kt, view, n);
  gb300_check(gbk_sort((gbk_dtype_t)dt, (void*)kt.data(), n, (gbk_stream_t)exec.stream()), "sort");
  gb300_copy_view(exec, view, kt, n);
}

template <class KeysDataType, class... KeysProperties, class ValuesDataType, class... ValuesProperties>
void sort_by_key_device_view_without_comparator(const Kokkos::Experimental::GB300& exec,
                                                const Kokkos::View<KeysDataType, KeysProperties...>& keys,
                                                const Kokkos::View<ValuesDataType, ValuesProperties...>& values) {
  using K = typename Kokkos::View<KeysDataType, KeysProperties...>::non_const_value_type;
  using V = typename Kokkos::View<ValuesDataType, ValuesProperties...>::non_const_value_type;
  constexpr int dt = gb300_sort_dtype<K>();
  static_assert(dt >= 0, "Kokkos::sort_by_key on GB300: keys must be 4- or 8-byte integers or floating point");
  constexpr bool MOVED = sizeof(V) == 4 || sizeof(V) == 8;  // values the library moves with the keys
  const int64_t n = (int64_t)keys.extent(0);
  if (n <= 1) return;
  const gbk_stream_t s = (gbk_stream_t)exec.stream();
  if constexpr (MOVED) {
    if (keys.span_is_contiguous() && values.span_is_contiguous()) {
      gb300_check(gbk_sort_by_key((gbk_dtype_t)dt, (void*)keys.data(), (int)sizeof(V), (void*)values.data(), n, s),
                  "sort_by_key");
      return;
    }
  }
  auto kt = gb300_sort_temp<K>(exec, "Kokkos::sort_by_key keys", n);
  gb300_copy_view(exec, kt, keys, n);
  if constexpr (MOVED) {
    auto vt = gb300_sort_temp<V>(exec, "Kokkos::sort_by_key values", n);
    gb300_copy_view(exec, vt, values, n);
    gb300_check(gbk_sort_by_key((gbk_dtype_t)dt, (void*)kt.data(), (int)sizeof(V), (void*)vt.data(), n, s),
                "sort_by_key");
    gb300_copy_view(exec, values, vt, n);
  } else {
    // the stable permutation, then the values gathered through it
    using P = uint64_t;
    auto perm = gb300_sort_temp<P>(exec, "Kokkos::sort_by_key permutation", n);
    k_gb300_iota<P><<<gb300_copy_grid(exec, n), 256, 0, exec.stream()>>>(perm.data(), n);
    gb300_check_cuda(cudaGetLastError(), "Kokkos::sort_by_key on GB300: permutation");
    gbk_note_launches(1);
    gb300_check(gbk_sort_by_key((gbk_dtype_t)dt, (void*)kt.data(), (int)sizeof(P), (void*)perm.data(), n, s),
                "sort_by_key");
    auto vt = gb300_sort_temp<V>(exec, "Kokkos::sort_by_key values", n);
    k_gb300_gather<<<gb300_copy_grid(exec, n), 256, 0, exec.stream()>>>(vt, values, perm.data(), n);
    gb300_check_cuda(cudaGetLastError(), "Kokkos::sort_by_key on GB300: gather");
    gbk_note_launches(1);
    gb300_copy_view(exec, values, vt, n);
  }
  gb300_copy_view(exec, keys, kt, n);
}

}  // namespace Impl
}  // namespace Kokkos

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_HOOKS_HPP_
