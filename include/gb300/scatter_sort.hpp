// Atomics, ScatterView, sort / sort_by_key and BinSort of the header path.
//   atomics: Kokkos::atomic_add / fetch_add / min / max / compare_exchange
//     (core/src/Kokkos_Atomics_Desul_Wrapper.hpp; desul
//     tpls/desul/include/desul/atomics/Fetch_Op_CUDA.hpp:12-130)
//   ScatterView: containers/src/Kokkos_ScatterView.hpp:41-198 (tags and the
//     device defaults NonDuplicated + Atomic, :152-165), :207-460
//     (ScatterValue), :1456-1580 (access, create_scatter_view, contribute)
//   sort / sort_by_key / BinSort: algorithms/src/sorting/* routed to the
//     library's stable radix sort (gbk_sort, gbk_sort_by_key, gbk_binsort_u64)
#pragma once

#include <cstdio>

#include "parallel.hpp"

namespace gb300k {

namespace Impl {
template <class T> struct dtype_code;
template <> struct dtype_code<int32_t> { static constexpr int value = GBK_I32; };
template <> struct dtype_code<int64_t> { static constexpr int value = GBK_I64; };
template <> struct dtype_code<uint32_t> { static constexpr int value = GBK_U32; };
template <> struct dtype_code<uint64_t> { static constexpr int value = GBK_U64; };
template <> struct dtype_code<float> { static constexpr int value = GBK_F32; };
template <> struct dtype_code<double> { static constexpr int value = GBK_F64; };
template <> struct dtype_code<long long> { static constexpr int value = GBK_I64; };
template <> struct dtype_code<unsigned long long> { static constexpr int value = GBK_U64; };

// Kokkos::abort on size mismatches (Kokkos_SortByKeyPublicAPI.hpp:55-60);
// here a std::runtime_error, so a caller can observe it.
inline void abort_msg(const char* m) { throw std::runtime_error(m); }

template <class T, class Fn>
__device__ T cas_update(T* p, Fn fn) {
  using U = std::conditional_t<sizeof(T) == 4, unsigned, unsigned long long>;
  U* up = reinterpret_cast<U*>(p);
  U old = *reinterpret_cast<volatile U*>(up), assumed;
  do {
    assumed = old;
    T cur;
    memcpy(&cur, &assumed, sizeof(T));
    const T nv = fn(cur);
    U nu;
    memcpy(&nu, &nv, sizeof(T));
    old = atomicCAS(up, assumed, nu);
  } while (old != assumed);
  T r;
  memcpy(&r, &old, sizeof(T));
  return r;
}
}  // namespace Impl

// ---- atomics (host-device signatures, device-only effect) --------------------
template <class T>
KOKKOS_INLINE_FUNCTION T atomic_fetch_add(T* p, T v) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<T, int64_t>::value || std::is_same<T, long long>::value)
    return (T)atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  else if constexpr (std::is_same<T, uint64_t>::value)
    return (T)atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  else
    return atomicAdd(p, v);
#else
  const T o = *p;
  *p = o + v;
  return o;
#endif
}
template <class T>
KOKKOS_INLINE_FUNCTION void atomic_add(T* p, T v) {
  (void)atomic_fetch_add(p, v);
}
template <class T>
KOKKOS_INLINE_FUNCTION T atomic_fetch_min(T* p, T v) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_integral<T>::value && sizeof(T) == 4) return atomicMin(p, v);
  else if constexpr (std::is_same<T, int64_t>::value) return (T)atomicMin(reinterpret_cast<long long*>(p), (long long)v);
  else if constexpr (std::is_same<T, uint64_t>::value)
    return (T)atomicMin(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  else return Impl::cas_update(p, [v](T c) { return v < c ? v : c; });
#else
  const T o = *p;
  if (v < o) *p = v;
  return o;
#endif
}
template <class T>
KOKKOS_INLINE_FUNCTION T atomic_fetch_max(T* p, T v) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_integral<T>::value && sizeof(T) == 4) return atomicMax(p, v);
  else if constexpr (std::is_same<T, int64_t>::value) return (T)atomicMax(reinterpret_cast<long long*>(p), (long long)v);
  else if constexpr (std::is_same<T, uint64_t>::value)
    return (T)atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  else return Impl::cas_update(p, [v](T c) { return v > c ? v : c; });
#else
  const T o = *p;
  if (v > o) *p = v;
  return o;
#endif
}
template <class T>
KOKKOS_INLINE_FUNCTION void atomic_min(T* p, T v) { (void)atomic_fetch_min(p, v); }
template <class T>
KOKKOS_INLINE_FUNCTION void atomic_max(T* p, T v) { (void)atomic_fetch_max(p, v); }
template <class T>
KOKKOS_INLINE_FUNCTION T atomic_fetch_mul(T* p, T v) {
#ifdef __CUDA_ARCH__
  return Impl::cas_update(p, [v](T c) { return c * v; });
#else
  const T o = *p;
  *p = o * v;
  return o;
#endif
}
template <class T>
KOKKOS_INLINE_FUNCTION T atomic_compare_exchange(T* p, T expected, T desired) {
#ifdef __CUDA_ARCH__
  using U = std::conditional_t<sizeof(T) == 4, unsigned, unsigned long long>;
  U e, d;
  memcpy(&e, &expected, sizeof(T));
  memcpy(&d, &desired, sizeof(T));
  const U o = atomicCAS(reinterpret_cast<U*>(p), e, d);
  T r;
  memcpy(&r, &o, sizeof(T));
  return r;
#else
  const T o = *p;
  if (o == expected) *p = desired;
  return o;
#endif
}

namespace Experimental {
struct ScatterSum {};
struct ScatterProd {};
struct ScatterMin {};
struct ScatterMax {};
struct ScatterNonDuplicated {};
struct ScatterDuplicated {};
struct ScatterAtomic {};
struct ScatterNonAtomic {};

// ScatterValue<Op, ..., ScatterAtomic>: every contribution is one atomic.
template <class T, class Op>
struct ScatterValue {
  T* p;
  KOKKOS_INLINE_FUNCTION void operator+=(T v) const {
    static_assert(std::is_same<Op, ScatterSum>::value, "+= needs ScatterSum");
    atomic_add(p, v);
  }
  KOKKOS_INLINE_FUNCTION void operator-=(T v) const { atomic_add(p, (T)(-v)); }
  KOKKOS_INLINE_FUNCTION void operator++() const { atomic_add(p, (T)1); }
  KOKKOS_INLINE_FUNCTION void operator++(int) const { atomic_add(p, (T)1); }
  KOKKOS_INLINE_FUNCTION void operator*=(T v) const { (void)atomic_fetch_mul(p, v); }
  KOKKOS_INLINE_FUNCTION void update(T v) const {
    if constexpr (std::is_same<Op, ScatterSum>::value) atomic_add(p, v);
    else if constexpr (std::is_same<Op, ScatterProd>::value) (void)atomic_fetch_mul(p, v);
    else if constexpr (std::is_same<Op, ScatterMin>::value) atomic_min(p, v);
    else atomic_max(p, v);
  }
};

// The device default of the reference (NonDuplicated + Atomic): the scatter
// view contributes straight into its destination with atomics.
template <class DataType, class Layout = LayoutLeft, class Space = GB300, class Op = ScatterSum,
          class Dup = ScatterNonDuplicated, class Contrib = ScatterAtomic>
class ScatterView {
 public:
  using original_view_type = View<DataType, Layout>;
  using value_type = typename original_view_type::value_type;
  ScatterView() = default;
  explicit ScatterView(const original_view_type& v) : v_(v) {}
  struct Access {
    value_type* p;
    int64_t s0, s1, s2;
    KOKKOS_INLINE_FUNCTION ScatterValue<value_type, Op> operator()(int64_t i) const { return {p + i * s0}; }
    KOKKOS_INLINE_FUNCTION ScatterValue<value_type, Op> operator()(int64_t i, int64_t j) const {
      return {p + i * s0 + j * s1};
    }
    KOKKOS_INLINE_FUNCTION ScatterValue<value_type, Op> operator()(int64_t i, int64_t j, int64_t k) const {
      return {p + i * s0 + j * s1 + k * s2};
    }
    KOKKOS_INLINE_FUNCTION ScatterValue<value_type, Op> operator[](int64_t i) const { return {p + i}; }
  };
  __host__ __device__ Access access() const { return {v_.data(), v_.stride(0), v_.stride(1), v_.stride(2)}; }
  template <class D, class... P>
  void contribute_into(const View<D, P...>& dest) const {
    if (dest.data() != v_.data()) abort_msg_contribute();
  }
  void reset() {}
  const original_view_type& subview() const { return v_; }

 private:
  static void abort_msg_contribute() {
    Impl::abort_msg("ScatterView (non-duplicated): contribute into a different view is not supported");
  }
  original_view_type v_;
};

template <class Op = ScatterSum, class Dup = ScatterNonDuplicated, class Contrib = ScatterAtomic, class D, class... P>
ScatterView<D, typename View<D, P...>::array_layout, GB300, Op, Dup, Contrib> create_scatter_view(
    const View<D, P...>& v) {
  return ScatterView<D, typename View<D, P...>::array_layout, GB300, Op, Dup, Contrib>(v);
}
template <class D, class... P, class SV>
void contribute(const View<D, P...>& dest, const SV& sv) {
  sv.contribute_into(dest);
}
}  // namespace Experimental

// ---- sort -----------------------------------------------------------------------
template <class D, class... P>
void sort(const Experimental::GB300& ex, const View<D, P...>& v) {
  using T = std::remove_const_t<typename View<D, P...>::value_type>;
  check(gbk_sort((gbk_dtype_t)Impl::dtype_code<T>::value, v.data(), v.size(), ex.handle()), "Kokkos::sort");
}
template <class D, class... P>
void sort(const View<D, P...>& v) {
  sort(Experimental::GB300(), v);
  Experimental::GB300().fence();
}

namespace Experimental {
template <class DK, class... PK, class DV, class... PV>
void sort_by_key(const GB300& ex, const View<DK, PK...>& keys, const View<DV, PV...>& values) {
  using K = std::remove_const_t<typename View<DK, PK...>::value_type>;
  using V = typename View<DV, PV...>::value_type;
  static_assert(sizeof(V) == 4 || sizeof(V) == 8, "sort_by_key: values of 4 or 8 bytes");
  if (keys.size() != values.size()) Impl::abort_msg("values and keys extents must be the same");
  check(gbk_sort_by_key((gbk_dtype_t)Impl::dtype_code<K>::value, keys.data(), (int)sizeof(V), values.data(),
                        keys.size(), ex.handle()),
        "Kokkos::Experimental::sort_by_key");
}
template <class DK, class... PK, class DV, class... PV>
void sort_by_key(const View<DK, PK...>& keys, const View<DV, PV...>& values) {
  sort_by_key(GB300(), keys, values);
  GB300().fence();
}
}  // namespace Experimental

// BinOp1D (algorithms/src/sorting/Kokkos_BinOpsPublicAPI.hpp:25-71): the same
// bin count, multiplier and bin function.
template <class KeyViewType>
struct BinOp1D {
  using key_type = std::remove_const_t<typename KeyViewType::value_type>;
  int max_bins_ = 0;
  double mul_ = 0;
  double min_ = 0;
  BinOp1D(int max_bins, key_type min, key_type max)
      : max_bins_(max_bins + 1), mul_((double)max_bins / ((double)max - (double)min)), min_((double)min) {
    if (std::is_integral<key_type>::value && ((double)max - (double)min) <= (double)max_bins) mul_ = 1.;
  }
  __host__ __device__ int bin(const KeyViewType& keys, int64_t i) const { return (int)(mul_ * ((double)keys(i) - min_)); }
  __host__ __device__ int max_bins() const { return max_bins_; }
};

// BinSort (algorithms/src/sorting/Kokkos_BinSortPublicAPI.hpp:27-408) for
// uint64 keys: create_permute_vector() builds counts, offsets and the stable
// permutation by bin in one library call; sort(values) applies it.
template <class KeyViewType, class BinSortOp>
class BinSort {
 public:
  using offset_type = View<int64_t*>;
  using bin_count_type = View<int32_t*>;
  BinSort(const KeyViewType& keys, BinSortOp op, bool sort_within_bins = false)
      : keys_(keys), op_(op), within_(sort_within_bins), counts_("bin_count", op.max_bins()),
        offsets_("bin_offsets", op.max_bins()), perm_("permute_vector", keys.size()) {
    static_assert(sizeof(typename KeyViewType::value_type) == 8, "BinSort on this space takes 64-bit keys");
  }
  void create_permute_vector(const Experimental::GB300& ex = Experimental::GB300()) {
    check(gbk_binsort_u64((const uint64_t*)keys_.data(), keys_.size(), op_.max_bins(), op_.min_, op_.mul_,
                          within_ ? 1 : 0, counts_.data(), offsets_.data(), perm_.data(), ex.handle()),
          "BinSort::create_permute_vector");
    ex.fence();
  }
  template <class ValuesView>
  void sort(const Experimental::GB300& ex, const ValuesView& values) const {
    using V = typename ValuesView::value_type;
    View<V*> tmp("binsort_tmp", values.size());
    check(gbk_permute((int)sizeof(V), values.data(), perm_.data(), values.size(), tmp.data(), ex.handle()),
          "BinSort::sort");
    check(gbk_deep_copy(values.data(), tmp.data(), (int64_t)(sizeof(V) * values.size()), ex.handle()),
          "BinSort::sort");
    ex.fence();
  }
  template <class ValuesView>
  void sort(const ValuesView& values) const {
    sort(Experimental::GB300(), values);
  }
  const offset_type& get_bin_offsets() const { return offsets_; }
  const offset_type& get_permute_vector() const { return perm_; }
  const bin_count_type& get_bin_count() const { return counts_; }

 private:
  KeyViewType keys_;
  BinSortOp op_;
  bool within_;
  bin_count_type counts_;
  offset_type offsets_;
  offset_type perm_;
};

}  // namespace gb300k
