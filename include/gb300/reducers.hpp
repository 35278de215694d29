// Built-in reducers of the header-template path, with the reference's names,
// value layouts and identities (core/src/Kokkos_Parallel_Reduce.hpp:34-650,
// core/src/Kokkos_ReductionIdentity.hpp:30-398).  A reducer refers to its
// result: a host scalar (the call fences and copies the value back) or a
// rank-0-like View of one element in device memory (no fence).  init/join
// are the library's device reducers (kokkos_gb300/csrc/gbk_internal.cuh),
// so the header path and the typed C ABI reduce with the same rules: a
// *Loc join keeps the smaller loc on equal values.
#pragma once

#include <limits>

#include "../../kokkos_gb300/csrc/gbk_internal.cuh"
#include "core.hpp"

namespace gb300k {

template <class Scalar, class Index>
struct ValLocScalar {
  Scalar val;
  Index loc;
};
template <class Scalar>
struct MinMaxScalar {
  Scalar min_val, max_val;
};
template <class Scalar, class Index>
struct MinMaxLocScalar {
  Scalar min_val, max_val;
  Index min_loc, max_loc;
};

namespace Impl {
template <class T> struct DevR;  // scalar reducer -> library device reducer
// reduction_identity<Index>::min() of the reference: the index type's maximum
template <class I>
__host__ __device__ constexpr I loc_identity() {
  return gbk::lim<I>::hi();
}

// Result target of a reducer: host scalar or device memory.
template <class V>
struct ResultRef {
  V* ptr = nullptr;
  bool device = false;
};

template <class Derived, class V>
struct ReducerBase {
  using value_type = V;
  ResultRef<V> res;
  __host__ __device__ ReducerBase(V& r) { res.ptr = &r; res.device = false; }
  template <class D, class... P>
  ReducerBase(const View<D, P...>& v) {
    res.ptr = v.data();
    res.device = View<D, P...>::is_device;
  }
  __host__ __device__ V& reference() const { return *res.ptr; }
};
}  // namespace Impl

#define GBK_SCALAR_REDUCER(NAME, DEV)                                                                        \
  template <class T, class Space = GB300Space>                                                              \
  struct NAME : Impl::ReducerBase<NAME<T, Space>, T> {                                                      \
    using reducer = NAME;                                                                                   \
    using value_type = T;                                                                                   \
    __host__ __device__ NAME(T& r) : Impl::ReducerBase<NAME<T, Space>, T>(r) {}                             \
    template <class D, class... P>                                                                          \
    NAME(const View<D, P...>& v) : Impl::ReducerBase<NAME<T, Space>, T>(v) {}                               \
    __device__ void init(T& v) const { v = gbk::DEV<T>::init(); }                                           \
    __device__ void join(T& a, const T& b) const { gbk::DEV<T>::join(a, b); }                               \
  };
GBK_SCALAR_REDUCER(Sum, RSum)
GBK_SCALAR_REDUCER(Prod, RProd)
GBK_SCALAR_REDUCER(Min, RMin)
GBK_SCALAR_REDUCER(Max, RMax)
GBK_SCALAR_REDUCER(LAnd, RLAnd)
GBK_SCALAR_REDUCER(LOr, RLOr)
GBK_SCALAR_REDUCER(BAnd, RBAnd)
GBK_SCALAR_REDUCER(BOr, RBOr)
#undef GBK_SCALAR_REDUCER

// MinLoc / MaxLoc (Kokkos_Parallel_Reduce.hpp:412-530): value = {val, loc}.
template <class T, class I = int, class Space = GB300Space>
struct MinLoc : Impl::ReducerBase<MinLoc<T, I, Space>, ValLocScalar<T, I>> {
  using V = ValLocScalar<T, I>;
  using reducer = MinLoc;
  using value_type = V;
  __host__ __device__ MinLoc(V& r) : Impl::ReducerBase<MinLoc, V>(r) {}
  template <class D, class... P>
  MinLoc(const View<D, P...>& v) : Impl::ReducerBase<MinLoc, V>(v) {}
  __device__ void init(V& v) const { v.val = gbk::lim<T>::hi(); v.loc = Impl::loc_identity<I>(); }
  __device__ void join(V& a, const V& b) const {
    if (b.val < a.val || (b.val == a.val && b.loc < a.loc)) a = b;
  }
};
template <class T, class I = int, class Space = GB300Space>
struct MaxLoc : Impl::ReducerBase<MaxLoc<T, I, Space>, ValLocScalar<T, I>> {
  using V = ValLocScalar<T, I>;
  using reducer = MaxLoc;
  using value_type = V;
  __host__ __device__ MaxLoc(V& r) : Impl::ReducerBase<MaxLoc, V>(r) {}
  template <class D, class... P>
  MaxLoc(const View<D, P...>& v) : Impl::ReducerBase<MaxLoc, V>(v) {}
  __device__ void init(V& v) const { v.val = gbk::lim<T>::lo(); v.loc = Impl::loc_identity<I>(); }
  __device__ void join(V& a, const V& b) const {
    if (b.val > a.val || (b.val == a.val && b.loc < a.loc)) a = b;
  }
};
// MinMax (Kokkos_Parallel_Reduce.hpp:537-600)
template <class T, class Space = GB300Space>
struct MinMax : Impl::ReducerBase<MinMax<T, Space>, MinMaxScalar<T>> {
  using V = MinMaxScalar<T>;
  using reducer = MinMax;
  using value_type = V;
  __host__ __device__ MinMax(V& r) : Impl::ReducerBase<MinMax, V>(r) {}
  template <class D, class... P>
  MinMax(const View<D, P...>& v) : Impl::ReducerBase<MinMax, V>(v) {}
  __device__ void init(V& v) const { v.min_val = gbk::lim<T>::hi(); v.max_val = gbk::lim<T>::lo(); }
  __device__ void join(V& a, const V& b) const {
    if (b.min_val < a.min_val) a.min_val = b.min_val;
    if (b.max_val > a.max_val) a.max_val = b.max_val;
  }
};
// MinMaxLoc (Kokkos_Parallel_Reduce.hpp:601-650)
template <class T, class I = int, class Space = GB300Space>
struct MinMaxLoc : Impl::ReducerBase<MinMaxLoc<T, I, Space>, MinMaxLocScalar<T, I>> {
  using V = MinMaxLocScalar<T, I>;
  using reducer = MinMaxLoc;
  using value_type = V;
  __host__ __device__ MinMaxLoc(V& r) : Impl::ReducerBase<MinMaxLoc, V>(r) {}
  template <class D, class... P>
  MinMaxLoc(const View<D, P...>& v) : Impl::ReducerBase<MinMaxLoc, V>(v) {}
  __device__ void init(V& v) const {
    v.min_val = gbk::lim<T>::hi();
    v.max_val = gbk::lim<T>::lo();
    v.min_loc = v.max_loc = Impl::loc_identity<I>();
  }
  __device__ void join(V& a, const V& b) const {
    if (b.min_val < a.min_val || (b.min_val == a.min_val && b.min_loc < a.min_loc)) { a.min_val = b.min_val; a.min_loc = b.min_loc; }
    if (b.max_val > a.max_val || (b.max_val == a.max_val && b.max_loc < a.max_loc)) { a.max_val = b.max_val; a.max_loc = b.max_loc; }
  }
};

// Reducers of the std min_element / max_element / minmax_element
// (Kokkos_Parallel_Reduce.hpp:679-1100): equal values keep the smaller loc,
// except the max of MinMaxFirstLastLoc, which keeps the larger (std
// minmax_element returns the last largest element).  Comp(a, b) = "a is
// less than b" (std::less by default); the reducer's identity is an empty
// record (loc = the index type's maximum, or minimum for the last-loc max),
// joined by loc only when the values are equivalent.
namespace Impl {
struct Less {
  template <class T>
  __host__ __device__ bool operator()(const T& a, const T& b) const { return a < b; }
};
}  // namespace Impl

template <class T, class I = int64_t, class Comp = Impl::Less, class Space = GB300Space>
struct MinFirstLocCustomComparator : Impl::ReducerBase<MinFirstLocCustomComparator<T, I, Comp, Space>, ValLocScalar<T, I>> {
  using V = ValLocScalar<T, I>;
  using reducer = MinFirstLocCustomComparator;
  using value_type = V;
  Comp comp;
  __host__ __device__ MinFirstLocCustomComparator(V& r, Comp c = Comp()) : Impl::ReducerBase<MinFirstLocCustomComparator, V>(r), comp(c) {}
  template <class D, class... P>
  MinFirstLocCustomComparator(const View<D, P...>& v, Comp c = Comp()) : Impl::ReducerBase<MinFirstLocCustomComparator, V>(v), comp(c) {}
  __device__ void init(V& v) const { v.val = gbk::lim<T>::hi(); v.loc = Impl::loc_identity<I>(); }
  __device__ void join(V& a, const V& b) const {
    if (b.loc == Impl::loc_identity<I>()) return;
    if (a.loc == Impl::loc_identity<I>() || comp(b.val, a.val)) { a = b; return; }
    if (!comp(a.val, b.val) && b.loc < a.loc) a.loc = b.loc;
  }
};
template <class T, class I = int64_t, class Comp = Impl::Less, class Space = GB300Space>
struct MaxFirstLocCustomComparator : Impl::ReducerBase<MaxFirstLocCustomComparator<T, I, Comp, Space>, ValLocScalar<T, I>> {
  using V = ValLocScalar<T, I>;
  using reducer = MaxFirstLocCustomComparator;
  using value_type = V;
  Comp comp;
  __host__ __device__ MaxFirstLocCustomComparator(V& r, Comp c = Comp()) : Impl::ReducerBase<MaxFirstLocCustomComparator, V>(r), comp(c) {}
  template <class D, class... P>
  MaxFirstLocCustomComparator(const View<D, P...>& v, Comp c = Comp()) : Impl::ReducerBase<MaxFirstLocCustomComparator, V>(v), comp(c) {}
  __device__ void init(V& v) const { v.val = gbk::lim<T>::lo(); v.loc = Impl::loc_identity<I>(); }
  __device__ void join(V& a, const V& b) const {
    if (b.loc == Impl::loc_identity<I>()) return;
    if (a.loc == Impl::loc_identity<I>() || comp(a.val, b.val)) { a = b; return; }
    if (!comp(b.val, a.val) && b.loc < a.loc) a.loc = b.loc;
  }
};
template <class T, class I = int64_t, class Comp = Impl::Less, class Space = GB300Space>
struct MinMaxFirstLastLocCustomComparator
    : Impl::ReducerBase<MinMaxFirstLastLocCustomComparator<T, I, Comp, Space>, MinMaxLocScalar<T, I>> {
  using V = MinMaxLocScalar<T, I>;
  using reducer = MinMaxFirstLastLocCustomComparator;
  using value_type = V;
  Comp comp;
  __host__ __device__ MinMaxFirstLastLocCustomComparator(V& r, Comp c = Comp())
      : Impl::ReducerBase<MinMaxFirstLastLocCustomComparator, V>(r), comp(c) {}
  template <class D, class... P>
  MinMaxFirstLastLocCustomComparator(const View<D, P...>& v, Comp c = Comp())
      : Impl::ReducerBase<MinMaxFirstLastLocCustomComparator, V>(v), comp(c) {}
  __device__ void init(V& v) const {
    v.min_val = gbk::lim<T>::hi();
    v.max_val = gbk::lim<T>::lo();
    v.min_loc = Impl::loc_identity<I>();
    v.max_loc = gbk::lim<I>::lo();
  }
  __device__ void join(V& a, const V& b) const {
    if (b.min_loc != Impl::loc_identity<I>()) {
      if (a.min_loc == Impl::loc_identity<I>() || comp(b.min_val, a.min_val)) {
        a.min_val = b.min_val;
        a.min_loc = b.min_loc;
      } else if (!comp(a.min_val, b.min_val) && b.min_loc < a.min_loc) {
        a.min_loc = b.min_loc;
      }
    }
    if (b.max_loc != gbk::lim<I>::lo()) {
      if (a.max_loc == gbk::lim<I>::lo() || comp(a.max_val, b.max_val)) {
        a.max_val = b.max_val;
        a.max_loc = b.max_loc;
      } else if (!comp(b.max_val, a.max_val) && b.max_loc > a.max_loc) {
        a.max_loc = b.max_loc;
      }
    }
  }
};
template <class T, class I = int64_t, class Space = GB300Space>
using MinFirstLoc = MinFirstLocCustomComparator<T, I, Impl::Less, Space>;
template <class T, class I = int64_t, class Space = GB300Space>
using MaxFirstLoc = MaxFirstLocCustomComparator<T, I, Impl::Less, Space>;
template <class T, class I = int64_t, class Space = GB300Space>
using MinMaxFirstLastLoc = MinMaxFirstLastLocCustomComparator<T, I, Impl::Less, Space>;

// FirstLoc / LastLoc (Kokkos_Parallel_Reduce.hpp:1103-1220): the smallest /
// largest index at which the functor found its predicate true; the
// identities are the index type's largest / smallest value.
template <class I>
struct FirstLocScalar {
  I min_loc_true;
};
template <class I>
struct LastLocScalar {
  I max_loc_true;
};
template <class I, class Space = GB300Space>
struct FirstLoc : Impl::ReducerBase<FirstLoc<I, Space>, FirstLocScalar<I>> {
  static_assert(std::is_integral<I>::value, "FirstLoc takes an integral index type");
  using V = FirstLocScalar<I>;
  using reducer = FirstLoc;
  using value_type = V;
  __host__ __device__ FirstLoc(V& r) : Impl::ReducerBase<FirstLoc, V>(r) {}
  template <class D, class... P>
  FirstLoc(const View<D, P...>& v) : Impl::ReducerBase<FirstLoc, V>(v) {}
  __device__ void init(V& v) const { v.min_loc_true = gbk::lim<I>::hi(); }
  __device__ void join(V& a, const V& b) const {
    if (b.min_loc_true < a.min_loc_true) a.min_loc_true = b.min_loc_true;
  }
};
template <class I, class Space = GB300Space>
struct LastLoc : Impl::ReducerBase<LastLoc<I, Space>, LastLocScalar<I>> {
  static_assert(std::is_integral<I>::value, "LastLoc takes an integral index type");
  using V = LastLocScalar<I>;
  using reducer = LastLoc;
  using value_type = V;
  __host__ __device__ LastLoc(V& r) : Impl::ReducerBase<LastLoc, V>(r) {}
  template <class D, class... P>
  LastLoc(const View<D, P...>& v) : Impl::ReducerBase<LastLoc, V>(v) {}
  __device__ void init(V& v) const { v.max_loc_true = gbk::lim<I>::lo(); }
  __device__ void join(V& a, const V& b) const {
    if (b.max_loc_true > a.max_loc_true) a.max_loc_true = b.max_loc_true;
  }
};

namespace Impl {
// A custom joiner with no neutral element (std transform_reduce / reduce with
// a user joiner): the value carries a "has a value" flag, the identity is an
// empty value, and join applies the joiner only to two non-empty values
// (the reference's ReducerWithArbitraryJoinerNoNeutralElement).
template <class T>
struct Opt {
  T val;
  int has;
};
template <class T, class Op>
struct OptJoin : ReducerBase<OptJoin<T, Op>, Opt<T>> {
  using reducer = OptJoin;
  using value_type = Opt<T>;
  Op op;
  OptJoin(Opt<T>& r, Op o) : ReducerBase<OptJoin, Opt<T>>(r), op(o) {}
  __device__ void init(Opt<T>& v) const {
    v.val = T();
    v.has = 0;
  }
  __device__ void join(Opt<T>& a, const Opt<T>& b) const {
    if (!b.has) return;
    if (!a.has) {
      a = b;
      return;
    }
    a.val = op(a.val, b.val);
  }
};
}  // namespace Impl

namespace Impl {
// Is R a reducer class (has a nested `reducer` type)?
template <class R, class = void> struct is_reducer : std::false_type {};
template <class R> struct is_reducer<R, std::void_t<typename R::reducer>> : std::true_type {};

// Shuffle of any trivially-copyable value made of 4-byte words.
template <class V>
__device__ __forceinline__ V shfl_xor_any(const V& v, int m) {
  static_assert(sizeof(V) % 4 == 0, "reduction value size must be a multiple of 4 bytes");
  V r;
  const unsigned* s = reinterpret_cast<const unsigned*>(&v);
  unsigned* d = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(V) / 4); ++i) d[i] = __shfl_xor_sync(0xffffffffu, s[i], m);
  return r;
}

// CTA tree over a reducer object (warp butterfly, then one warp over the
// warp results); result valid in thread 0.  sm holds blockDim/32 values.
template <class Red, class V>
__device__ V block_reduce_obj(const Red& red, V v, V* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    V o = shfl_xor_any(v, m);
    red.join(v, o);
  }
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    if (lane < nw) v = sm[lane];
    else red.init(v);
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      V o = shfl_xor_any(v, m);
      red.join(v, o);
    }
  }
  __syncthreads();
  return v;
}
}  // namespace Impl

}  // namespace gb300k
