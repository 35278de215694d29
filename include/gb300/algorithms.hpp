// std-algorithm reduce / inclusive_scan / exclusive_scan over contiguous
// views (algorithms/src/std_algorithms/Kokkos_Reduce.hpp,
// Kokkos_InclusiveScan.hpp, Kokkos_ExclusiveScan.hpp; impl files
// impl/Kokkos_Reduce.hpp:86-152, impl/Kokkos_ExclusiveScan.hpp:37-122,
// impl/Kokkos_InclusiveScan.hpp:85-360), routed to the typed C ABI, and
// Experimental::Graph (core/src/Kokkos_Graph.hpp:42-183,
// Kokkos_GraphNode.hpp:227-470) built by stream capture.
#pragma once

#include <utility>

#include "scan.hpp"
#include "scatter_sort.hpp"

namespace gb300k {
namespace Experimental {

// Random-access position in a contiguous view: begin(v) + k.
template <class T>
struct ViewIter {
  T* p;
  int64_t i;
  ViewIter operator+(int64_t k) const { return {p, i + k}; }
  ViewIter operator-(int64_t k) const { return {p, i - k}; }
  int64_t operator-(const ViewIter& o) const { return i - o.i; }
  T* ptr() const { return p + i; }
};
template <class D, class... P>
ViewIter<typename View<D, P...>::value_type> begin(const View<D, P...>& v) { return {v.data(), 0}; }
template <class D, class... P>
ViewIter<typename View<D, P...>::value_type> end(const View<D, P...>& v) { return {v.data(), v.size()}; }
template <class D, class... P>
ViewIter<typename View<D, P...>::value_type> cbegin(const View<D, P...>& v) { return begin(v); }
template <class D, class... P>
ViewIter<typename View<D, P...>::value_type> cend(const View<D, P...>& v) { return end(v); }
template <class T>
int64_t distance(const ViewIter<T>& a, const ViewIter<T>& b) { return b - a; }

// reduce(ex, first, last, init) = init + sum of [first, last), in the init's
// type when it matches the elements (the default functor of
// impl/Kokkos_Reduce.hpp:31-41).
template <class T, class V>
V reduce(const GB300& ex, ViewIter<T> first, ViewIter<T> last, V init) {
  using E = std::remove_const_t<T>;
  E r{};
  E* d = nullptr;
  check_cuda(cudaMallocAsync((void**)&d, sizeof(E), ex.stream()), "reduce");
  check(gbk_reduce(GBK_SUM, (gbk_dtype_t)Impl::dtype_code<E>::value, first.ptr(), last - first, d, ex.handle(), nullptr),
        "Kokkos::Experimental::reduce");
  check_cuda(cudaMemcpyAsync(&r, d, sizeof(E), cudaMemcpyDeviceToHost, ex.stream()), "reduce");
  check_cuda(cudaFreeAsync(d, ex.stream()), "reduce");
  ex.fence();
  return init + (V)r;
}
template <class T>
std::remove_const_t<T> reduce(const GB300& ex, ViewIter<T> first, ViewIter<T> last) {
  return reduce(ex, first, last, std::remove_const_t<T>(0));
}
template <class D, class... P, class V>
V reduce(const GB300& ex, const View<D, P...>& v, V init) {
  return reduce(ex, begin(v), end(v), init);
}
template <class D, class... P>
auto reduce(const GB300& ex, const View<D, P...>& v) {
  return reduce(ex, begin(v), end(v));
}

// exclusive_scan(ex, first, last, dest, init): dest[i] = init + sum [0, i),
// accumulated in the init's type (int32 in -> int64 out widens).
template <class TI, class TO, class V>
ViewIter<TO> exclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, V init) {
  using EI = std::remove_const_t<TI>;
  using EO = std::remove_const_t<TO>;
  EO iv = (EO)init;
  check(gbk_scan(0, (gbk_dtype_t)Impl::dtype_code<EI>::value, (gbk_dtype_t)Impl::dtype_code<EO>::value, first.ptr(),
                 last - first, &iv, dest.ptr(), nullptr, ex.handle(), nullptr),
        "Kokkos::Experimental::exclusive_scan");
  ex.fence();
  return dest + (last - first);
}
template <class TI, class TO>
ViewIter<TO> inclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest) {
  using EI = std::remove_const_t<TI>;
  using EO = std::remove_const_t<TO>;
  check(gbk_scan(1, (gbk_dtype_t)Impl::dtype_code<EI>::value, (gbk_dtype_t)Impl::dtype_code<EO>::value, first.ptr(),
                 last - first, nullptr, dest.ptr(), nullptr, ex.handle(), nullptr),
        "Kokkos::Experimental::inclusive_scan");
  ex.fence();
  return dest + (last - first);
}
template <class D1, class... P1, class D2, class... P2, class V>
auto exclusive_scan(const GB300& ex, const View<D1, P1...>& src, const View<D2, P2...>& dst, V init) {
  return exclusive_scan(ex, begin(src), end(src), begin(dst), init);
}
template <class D1, class... P1, class D2, class... P2>
auto inclusive_scan(const GB300& ex, const View<D1, P1...>& src, const View<D2, P2...>& dst) {
  return inclusive_scan(ex, begin(src), end(src), begin(dst));
}

// ---- min_element / max_element / minmax_element ------------------------------
// (algorithms/src/std_algorithms/impl/Kokkos_MinMaxMinmaxElement.hpp): the
// first smallest / first largest element, and (first smallest, last
// largest) for minmax_element.  Arithmetic elements without a comparator
// take the typed MinLoc / MaxLoc reduce of the C ABI (first occurrence on
// ties); a comparator goes through the header reduce with the
// *FirstLoc*CustomComparator reducers.  An empty range returns last.
namespace StdImpl {
template <class T, class Red>
struct ElemLocFn {
  const T* p;
  Red red;
  __device__ void operator()(int64_t i, typename Red::value_type& u) const {
    typename Red::value_type t{p[i], i};
    red.join(u, t);
  }
};
template <class T, class Red>
struct ElemMinMaxLocFn {
  const T* p;
  Red red;
  __device__ void operator()(int64_t i, typename Red::value_type& u) const {
    typename Red::value_type t{p[i], p[i], i, i};
    red.join(u, t);
  }
};
template <class T, class = void> struct has_dtype : std::false_type {};
template <class T> struct has_dtype<T, std::void_t<decltype(gb300k::Impl::dtype_code<T>::value)>> : std::true_type {};
template <class E>
int64_t typed_loc(const GB300& ex, int op, const E* p, int64_t n, const char* what) {
  gbk::ValLoc<E> r{};
  gbk::ValLoc<E>* d = nullptr;
  check_cuda(cudaMallocAsync((void**)&d, sizeof(r), ex.stream()), what);
  check(gbk_reduce((gbk_reducer_t)op, (gbk_dtype_t)gb300k::Impl::dtype_code<E>::value, p, n, d, ex.handle(), nullptr), what);
  check_cuda(cudaMemcpyAsync(&r, d, sizeof(r), cudaMemcpyDeviceToHost, ex.stream()), what);
  check_cuda(cudaFreeAsync(d, ex.stream()), what);
  ex.fence();
  return r.loc;
}
}  // namespace StdImpl

template <class T, class Comp>
ViewIter<T> min_element(const GB300& ex, ViewIter<T> first, ViewIter<T> last, Comp comp) {
  using E = std::remove_const_t<T>;
  const int64_t n = last - first;
  if (n <= 0) return last;
  ValLocScalar<E, int64_t> r;
  MinFirstLocCustomComparator<E, int64_t, Comp> red(r, comp);
  parallel_reduce(RangePolicy<GB300>(ex, 0, n), StdImpl::ElemLocFn<E, decltype(red)>{first.ptr(), red}, red);
  return first + r.loc;
}
template <class T, class Comp>
ViewIter<T> max_element(const GB300& ex, ViewIter<T> first, ViewIter<T> last, Comp comp) {
  using E = std::remove_const_t<T>;
  const int64_t n = last - first;
  if (n <= 0) return last;
  ValLocScalar<E, int64_t> r;
  MaxFirstLocCustomComparator<E, int64_t, Comp> red(r, comp);
  parallel_reduce(RangePolicy<GB300>(ex, 0, n), StdImpl::ElemLocFn<E, decltype(red)>{first.ptr(), red}, red);
  return first + r.loc;
}
template <class T>
ViewIter<T> min_element(const GB300& ex, ViewIter<T> first, ViewIter<T> last) {
  using E = std::remove_const_t<T>;
  if constexpr (StdImpl::has_dtype<E>::value) {
    const int64_t n = last - first;
    if (n <= 0) return last;
    return first + StdImpl::typed_loc<E>(ex, GBK_MINLOC, first.ptr(), n, "Kokkos::Experimental::min_element");
  } else {
    return min_element(ex, first, last, Impl::Less{});
  }
}
template <class T>
ViewIter<T> max_element(const GB300& ex, ViewIter<T> first, ViewIter<T> last) {
  using E = std::remove_const_t<T>;
  if constexpr (StdImpl::has_dtype<E>::value) {
    const int64_t n = last - first;
    if (n <= 0) return last;
    return first + StdImpl::typed_loc<E>(ex, GBK_MAXLOC, first.ptr(), n, "Kokkos::Experimental::max_element");
  } else {
    return max_element(ex, first, last, Impl::Less{});
  }
}
template <class T, class Comp = Impl::Less>
std::pair<ViewIter<T>, ViewIter<T>> minmax_element(const GB300& ex, ViewIter<T> first, ViewIter<T> last,
                                                   Comp comp = Comp()) {
  using E = std::remove_const_t<T>;
  const int64_t n = last - first;
  if (n <= 0) return {last, last};
  MinMaxLocScalar<E, int64_t> r;
  MinMaxFirstLastLocCustomComparator<E, int64_t, Comp> red(r, comp);
  parallel_reduce(RangePolicy<GB300>(ex, 0, n), StdImpl::ElemMinMaxLocFn<E, decltype(red)>{first.ptr(), red}, red);
  return {first + r.min_loc, first + r.max_loc};
}
template <class D, class... P, class... C>
auto min_element(const GB300& ex, const View<D, P...>& v, C... comp) {
  return min_element(ex, begin(v), end(v), comp...);
}
template <class D, class... P, class... C>
auto max_element(const GB300& ex, const View<D, P...>& v, C... comp) {
  return max_element(ex, begin(v), end(v), comp...);
}
template <class D, class... P, class... C>
auto minmax_element(const GB300& ex, const View<D, P...>& v, C... comp) {
  return minmax_element(ex, begin(v), end(v), comp...);
}

// ---- transform_reduce and reduce with a joiner -----------------------------
// (algorithms/src/std_algorithms/impl/Kokkos_TransformReduce.hpp:117-220,
// impl/Kokkos_Reduce.hpp): joiner(reduction of transform(x), init); an
// empty range returns init.  The joiner needs no neutral element (the
// values carry a "has a value" flag).  The two-range form without functors
// is init + sum of first1[i] * first2[i].
namespace StdImpl {
template <class V, class T, class U, class J>
struct UnaryJoinFn {
  const T* p;
  U u;
  J j;
  __device__ void operator()(int64_t i, gb300k::Impl::Opt<V>& acc) const {
    const V t = (V)u(p[i]);
    acc.val = acc.has ? (V)j(acc.val, t) : t;
    acc.has = 1;
  }
};
template <class V, class T1, class T2, class B, class J>
struct BinaryJoinFn {
  const T1* a;
  const T2* b;
  B bt;
  J j;
  __device__ void operator()(int64_t i, gb300k::Impl::Opt<V>& acc) const {
    const V t = (V)bt(a[i], b[i]);
    acc.val = acc.has ? (V)j(acc.val, t) : t;
    acc.has = 1;
  }
};
template <class V, class T1, class T2>
struct DotFn {
  const T1* a;
  const T2* b;
  __device__ void operator()(int64_t i, V& acc) const { acc += (V)(a[i] * b[i]); }
};
struct Identity {
  template <class T>
  __host__ __device__ T operator()(const T& x) const { return x; }
};
}  // namespace StdImpl

template <class T, class V, class J, class U>
V transform_reduce(const GB300& ex, ViewIter<T> first, ViewIter<T> last, V init, J joiner, U transformer) {
  const int64_t n = last - first;
  if (n <= 0) return init;
  Impl::Opt<V> r{};
  Impl::OptJoin<V, J> red(r, joiner);
  parallel_reduce(RangePolicy<GB300>(ex, 0, n),
                  StdImpl::UnaryJoinFn<V, std::remove_const_t<T>, U, J>{first.ptr(), transformer, joiner}, red);
  return joiner(r.val, init);
}
template <class T1, class T2, class V, class J, class B>
V transform_reduce(const GB300& ex, ViewIter<T1> first1, ViewIter<T1> last1, ViewIter<T2> first2, V init, J joiner,
                   B transformer) {
  const int64_t n = last1 - first1;
  if (n <= 0) return init;
  Impl::Opt<V> r{};
  Impl::OptJoin<V, J> red(r, joiner);
  parallel_reduce(RangePolicy<GB300>(ex, 0, n),
                  StdImpl::BinaryJoinFn<V, std::remove_const_t<T1>, std::remove_const_t<T2>, B, J>{
                      first1.ptr(), first2.ptr(), transformer, joiner},
                  red);
  return joiner(r.val, init);
}
template <class T1, class T2, class V>
V transform_reduce(const GB300& ex, ViewIter<T1> first1, ViewIter<T1> last1, ViewIter<T2> first2, V init) {
  const int64_t n = last1 - first1;
  if (n <= 0) return init;
  V r = V(0);
  parallel_reduce(RangePolicy<GB300>(ex, 0, n),
                  StdImpl::DotFn<V, std::remove_const_t<T1>, std::remove_const_t<T2>>{first1.ptr(), first2.ptr()}, r);
  return r + init;
}
template <class T, class V, class J>
V reduce(const GB300& ex, ViewIter<T> first, ViewIter<T> last, V init, J joiner) {
  return transform_reduce(ex, first, last, init, joiner, StdImpl::Identity{});
}
template <class D, class... P, class V, class J, class U>
V transform_reduce(const GB300& ex, const View<D, P...>& v, V init, J joiner, U transformer) {
  return transform_reduce(ex, begin(v), end(v), init, joiner, transformer);
}
template <class D1, class... P1, class D2, class... P2, class V, class J, class B>
V transform_reduce(const GB300& ex, const View<D1, P1...>& a, const View<D2, P2...>& b, V init, J joiner,
                   B transformer) {
  return transform_reduce(ex, begin(a), end(a), begin(b), init, joiner, transformer);
}
template <class D1, class... P1, class D2, class... P2, class V>
V transform_reduce(const GB300& ex, const View<D1, P1...>& a, const View<D2, P2...>& b, V init) {
  return transform_reduce(ex, begin(a), end(a), begin(b), init);
}
template <class D, class... P, class V, class J>
V reduce(const GB300& ex, const View<D, P...>& v, V init, J joiner) {
  return reduce(ex, begin(v), end(v), init, joiner);
}

// ---- scans with a binary op, transform scans --------------------------------
// (impl/Kokkos_TransformExclusiveScan.hpp, impl/Kokkos_TransformInclusiveScan.hpp,
// impl/Kokkos_FunctorsForExclusiveScan.hpp:110-206): the header scan kernel
// with an ordered join on (value, has-value) records, so the binary op needs
// no neutral element and is applied in index order.  Exclusive: dest[0] =
// init, dest[i] = bop(op-prefix of uop(x[0..i)), init); inclusive: dest[i] =
// op-prefix of uop(x[0..i]), or bop(init, that) when an init is given.
namespace StdImpl {
template <class V, class B>
struct OptScanJ {
  B bop;
  __device__ gb300k::Impl::Opt<V> zero() const { return gb300k::Impl::Opt<V>{V(), 0}; }
  __device__ gb300k::Impl::Opt<V> add(const gb300k::Impl::Opt<V>& a, const gb300k::Impl::Opt<V>& b) const {
    if (!a.has) return b;
    if (!b.has) return a;
    return gb300k::Impl::Opt<V>{(V)bop(a.val, b.val), 1};
  }
};
template <class V, class TI, class TO, class B, class U>
struct TExclFn {
  const TI* x;
  TO* y;
  V init;
  B bop;
  U uop;
  __device__ void operator()(int64_t i, gb300k::Impl::Opt<V>& u, bool fin) const {
    if (fin) y[i] = u.has ? (TO)bop(u.val, init) : (TO)init;
    const V t = (V)uop(x[i]);
    u.val = u.has ? (V)bop(u.val, t) : t;
    u.has = 1;
  }
};
template <class V, class TI, class TO, class B, class U, bool INIT>
struct TInclFn {
  const TI* x;
  TO* y;
  V init;
  B bop;
  U uop;
  __device__ void operator()(int64_t i, gb300k::Impl::Opt<V>& u, bool fin) const {
    const V t = (V)uop(x[i]);
    u.val = u.has ? (V)bop(u.val, t) : t;
    u.has = 1;
    if (fin) y[i] = INIT ? (TO)bop(init, u.val) : (TO)u.val;
  }
};
}  // namespace StdImpl

template <class TI, class TO, class V, class B, class U>
ViewIter<TO> transform_exclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, V init,
                                      B bop, U uop) {
  const int64_t n = last - first;
  StdImpl::TExclFn<V, std::remove_const_t<TI>, TO, B, U> f{first.ptr(), dest.ptr(), init, bop, uop};
  parallel_scan_impl<Impl::Opt<V>>(RangePolicy<GB300>(ex, 0, n), f, nullptr, StdImpl::OptScanJ<V, B>{bop});
  ex.fence();
  return dest + n;
}
template <class TI, class TO, class B, class U>
ViewIter<TO> transform_inclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, B bop,
                                      U uop) {
  using V = std::remove_const_t<TO>;
  const int64_t n = last - first;
  StdImpl::TInclFn<V, std::remove_const_t<TI>, TO, B, U, false> f{first.ptr(), dest.ptr(), V(), bop, uop};
  parallel_scan_impl<Impl::Opt<V>>(RangePolicy<GB300>(ex, 0, n), f, nullptr, StdImpl::OptScanJ<V, B>{bop});
  ex.fence();
  return dest + n;
}
template <class TI, class TO, class B, class U, class V>
ViewIter<TO> transform_inclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, B bop,
                                      U uop, V init) {
  const int64_t n = last - first;
  StdImpl::TInclFn<V, std::remove_const_t<TI>, TO, B, U, true> f{first.ptr(), dest.ptr(), init, bop, uop};
  parallel_scan_impl<Impl::Opt<V>>(RangePolicy<GB300>(ex, 0, n), f, nullptr, StdImpl::OptScanJ<V, B>{bop});
  ex.fence();
  return dest + n;
}
// exclusive_scan / inclusive_scan with a binary op (no transform).
template <class TI, class TO, class V, class B>
ViewIter<TO> exclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, V init, B bop) {
  return transform_exclusive_scan(ex, first, last, dest, init, bop, StdImpl::Identity{});
}
template <class TI, class TO, class B>
ViewIter<TO> inclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, B bop) {
  return transform_inclusive_scan(ex, first, last, dest, bop, StdImpl::Identity{});
}
template <class TI, class TO, class B, class V>
ViewIter<TO> inclusive_scan(const GB300& ex, ViewIter<TI> first, ViewIter<TI> last, ViewIter<TO> dest, B bop, V init) {
  return transform_inclusive_scan(ex, first, last, dest, bop, StdImpl::Identity{}, init);
}
template <class D1, class... P1, class D2, class... P2, class V, class B, class U>
auto transform_exclusive_scan(const GB300& ex, const View<D1, P1...>& src, const View<D2, P2...>& dst, V init, B bop,
                              U uop) {
  return transform_exclusive_scan(ex, begin(src), end(src), begin(dst), init, bop, uop);
}
template <class D1, class... P1, class D2, class... P2, class B, class U, class... V>
auto transform_inclusive_scan(const GB300& ex, const View<D1, P1...>& src, const View<D2, P2...>& dst, B bop, U uop,
                              V... init) {
  return transform_inclusive_scan(ex, begin(src), end(src), begin(dst), bop, uop, init...);
}

// ---- Graph ----------------------------------------------------------------
// create_graph(ex, [&](auto root){ root.then_parallel_for(...).then_parallel_reduce(...); })
// captures the nodes' launches on ex's stream into one CUDA graph; each node
// depends on the one it was chained from (a chain).  Reduce nodes write
// their result into a View (no host result inside a graph, as in the
// reference); submit() replays the graph on ex's stream.
class Graph {
 public:
  Graph() = default;
  Graph(const GB300& ex, gbk_graph_t h) : ex_(ex), h_(h) {}
  Graph(Graph&& o) noexcept : ex_(o.ex_), h_(o.h_) { o.h_ = nullptr; }
  Graph& operator=(Graph&& o) noexcept {
    std::swap(h_, o.h_);
    ex_ = o.ex_;
    return *this;
  }
  Graph(const Graph&) = delete;
  ~Graph() {
    if (h_) gbk_graph_destroy(h_);
  }
  void submit() const { check(gbk_graph_launch(h_, ex_.handle()), "Graph::submit"); }
  void submit(const GB300& ex) const { check(gbk_graph_launch(h_, ex.handle()), "Graph::submit"); }

 private:
  GB300 ex_;
  gbk_graph_t h_ = nullptr;
};

class GraphNodeRef {
 public:
  explicit GraphNodeRef(const GB300& ex) : ex_(ex) {}
  template <class F>
  GraphNodeRef then_parallel_for(int64_t n, const F& f) const {
    parallel_for(RangePolicy<GB300>(ex_, 0, n), f);
    return *this;
  }
  template <class P, class F>
  GraphNodeRef then_parallel_for(const P& p, const F& f) const {
    parallel_for(with_space(p), f);
    return *this;
  }
  template <class F, class Red>
  GraphNodeRef then_parallel_reduce(int64_t n, const F& f, const Red& red) const {
    static_assert(Impl::is_reducer<Red>::value, "graph reduce nodes take a reducer on a View");
    if (!red.res.device) Impl::abort_msg("graph reduce nodes write their result into a device View");
    parallel_reduce(RangePolicy<GB300>(ex_, 0, n), f, red);
    return *this;
  }
  template <class F>
  GraphNodeRef then_parallel_scan(int64_t n, const F& f) const {
    parallel_scan(RangePolicy<GB300>(ex_, 0, n), f);
    return *this;
  }
  // then(): any sequence of library calls on ex's stream (the reference's
  // cuda_capture node, Kokkos_GraphNode.hpp:259).
  template <class F>
  GraphNodeRef then(const F& f) const {
    f(ex_);
    return *this;
  }
  const GB300& space() const { return ex_; }

 private:
  template <class E, class... R>
  RangePolicy<GB300> with_space(const RangePolicy<E, R...>& p) const {
    return RangePolicy<GB300>(ex_, p.begin(), p.end());
  }
  GB300 ex_;
};

template <class Closure>
Graph create_graph(const GB300& ex, Closure&& closure, int64_t workspace_bytes = 64 << 20) {
  if (!ex.stream()) Impl::abort_msg("create_graph: the execution space needs its own (non-default) stream");
  check(gbk_workspace_reserve(ex.handle(), workspace_bytes), "create_graph");
  check(gbk_graph_begin(ex.handle()), "create_graph");
  try {
    closure(GraphNodeRef(ex));
  } catch (...) {
    gbk_graph_t dummy = nullptr;
    gbk_graph_end(ex.handle(), &dummy);
    if (dummy) gbk_graph_destroy(dummy);
    throw;
  }
  gbk_graph_t h = nullptr;
  check(gbk_graph_end(ex.handle(), &h), "create_graph");
  return Graph(ex, h);
}

}  // namespace Experimental
}  // namespace gb300k
