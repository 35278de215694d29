// std-algorithm reduce / inclusive_scan / exclusive_scan over contiguous
// views (algorithms/src/std_algorithms/Kokkos_Reduce.hpp,
// Kokkos_InclusiveScan.hpp, Kokkos_ExclusiveScan.hpp; impl files
// impl/Kokkos_Reduce.hpp:86-152, impl/Kokkos_ExclusiveScan.hpp:37-122,
// impl/Kokkos_InclusiveScan.hpp:85-360), routed to the typed C ABI, and
// Experimental::Graph (core/src/Kokkos_Graph.hpp:42-183,
// Kokkos_GraphNode.hpp:227-470) built by stream capture.
#pragma once

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
