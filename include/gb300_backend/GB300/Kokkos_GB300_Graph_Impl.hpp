// Kokkos::Experimental::Graph on the GB300 space as one CUDA graph
// (the CUDA space's version: core/src/Cuda/Kokkos_Cuda_Graph_Impl.hpp, which
// builds kernel nodes one by one; the generic host version:
// core/src/impl/Kokkos_Default_Graph_Impl.hpp).
//
// The nodes keep Kokkos' generic node bookkeeping (each node runs its
// predecessors first, GraphNodeBackendSpecificDetails); this GraphImpl keeps
// the graph's sinks and, at instantiate(), runs every node once on the
// instance's stream under stream capture: each node's kernel becomes a node
// of a CUDA graph, in an order that respects every predecessor edge.
// submit() launches the instantiated graph on the given instance's stream,
// stream-ordered after the work already queued there (no fence).  The
// library workspace is reserved before the capture, since no device memory
// may be allocated while a stream is captured.  An instance on the legacy
// default stream (which cannot be captured) runs the nodes directly at each
// submit, as the generic implementation does.
//
// Kokkos_Graph.hpp includes each backend's graph header beside its own; with
// this backend kept outside the Kokkos tree, a translation unit that builds a
// Graph on GB300 includes this header after Kokkos_Graph.hpp.
#ifndef KOKKOS_GB300_GRAPH_IMPL_HPP_
#define KOKKOS_GB300_GRAPH_IMPL_HPP_

#include <Kokkos_Macros.hpp>
#if defined(KOKKOS_ENABLE_GB300)

#include <Kokkos_Graph.hpp>

#include <GB300/Kokkos_GB300.hpp>

#include <memory>
#include <set>

namespace Kokkos {
namespace Impl {

template <>
struct GraphImpl<Kokkos::Experimental::GB300> {
  using execution_space = Kokkos::Experimental::GB300;
  using root_node_impl_t =
      GraphNodeImpl<execution_space, Kokkos::Experimental::TypeErasedTag, Kokkos::Experimental::TypeErasedTag>;
  using aggregate_impl_t = GraphNodeAggregateDefaultImpl<execution_space>;
  using node_details_t = GraphNodeBackendSpecificDetails<execution_space>;

  // device memory the library may need for the nodes' kernels, reserved
  // before the capture
  static constexpr int64_t kWorkspaceBytes = int64_t(64) << 20;

  GraphImpl() = default;
  explicit GraphImpl(execution_space space) : m_space(std::move(space)) {}
  GraphImpl(GraphImpl const&) = delete;
  GraphImpl(GraphImpl&&) = delete;
  GraphImpl& operator=(GraphImpl const&) = delete;
  GraphImpl& operator=(GraphImpl&&) = delete;
  ~GraphImpl() {
    if (m_exec) cudaGraphExecDestroy(m_exec);
  }

  execution_space const& get_execution_space() const { return m_space; }

  // A new node has no successor yet: it is a sink until one is added.
  template <class NodeImpl>
  void add_node(std::shared_ptr<NodeImpl> const& node) {
    node->node_details_t::set_kernel(node->get_kernel());
    m_sinks.insert(std::shared_ptr<node_details_t>(node));
  }

  // node runs after pred: pred is no longer a sink (node runs it first).
  template <class NodeImplPtr, class PredecessorRef>
  void add_predecessor(NodeImplPtr node, PredecessorRef pred_ref) {
    std::shared_ptr<node_details_t> pred(GraphAccess::get_node_ptr(pred_ref));
    std::shared_ptr<node_details_t>(node)->set_predecessor(pred);
    m_sinks.erase(pred);
  }

  template <class... PredecessorRefs>
  auto create_aggregate_ptr(PredecessorRefs&&...) {
    // the edges to the predecessors arrive through add_predecessor
    using aggregate_node_impl_t = GraphNodeImpl<execution_space, aggregate_impl_t, Kokkos::Experimental::TypeErasedTag>;
    return GraphAccess::make_node_shared_ptr<aggregate_node_impl_t>(m_space, _graph_node_kernel_ctor_tag{},
                                                                    aggregate_impl_t{});
  }

  auto create_root_node_ptr() {
    auto root = GraphAccess::make_node_shared_ptr<root_node_impl_t>(m_space, _graph_node_is_root_ctor_tag{});
    m_sinks.insert(std::shared_ptr<node_details_t>(root));
    return root;
  }

  void instantiate() {
    KOKKOS_EXPECTS(!m_instantiated)
    m_instantiated = true;
    cudaStream_t s = m_space.stream();
    if (s == nullptr) return;  // the legacy stream cannot be captured: nodes run at submit
    gb300_check(gbk_workspace_reserve((gbk_stream_t)s, kWorkspaceBytes), "Graph::instantiate");
    reset();
    gb300_check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "Graph::instantiate");
    cudaGraph_t g = nullptr;
    try {
      for (auto& sink : m_sinks) sink->execute_node(m_space);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    gb300_check_cuda(cudaStreamEndCapture(s, &g), "Graph::instantiate");
    const cudaError_t e = cudaGraphInstantiate(&m_exec, g, 0);
    cudaGraphDestroy(g);
    gb300_check_cuda(e, "Graph::instantiate");
  }

  void submit(const execution_space& exec) {
    if (!m_instantiated) instantiate();
    if (m_exec) {
      gb300_check_cuda(cudaGraphLaunch(m_exec, exec.stream()), "Graph::submit");
      return;
    }
    // not captured: run the nodes in order on exec's stream
    reset();
    for (auto& sink : m_sinks) sink->execute_node(exec);
  }

 private:
  void reset() {
    for (auto& sink : m_sinks) sink->reset_has_executed();
  }

  execution_space m_space{};
  std::set<std::shared_ptr<node_details_t>> m_sinks;
  cudaGraphExec_t m_exec = nullptr;
  bool m_instantiated = false;
};

}  // namespace Impl
}  // namespace Kokkos

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_GRAPH_IMPL_HPP_
