// TeamPolicy on the GB300 space: the policy (Impl::TeamPolicyInternal), the
// team member handed to the functor, ParallelFor / ParallelReduce over it,
// and the nested TeamThreadRange / TeamVectorRange / ThreadVectorRange
// patterns and single() for that member (the CUDA space's versions:
// core/src/Cuda/Kokkos_Cuda_Parallel_Team.hpp:51-980 and
// Kokkos_Cuda_Team.hpp:72-1075).
//
// Mapping: one CTA of team_size threads per team (vector length 1: a
// ThreadVectorRange runs in its thread), league ranks strided over a grid of
// at most SMs x (2048 / team_size) CTAs; level-0 team scratch (and per-thread
// scratch x team size) is the CTA's dynamic shared memory.  Team sizes need
// not be a multiple of 32: every team-wide join handles a partial last warp.
// Level-1 scratch is global memory: each CTA owns one slice of the stream's
// workspace (the launch's grid x the policy's level-1 bytes, 256-byte
// aligned slices) and hands it to each team it runs, as a team's scratch
// lives only as long as the team.
#ifndef KOKKOS_GB300_PARALLEL_TEAM_HPP_
#define KOKKOS_GB300_PARALLEL_TEAM_HPP_

#include <Kokkos_Macros.hpp>
#if defined(KOKKOS_ENABLE_GB300)

#include <cstring>
#include <type_traits>

#include <Kokkos_Atomic.hpp>
#include <Kokkos_ExecPolicy.hpp>

#include <GB300/Kokkos_GB300_Parallel_Range.hpp>

namespace Kokkos {
namespace Impl {

// Opaque-value algebra of a Kokkos reducer object (Sum<T>, MinLoc<T,I>, ...)
// for the skeleton's team-wide joins.
template <class ReducerType>
struct GB300ReducerOps {
  const ReducerType& r;
  using V = typename ReducerType::value_type;
  __device__ void init(void* v) const { r.init(*static_cast<V*>(v)); }
  __device__ void join(void* d, const void* s) const { r.join(*static_cast<V*>(d), *static_cast<const V*>(s)); }
};
// A reducer wrapped by FunctorAnalysis (pointer interface: init / join /
// final on value_type*), as the nested reductions use it.
template <class WR>
struct GB300WrappedOps {
  const WR& r;
  using V = typename WR::value_type;
  __device__ void init(void* v) const { r.init(static_cast<V*>(v)); }
  __device__ void join(void* d, const void* s) const { r.join(static_cast<V*>(d), static_cast<const V*>(s)); }
};
template <class V>
struct GB300PlusOps {
  __device__ void init(void* v) const { *static_cast<V*>(v) = V(); }
  __device__ void join(void* d, const void* s) const { *static_cast<V*>(d) += *static_cast<const V*>(s); }
};

class GB300TeamMember {
 public:
  using execution_space = Kokkos::Experimental::GB300;
  using scratch_memory_space = execution_space::scratch_memory_space;
  using team_handle = GB300TeamMember;

 private:
  scratch_memory_space m_team_shared;
  int m_league_rank;
  int m_league_size;

  // Team-wide join of v over every thread (thread order); all threads get it.
  template <class V, class Ops>
  __device__ static V allreduce(const Ops& ops, const V& v) {
    constexpr int VB = gbk_skel::value_bytes(sizeof(V));
    gbk_skel::Val<VB> w;
    memcpy(&w, &v, sizeof(V));
    w = gbk_skel::cta_reduce_any<VB>(ops, w);
    __shared__ gbk_skel::Val<VB> s_out;
    if (threadIdx.x == 0) s_out = w;
    __syncthreads();
    V r;
    memcpy(&r, &s_out, sizeof(V));
    __syncthreads();
    return r;
  }

 public:
  KOKKOS_INLINE_FUNCTION GB300TeamMember(void* shmem, int shmem_size, int league_rank, int league_size,
                                         void* l1 = nullptr, size_t l1_size = 0)
      : m_team_shared(shmem, (size_t)shmem_size, l1, l1_size), m_league_rank(league_rank), m_league_size(league_size) {}

  KOKKOS_INLINE_FUNCTION int league_rank() const { return m_league_rank; }
  KOKKOS_INLINE_FUNCTION int league_size() const { return m_league_size; }
  KOKKOS_INLINE_FUNCTION int team_rank() const {
    KOKKOS_IF_ON_DEVICE((return (int)threadIdx.x;))
    KOKKOS_IF_ON_HOST((return 0;))
  }
  KOKKOS_INLINE_FUNCTION int team_size() const {
    KOKKOS_IF_ON_DEVICE((return (int)blockDim.x;))
    KOKKOS_IF_ON_HOST((return 1;))
  }
  KOKKOS_INLINE_FUNCTION const scratch_memory_space& team_shmem() const {
    return m_team_shared.set_team_thread_mode(0, 1, 0);
  }
  KOKKOS_INLINE_FUNCTION const scratch_memory_space& team_scratch(const int level) const {
    return m_team_shared.set_team_thread_mode(level, 1, 0);
  }
  KOKKOS_INLINE_FUNCTION const scratch_memory_space& thread_scratch(const int level) const {
    return m_team_shared.set_team_thread_mode(level, team_size(), team_rank());
  }
  KOKKOS_INLINE_FUNCTION void team_barrier() const { KOKKOS_IF_ON_DEVICE((__syncthreads();)) }

  template <class ValueType>
  KOKKOS_INLINE_FUNCTION void team_broadcast(ValueType& val, const int& root) const {
    (void)val;
    (void)root;
    KOKKOS_IF_ON_DEVICE((__shared__ gbk_skel::Val<gbk_skel::value_bytes(sizeof(ValueType))> s_b; __syncthreads();
                         if ((int)threadIdx.x == root) memcpy(&s_b, &val, sizeof(ValueType)); __syncthreads();
                         memcpy(&val, &s_b, sizeof(ValueType)); __syncthreads();))
  }
  template <class Closure, class ValueType>
  KOKKOS_INLINE_FUNCTION void team_broadcast(Closure const& f, ValueType& val, const int& root) const {
    (void)f;
    (void)val;
    (void)root;
    KOKKOS_IF_ON_DEVICE((if ((int)threadIdx.x == root) f(val); team_broadcast(val, root);))
  }

  template <class ReducerType>
  KOKKOS_INLINE_FUNCTION std::enable_if_t<is_reducer_v<ReducerType>> team_reduce(ReducerType const& reducer) const
      noexcept {
    team_reduce(reducer, reducer.reference());
  }
  template <class ReducerType>
  KOKKOS_INLINE_FUNCTION std::enable_if_t<is_reducer_v<ReducerType>> team_reduce(
      ReducerType const& reducer, typename ReducerType::value_type& value) const noexcept {
    (void)reducer;
    (void)value;
    KOKKOS_IF_ON_DEVICE((reducer.reference() = allreduce(GB300ReducerOps<ReducerType>{reducer}, value);))
  }

  // value joined over the team with a FunctorAnalysis-wrapped reducer (the
  // nested reductions: a reducer, or a closure with its own join / init).
  template <class WR>
  KOKKOS_INLINE_FUNCTION void impl_team_reduce_wrapped(const WR& wr, typename WR::value_type& value) const {
    (void)wr;
    (void)value;
    KOKKOS_IF_ON_DEVICE((value = allreduce(GB300WrappedOps<WR>{wr}, value);))
  }

  // Exclusive prefix (team_rank order) of value; the team's total is added
  // to *global_accum (if given) once, and the prefixes start from the old
  // value of *global_accum (core/src/Cuda/Kokkos_Cuda_Team.hpp:222-262).
  template <typename Type>
  KOKKOS_INLINE_FUNCTION Type team_scan(const Type& value, Type* const global_accum) const {
    (void)value;
    (void)global_accum;
    KOKKOS_IF_ON_DEVICE((return device_team_scan(value, global_accum);))
    KOKKOS_IF_ON_HOST((return Type();))
  }
  template <typename Type>
  KOKKOS_INLINE_FUNCTION Type team_scan(const Type& value) const {
    return team_scan<Type>(value, nullptr);
  }

 private:
  template <typename Type>
  __device__ Type device_team_scan(const Type& value, Type* const global_accum) const {
    __shared__ Type s_w[33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    const int cnt = min(32, (int)blockDim.x - warp * 32);
    const unsigned mask = gbk_skel::warp_mask_of(cnt);
    // inclusive warp scan by shifts up within the warp's active lanes
    constexpr int W = (int)((sizeof(Type) + 3) / 4);
    auto shift_up = [&](const Type& x, int d) {
      unsigned tmp[W] = {};
      memcpy(tmp, &x, sizeof(Type));
#pragma unroll
      for (int k = 0; k < W; ++k) tmp[k] = __shfl_up_sync(mask, tmp[k], d);
      Type o;
      memcpy(&o, tmp, sizeof(Type));
      return o;
    };
    Type inc = value;
    for (int d = 1; d < 32; d <<= 1) {
      const Type o = shift_up(inc, d);
      if (lane >= d) inc = o + inc;
    }
    Type ex = shift_up(inc, 1);
    if (lane == 0) ex = Type();
    if (lane == cnt - 1) s_w[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
      Type tot = Type();
      for (int w = 0; w < nw; ++w) tot += s_w[w];
      Type run = global_accum ? Kokkos::atomic_fetch_add(global_accum, tot) : Type();
      for (int w = 0; w < nw; ++w) {
        const Type t = s_w[w];
        s_w[w] = run;
        run += t;
      }
    }
    __syncthreads();
    const Type r = s_w[warp] + ex;
    __syncthreads();
    return r;
  }
};

// ---- the policy ---------------------------------------------------------------
template <class... Properties>
class TeamPolicyInternal<Kokkos::Experimental::GB300, Properties...> : public PolicyTraits<Properties...> {
 public:
  using execution_policy = TeamPolicyInternal;
  using traits = PolicyTraits<Properties...>;
  using execution_space = Kokkos::Experimental::GB300;
  using member_type = GB300TeamMember;

  template <class ExecSpace, class... OtherProperties>
  friend class TeamPolicyInternal;

 private:
  static constexpr int kDefaultTeam = 256;
  execution_space m_space;
  int m_league_size = 0;
  int m_team_size = -1;
  int m_chunk_size = 1;
  size_t m_team_scratch_size[2] = {0, 0};
  size_t m_thread_scratch_size[2] = {0, 0};
  bool m_tune_team = false;

  void check() const {
    if (m_team_size > 1024) Kokkos::abort("Kokkos::TeamPolicy<GB300>: team size above 1024");
  }

 public:
  const execution_space& space() const { return m_space; }

  template <class... OtherProperties>
  TeamPolicyInternal(const TeamPolicyInternal<Kokkos::Experimental::GB300, OtherProperties...>& p)
      : traits(p),
        m_space(p.m_space),
        m_league_size(p.m_league_size),
        m_team_size(p.m_team_size),
        m_chunk_size(p.m_chunk_size),
        m_tune_team(p.m_tune_team) {
    for (int l = 0; l < 2; ++l) {
      m_team_scratch_size[l] = p.m_team_scratch_size[l];
      m_thread_scratch_size[l] = p.m_thread_scratch_size[l];
    }
  }

  TeamPolicyInternal(const execution_space& space, int league_size_request, int team_size_request,
                     int /*vector_length_request*/ = 1)
      : m_space(space), m_league_size(league_size_request), m_team_size(team_size_request) {
    if (m_team_size <= 0) {
      m_team_size = kDefaultTeam;
      m_tune_team = true;
    }
    check();
  }
  TeamPolicyInternal(const execution_space& space, int league_size_request, const Kokkos::AUTO_t&,
                     int vector_length_request = 1)
      : TeamPolicyInternal(space, league_size_request, -1, vector_length_request) {}
  TeamPolicyInternal(const execution_space& space, int league_size_request, const Kokkos::AUTO_t&,
                     const Kokkos::AUTO_t&)
      : TeamPolicyInternal(space, league_size_request, -1, 1) {}
  TeamPolicyInternal(const execution_space& space, int league_size_request, int team_size_request,
                     const Kokkos::AUTO_t&)
      : TeamPolicyInternal(space, league_size_request, team_size_request, 1) {}
  TeamPolicyInternal(int league_size_request, const Kokkos::AUTO_t& t, int vector_length_request = 1)
      : TeamPolicyInternal(execution_space(), league_size_request, t, vector_length_request) {}
  TeamPolicyInternal(int league_size_request, const Kokkos::AUTO_t& t, const Kokkos::AUTO_t& v)
      : TeamPolicyInternal(execution_space(), league_size_request, t, v) {}
  TeamPolicyInternal(int league_size_request, int team_size_request, const Kokkos::AUTO_t& v)
      : TeamPolicyInternal(execution_space(), league_size_request, team_size_request, v) {}
  TeamPolicyInternal(int league_size_request, int team_size_request, int vector_length_request = 1)
      : TeamPolicyInternal(execution_space(), league_size_request, team_size_request, vector_length_request) {}

  // The largest team the pattern's kernel can launch with (its registers
  // per thread bound the threads of a CTA), at most 1024; the pattern types
  // are those the reference's CUDA policy names for the same query.
  template <class FunctorType>
  int team_size_max(const FunctorType&, const ParallelForTag&) const {
    return ParallelFor<FunctorType, Kokkos::TeamPolicy<Properties...>, Kokkos::Experimental::GB300>::max_team_threads();
  }
  template <class FunctorType>
  int team_size_max(const FunctorType&, const ParallelReduceTag&) const {
    using FA = FunctorAnalysis<FunctorPatternInterface::REDUCE, TeamPolicyInternal, FunctorType, void>;
    return ParallelReduce<CombinedFunctorReducer<FunctorType, typename FA::Reducer>, Kokkos::TeamPolicy<Properties...>,
                          Kokkos::Experimental::GB300>::max_team_threads();
  }
  template <class FunctorType, class ReducerType>
  int team_size_max(const FunctorType&, const ReducerType&, const ParallelReduceTag&) const {
    return ParallelReduce<CombinedFunctorReducer<FunctorType, ReducerType>, Kokkos::TeamPolicy<Properties...>,
                          Kokkos::Experimental::GB300>::max_team_threads();
  }
  template <class FunctorType>
  int team_size_recommended(const FunctorType& f, const ParallelForTag& t) const {
    const int m = team_size_max(f, t);
    return m < kDefaultTeam ? m : kDefaultTeam;
  }
  template <class FunctorType>
  int team_size_recommended(const FunctorType& f, const ParallelReduceTag& t) const {
    const int m = team_size_max(f, t);
    return m < kDefaultTeam ? m : kDefaultTeam;
  }
  template <class FunctorType, class ReducerType>
  int team_size_recommended(const FunctorType& f, const ReducerType& r, const ParallelReduceTag& t) const {
    const int m = team_size_max(f, r, t);
    return m < kDefaultTeam ? m : kDefaultTeam;
  }

  int team_size() const { return m_team_size; }
  int league_size() const { return m_league_size; }
  int chunk_size() const { return m_chunk_size; }
  int impl_vector_length() const { return 1; }
  static int vector_length_max() { return 1; }
  bool impl_auto_team_size() const { return m_tune_team; }
  bool impl_auto_vector_length() const { return false; }
  void impl_set_team_size(size_t t) { m_team_size = (int)t; }
  void impl_set_vector_length(size_t) {}
  // level 1: as the CUDA space, 20 MiB per team
  static int scratch_size_max(int level) { return level == 0 ? 160 * 1024 : 20 * 1024 * 1024; }
  size_t scratch_size(const int& level, int team_size_ = -1) const {
    if (team_size_ < 0) team_size_ = m_team_size;
    return m_team_scratch_size[level] + (size_t)team_size_ * m_thread_scratch_size[level];
  }
  size_t team_scratch_size(const int& level) const { return m_team_scratch_size[level]; }
  size_t thread_scratch_size(const int& level) const { return m_thread_scratch_size[level]; }

  TeamPolicyInternal& set_chunk_size(typename traits::index_type chunk) {
    m_chunk_size = (int)chunk;
    return *this;
  }
  TeamPolicyInternal& set_scratch_size(const int& level, const PerTeamValue& per_team) {
    m_team_scratch_size[level] = per_team.value;
    check();
    return *this;
  }
  TeamPolicyInternal& set_scratch_size(const int& level, const PerThreadValue& per_thread) {
    m_thread_scratch_size[level] = per_thread.value;
    check();
    return *this;
  }
  TeamPolicyInternal& set_scratch_size(const int& level, const PerTeamValue& per_team,
                                       const PerThreadValue& per_thread) {
    m_team_scratch_size[level] = per_team.value;
    m_thread_scratch_size[level] = per_thread.value;
    check();
    return *this;
  }
};

// Threads a CTA of this kernel can have (its registers per thread), at most
// 1024, whole warps.
inline int gb300_kernel_max_threads(const void* kernel) {
  cudaFuncAttributes a{};
  gb300_check_cuda(cudaFuncGetAttributes(&a, kernel), "TeamPolicy::team_size_max");
  const int t = a.maxThreadsPerBlock < 1024 ? a.maxThreadsPerBlock : 1024;
  return t >= 32 ? t / 32 * 32 : t;
}

// Grid and dynamic shared memory of a team launch.
template <class Policy>
// One CTA per league rank, up to max_grid CTAs (then each strides): the block
// scheduler hands the next team to whichever SM frees up first, so a long
// team does not hold back the teams that would have followed it on its CTA.
// With level-1 scratch the grid is the resident CTAs at most (each holds a
// slice of global memory): *l1 is the size a team sees (what the policy asked
// for, exactly) and *l1_stride the slice's 256-byte-aligned stride.
// extra_l0: the functor's own team_shmem_size(team_size), added to the
// policy's level-0 bytes as the reference does.
void gb300_team_shape(const Policy& p, const void* kernel, int64_t max_grid, int64_t* grid, int* shmem,
                      size_t* l1 = nullptr, size_t* l1_stride = nullptr, size_t extra_l0 = 0) {
  const int ts = p.team_size();
  *shmem = (int)(p.scratch_size(0, ts) + extra_l0);
  if (*shmem > 48 * 1024)
    gb300_check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, *shmem),
                     "TeamPolicy scratch");
  const size_t l1req = p.scratch_size(1, ts);
  const size_t l1b = (l1req + 255) / 256 * 256;
  if (l1) *l1 = l1req;
  if (l1_stride) *l1_stride = l1b;
  if (l1b) {
    const int64_t resident = (int64_t)p.space().sm_count() * (2048 / (ts > 0 ? ts : 1));
    if (max_grid > resident) max_grid = resident;
  }
  int64_t g = p.league_size();
  if (g > max_grid) g = max_grid;
  *grid = g < 1 ? 1 : g;
}

// ---- ParallelFor<TeamPolicy> -------------------------------------------------
template <class FunctorType, class... Properties>
class ParallelFor<FunctorType, Kokkos::TeamPolicy<Properties...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::TeamPolicy<Properties...>;
  using functor_type = FunctorType;

 private:
  using WorkTag = typename Policy::work_tag;
  const FunctorType m_functor;
  const Policy m_policy;

 public:
  struct Closure {
    FunctorType f;
    int shmem;
    char* l1;          // level-1 slices, one per CTA
    size_t l1_size;    // a team's level-1 bytes
    size_t l1_stride;  // slice stride
    __device__ void exec_team(int64_t lr, int64_t league, unsigned char* sm) const {
      gb300_call<WorkTag>(f, GB300TeamMember(sm, shmem, (int)lr, (int)league,
                                             l1 ? l1 + (size_t)blockIdx.x * l1_stride : nullptr, l1_size));
    }
  };

  Policy const& get_policy() const { return m_policy; }
  static int max_team_threads() { return gb300_kernel_max_threads((const void*)gbk_skel::k_team_for<Closure>); }
  ParallelFor(const FunctorType& arg_functor, const Policy& arg_policy)
      : m_functor(arg_functor), m_policy(arg_policy) {}

  void execute() const {
    if (m_policy.league_size() <= 0) return;
    const auto& exec = m_policy.space();
    int64_t g = 1;
    int shmem = 0;
    size_t l1 = 0, l1s = 0;
    gb300_team_shape(m_policy, (const void*)gbk_skel::k_team_for<Closure>, int64_t(1) << 20, &g, &shmem, &l1,
                     &l1s, FunctorTeamShmemSize<FunctorType>::value(m_functor, m_policy.team_size()));
    GB300Scratch sc = gb300_scratch(exec, (size_t)g * l1s);
    gbk_skel::k_team_for<Closure><<<(unsigned)g, m_policy.team_size(), shmem, exec.stream()>>>(
        Closure{m_functor, shmem, l1s ? sc.base : nullptr, l1, l1s}, m_policy.league_size(), sc.err);
    gb300_launched("parallel_for(TeamPolicy)");
  }
};

// ---- ParallelReduce<TeamPolicy> ----------------------------------------------
template <class CombinedFunctorReducerType, class... Properties>
class ParallelReduce<CombinedFunctorReducerType, Kokkos::TeamPolicy<Properties...>, Kokkos::Experimental::GB300> {
 public:
  using Policy = Kokkos::TeamPolicy<Properties...>;
  using FunctorType = typename CombinedFunctorReducerType::functor_type;
  using ReducerType = typename CombinedFunctorReducerType::reducer_type;
  using pointer_type = typename ReducerType::pointer_type;
  using value_type = typename ReducerType::value_type;
  using reference_type = typename ReducerType::reference_type;
  using functor_type = FunctorType;
  using reducer_type = ReducerType;

 private:
  using WorkTag = typename Policy::work_tag;
  const CombinedFunctorReducerType m_functor_reducer;
  const Policy m_policy;
  const pointer_type m_result_ptr;
  const bool m_result_ptr_device_accessible;

 public:
  struct Closure : GB300ValueOps<ReducerType> {
    FunctorType f;
    int shmem;
    char* l1;          // level-1 slices, one per CTA
    size_t l1_size;    // a team's level-1 bytes
    size_t l1_stride;  // slice stride
    __device__ void exec_team(int64_t lr, int64_t league, unsigned char* sm, void* v) const {
      gb300_call<WorkTag>(f,
                          GB300TeamMember(sm, shmem, (int)lr, (int)league,
                                          l1 ? l1 + (size_t)blockIdx.x * l1_stride : nullptr, l1_size),
                          this->r.reference(static_cast<pointer_type>(v)));
    }
  };

  Policy const& get_policy() const { return m_policy; }
  static int max_team_threads() {
    return gb300_kernel_max_threads((const void*)gbk_skel::k_team_reduce<gb300_value_bytes<ReducerType>(), Closure>);
  }

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
    const auto& exec = m_policy.space();
    int64_t g = 1;
    int shmem = 0;
    size_t l1 = 0, l1s = 0;
    gb300_team_shape(m_policy, (const void*)gbk_skel::k_team_reduce<VB, Closure>, int64_t(1) << 16, &g, &shmem,
                     &l1, &l1s,
                     FunctorTeamShmemSize<FunctorType>::value(m_functor_reducer.get_functor(), m_policy.team_size()));
    const int64_t league = m_policy.league_size() > 0 ? m_policy.league_size() : 0;
    Closure c{{m_functor_reducer.get_reducer()}, m_functor_reducer.get_functor(), shmem, nullptr, l1, l1s};
    const int ts = m_policy.team_size();
    // the level-1 slices follow the reduce's partials in the stream's workspace
    gb300_run_reduce<VB>(exec, m_functor_reducer.get_reducer(), g, m_result_ptr, m_result_ptr_device_accessible,
                         [&](gbk_skel::Val<VB>* part, unsigned* ctr, gbk_skel::Val<VB>* out, int* err, char* extra) {
                           if (l1s) c.l1 = extra;
                           gbk_skel::k_team_reduce<VB, Closure><<<(unsigned)g, ts, shmem, exec.stream()>>>(
                               c, league, part, ctr, out, err);
                         },
                         (size_t)g * l1s);
  }
};

// ---- nested range boundaries for this member ---------------------------------
template <typename iType>
struct TeamThreadRangeBoundariesStruct<iType, GB300TeamMember> {
  using index_type = iType;
  const GB300TeamMember& member;
  const iType start;
  const iType end;
  KOKKOS_INLINE_FUNCTION TeamThreadRangeBoundariesStruct(const GB300TeamMember& m, iType count)
      : member(m), start(0), end(count) {}
  KOKKOS_INLINE_FUNCTION TeamThreadRangeBoundariesStruct(const GB300TeamMember& m, iType b, iType e)
      : member(m), start(b), end(e) {}
};
template <typename iType>
struct TeamVectorRangeBoundariesStruct<iType, GB300TeamMember> {
  using index_type = iType;
  const GB300TeamMember& member;
  const iType start;
  const iType end;
  KOKKOS_INLINE_FUNCTION TeamVectorRangeBoundariesStruct(const GB300TeamMember& m, const iType& count)
      : member(m), start(0), end(count) {}
  KOKKOS_INLINE_FUNCTION TeamVectorRangeBoundariesStruct(const GB300TeamMember& m, const iType& b, const iType& e)
      : member(m), start(b), end(e) {}
};
template <typename iType>
struct ThreadVectorRangeBoundariesStruct<iType, GB300TeamMember> {
  using index_type = iType;
  const index_type start;
  const index_type end;
  KOKKOS_INLINE_FUNCTION ThreadVectorRangeBoundariesStruct(const GB300TeamMember, index_type count)
      : start(0), end(count) {}
  KOKKOS_INLINE_FUNCTION ThreadVectorRangeBoundariesStruct(const GB300TeamMember, index_type b, index_type e)
      : start(b), end(e) {}
};

// Team-strided walk of [start, end): thread r takes start + r, + team_size,
// ..., 32 of them per loop trip while that many remain, then 8, then one at
// a time, so that up to 32 loads of the closure are in flight (calls stay in
// increasing index order per thread).  With one team per league rank the
// longest range is the league's tail, streamed by one CTA at the rate of
// the bytes it keeps in flight.
template <int U, class I, class F>
__device__ __forceinline__ void gb300_team_steps(I& i, I end, I step, const F& f) {
  for (; i < end && (end - i) > (I)(U - 1) * step; i += (I)U * step) {
#pragma unroll
    for (int u = 0; u < U; ++u) f(i + (I)u * step);
  }
}
template <class B, class F>
__device__ __forceinline__ void gb300_team_walk(const B& b, const F& f) {
  using I = std::remove_cv_t<decltype(b.start)>;
  const I step = (I)blockDim.x;
  I i = b.start + (I)threadIdx.x;
  gb300_team_steps<32>(i, (I)b.end, step, f);
  gb300_team_steps<8>(i, (I)b.end, step, f);
  for (; i < b.end; i += step) f(i);
}

}  // namespace Impl

template <typename iType>
KOKKOS_INLINE_FUNCTION Impl::TeamThreadRangeBoundariesStruct<iType, Impl::GB300TeamMember> TeamThreadRange(
    const Impl::GB300TeamMember& m, iType count) {
  return Impl::TeamThreadRangeBoundariesStruct<iType, Impl::GB300TeamMember>(m, count);
}
template <typename iType1, typename iType2>
KOKKOS_INLINE_FUNCTION Impl::TeamThreadRangeBoundariesStruct<std::common_type_t<iType1, iType2>, Impl::GB300TeamMember>
TeamThreadRange(const Impl::GB300TeamMember& m, iType1 b, iType2 e) {
  using iType = std::common_type_t<iType1, iType2>;
  return Impl::TeamThreadRangeBoundariesStruct<iType, Impl::GB300TeamMember>(m, iType(b), iType(e));
}
template <typename iType>
KOKKOS_INLINE_FUNCTION Impl::TeamVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember> TeamVectorRange(
    const Impl::GB300TeamMember& m, const iType& count) {
  return Impl::TeamVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>(m, count);
}
template <typename iType1, typename iType2>
KOKKOS_INLINE_FUNCTION Impl::TeamVectorRangeBoundariesStruct<std::common_type_t<iType1, iType2>, Impl::GB300TeamMember>
TeamVectorRange(const Impl::GB300TeamMember& m, const iType1& b, const iType2& e) {
  using iType = std::common_type_t<iType1, iType2>;
  return Impl::TeamVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>(m, iType(b), iType(e));
}
template <typename iType>
KOKKOS_INLINE_FUNCTION Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember> ThreadVectorRange(
    const Impl::GB300TeamMember& m, iType count) {
  return Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>(m, count);
}
template <typename iType1, typename iType2>
KOKKOS_INLINE_FUNCTION
    Impl::ThreadVectorRangeBoundariesStruct<std::common_type_t<iType1, iType2>, Impl::GB300TeamMember>
    ThreadVectorRange(const Impl::GB300TeamMember& m, iType1 b, iType2 e) {
  using iType = std::common_type_t<iType1, iType2>;
  return Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>(m, iType(b), iType(e));
}
KOKKOS_INLINE_FUNCTION Impl::ThreadSingleStruct<Impl::GB300TeamMember> PerTeam(const Impl::GB300TeamMember& m) {
  return Impl::ThreadSingleStruct<Impl::GB300TeamMember>(m);
}
KOKKOS_INLINE_FUNCTION Impl::VectorSingleStruct<Impl::GB300TeamMember> PerThread(const Impl::GB300TeamMember& m) {
  return Impl::VectorSingleStruct<Impl::GB300TeamMember>(m);
}

// ---- TeamThreadRange / TeamVectorRange patterns --------------------------------
#define KOKKOS_GB300_TEAM_PATTERNS(BOUNDS)                                                                          \
  template <typename iType, class Closure>                                                                         \
  KOKKOS_INLINE_FUNCTION void parallel_for(const Impl::BOUNDS<iType, Impl::GB300TeamMember>& b,                    \
                                           const Closure& closure) {                                               \
    (void)b;                                                                                                        \
    (void)closure;                                                                                                  \
    KOKKOS_IF_ON_DEVICE((Impl::gb300_team_walk(b, [&](iType i) { closure(i); });))                                  \
  }                                                                                                                 \
  template <typename iType, class Closure, class ReducerType>                                                      \
  KOKKOS_INLINE_FUNCTION std::enable_if_t<Kokkos::is_reducer<ReducerType>::value> parallel_reduce(                 \
      const Impl::BOUNDS<iType, Impl::GB300TeamMember>& b, const Closure& closure, const ReducerType& reducer) {    \
    (void)b;                                                                                                        \
    (void)closure;                                                                                                  \
    (void)reducer;                                                                                                  \
    KOKKOS_IF_ON_DEVICE((using value_type = typename ReducerType::value_type;                                      \
                         using WR = typename Kokkos::Impl::FunctorAnalysis<                                         \
                             Kokkos::Impl::FunctorPatternInterface::REDUCE,                                         \
                             Kokkos::TeamPolicy<Kokkos::Experimental::GB300>, ReducerType, value_type>::Reducer;    \
                         WR wr(reducer); value_type v; wr.init(&v);                                                 \
                         Impl::gb300_team_walk(b, [&](iType i) { closure(i, v); });                                 \
                         b.member.impl_team_reduce_wrapped(wr, v); wr.final(&v); reducer.reference() = v;))         \
  }                                                                                                                 \
  template <typename iType, class Closure, class ValueType>                                                        \
  KOKKOS_INLINE_FUNCTION std::enable_if_t<!Kokkos::is_reducer<ValueType>::value> parallel_reduce(                  \
      const Impl::BOUNDS<iType, Impl::GB300TeamMember>& b, const Closure& closure, ValueType& result) {             \
    (void)b;                                                                                                        \
    (void)closure;                                                                                                  \
    (void)result;                                                                                                   \
    KOKKOS_IF_ON_DEVICE((using WR = typename Kokkos::Impl::FunctorAnalysis<                                         \
                             Kokkos::Impl::FunctorPatternInterface::REDUCE,                                         \
                             Kokkos::TeamPolicy<Kokkos::Experimental::GB300>, Closure, ValueType>::Reducer;         \
                         using value_type = typename WR::value_type;                                                \
                         WR wr(closure); value_type v{}; wr.init(&v);                                               \
                         Impl::gb300_team_walk(b, [&](iType i) { closure(i, v); });                                 \
                         b.member.impl_team_reduce_wrapped(wr, v); wr.final(&v); result = v;))                      \
  }                                                                                                                 \
  /* scan: the team's indices in order; each thread folds its own strided */                                      \
  /* indices, so the scan runs in rounds of team_size consecutive indices */                                       \
  template <typename iType, class Closure, class ValueType>                                                        \
  KOKKOS_INLINE_FUNCTION void parallel_scan(const Impl::BOUNDS<iType, Impl::GB300TeamMember>& b,                   \
                                            const Closure& closure, ValueType& return_val) {                       \
    (void)b;                                                                                                        \
    (void)closure;                                                                                                  \
    (void)return_val;                                                                                               \
    KOKKOS_IF_ON_DEVICE((ValueType carry = ValueType(); const iType ts = (iType)blockDim.x;                         \
                         for (iType base = b.start; base < b.end; base += ts) {                                     \
                           const iType i = base + (iType)threadIdx.x;                                               \
                           ValueType mine = ValueType();                                                           \
                           if (i < b.end) closure(i, mine, false);                                                  \
                           ValueType pre = b.member.team_scan(mine);                                               \
                           ValueType tot = pre + mine;                                                              \
                           b.member.team_broadcast(tot, (int)((b.end - base < ts ? b.end - base : ts) - 1));        \
                           ValueType upd = carry + pre;                                                             \
                           if (i < b.end) closure(i, upd, true);                                                    \
                           carry += tot;                                                                            \
                         } return_val = carry;))                                                                    \
  }                                                                                                                 \
  template <typename iType, class Closure>                                                                         \
  KOKKOS_INLINE_FUNCTION void parallel_scan(const Impl::BOUNDS<iType, Impl::GB300TeamMember>& b,                   \
                                            const Closure& closure) {                                              \
    using value_type = typename Kokkos::Impl::FunctorAnalysis<Kokkos::Impl::FunctorPatternInterface::SCAN, void,    \
                                                              Closure, void>::value_type;                          \
    value_type total;                                                                                               \
    parallel_scan(b, closure, total);                                                                               \
  }

KOKKOS_GB300_TEAM_PATTERNS(TeamThreadRangeBoundariesStruct)
KOKKOS_GB300_TEAM_PATTERNS(TeamVectorRangeBoundariesStruct)
#undef KOKKOS_GB300_TEAM_PATTERNS

// ---- ThreadVectorRange patterns (vector length 1: the thread runs them) ------------
template <typename iType, class Closure>
KOKKOS_INLINE_FUNCTION void parallel_for(const Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>& b,
                                         const Closure& closure) {
  for (iType i = b.start; i < b.end; ++i) closure(i);
}
template <typename iType, class Closure, class ReducerType>
KOKKOS_INLINE_FUNCTION std::enable_if_t<Kokkos::is_reducer<ReducerType>::value> parallel_reduce(
    const Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>& b, const Closure& closure,
    const ReducerType& reducer) {
  using value_type = typename ReducerType::value_type;
  using WR = typename Kokkos::Impl::FunctorAnalysis<Kokkos::Impl::FunctorPatternInterface::REDUCE,
                                                    Kokkos::TeamPolicy<Kokkos::Experimental::GB300>, ReducerType,
                                                    value_type>::Reducer;
  WR wr(reducer);
  value_type v;
  wr.init(&v);
  for (iType i = b.start; i < b.end; ++i) closure(i, v);
  wr.final(&v);
  reducer.reference() = v;
}
template <typename iType, class Closure, class ValueType>
KOKKOS_INLINE_FUNCTION std::enable_if_t<!Kokkos::is_reducer<ValueType>::value> parallel_reduce(
    const Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>& b, const Closure& closure,
    ValueType& result) {
  // a closure with its own join / init / final reduces with them (vector
  // length 1: init, the loop, final)
  using WR = typename Kokkos::Impl::FunctorAnalysis<Kokkos::Impl::FunctorPatternInterface::REDUCE,
                                                    Kokkos::TeamPolicy<Kokkos::Experimental::GB300>, Closure,
                                                    ValueType>::Reducer;
  using value_type = typename WR::value_type;
  WR wr(closure);
  value_type v{};
  wr.init(&v);
  for (iType i = b.start; i < b.end; ++i) closure(i, v);
  wr.final(&v);
  result = v;
}
template <typename iType, class Closure, class ReducerType>
KOKKOS_INLINE_FUNCTION std::enable_if_t<Kokkos::is_reducer<ReducerType>::value> parallel_scan(
    const Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>& b, const Closure& closure,
    const ReducerType& reducer) {
  typename ReducerType::value_type v;
  reducer.init(v);
  for (iType i = b.start; i < b.end; ++i) closure(i, v, true);
  reducer.reference() = v;
}
template <typename iType, class Closure, class ValueType>
KOKKOS_INLINE_FUNCTION std::enable_if_t<!Kokkos::is_reducer<ValueType>::value> parallel_scan(
    const Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>& b, const Closure& closure,
    ValueType& return_val) {
  ValueType v = ValueType();
  for (iType i = b.start; i < b.end; ++i) closure(i, v, true);
  return_val = v;
}
template <typename iType, class Closure>
KOKKOS_INLINE_FUNCTION void parallel_scan(
    const Impl::ThreadVectorRangeBoundariesStruct<iType, Impl::GB300TeamMember>& b, const Closure& closure) {
  using value_type =
      typename Kokkos::Impl::FunctorAnalysis<Kokkos::Impl::FunctorPatternInterface::SCAN, void, Closure,
                                             void>::value_type;
  value_type v = value_type();
  for (iType i = b.start; i < b.end; ++i) closure(i, v, true);
}

// ---- single ------------------------------------------------------------------------
template <class FunctorType>
KOKKOS_INLINE_FUNCTION void single(const Impl::VectorSingleStruct<Impl::GB300TeamMember>&, const FunctorType& lambda) {
  lambda();
}
template <class FunctorType>
KOKKOS_INLINE_FUNCTION void single(const Impl::ThreadSingleStruct<Impl::GB300TeamMember>& s,
                                   const FunctorType& lambda) {
  if (s.team_member.team_rank() == 0) lambda();
}
template <class FunctorType, class ValueType>
KOKKOS_INLINE_FUNCTION void single(const Impl::VectorSingleStruct<Impl::GB300TeamMember>&, const FunctorType& lambda,
                                   ValueType& val) {
  lambda(val);
}
template <class FunctorType, class ValueType>
KOKKOS_INLINE_FUNCTION void single(const Impl::ThreadSingleStruct<Impl::GB300TeamMember>& s,
                                   const FunctorType& lambda, ValueType& val) {
  if (s.team_member.team_rank() == 0) lambda(val);
  s.team_member.team_broadcast(val, 0);
}

}  // namespace Kokkos

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_PARALLEL_TEAM_HPP_
