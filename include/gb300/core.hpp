// Core of the header-template path: execution space, memory spaces, View,
// deep_copy and the execution policies, with the names and argument meaning
// of the reference (core/src/Kokkos_Core.hpp, View core/src/View/*,
// policies core/src/Kokkos_ExecPolicy.hpp:77-1000,
// core/src/KokkosExp_MDRangePolicy.hpp:159-425).  Compiled by nvcc in the
// user's translation unit (-std=c++17 --extended-lambda).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../gbk.h"
#include "../gbk_tools.h"
#include "tools.hpp"

#ifndef KOKKOS_LAMBDA
#define KOKKOS_LAMBDA [=] __host__ __device__
#define KOKKOS_CLASS_LAMBDA [ =, *this ] __host__ __device__
#define KOKKOS_FUNCTION __host__ __device__
#define KOKKOS_INLINE_FUNCTION __host__ __device__ inline
#define KOKKOS_FORCEINLINE_FUNCTION __host__ __device__ __forceinline__
#endif

namespace gb300k {

// Error convention of the reference: a failing device call throws
// (core/src/Cuda/Kokkos_Cuda_Error.hpp:33-67, impl/Kokkos_Error.hpp).
inline void check(int status, const char* what) {
  if (status != GBK_OK) throw std::runtime_error(std::string(what) + ": " + gbk_status_string(status));
}
inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

struct LayoutLeft {};
struct LayoutRight {};
struct HostSpace {};
struct GB300Space {};

// Kokkos::InitializationSettings (core/src/impl/Kokkos_InitializationSettings.hpp):
// the settings a space's impl_initialize receives; this space reads the
// device id only (the library runs on the current device).
class InitializationSettings {
 public:
  InitializationSettings& set_device_id(int d) {
    device_id_ = d;
    return *this;
  }
  InitializationSettings& set_num_threads(int t) {
    num_threads_ = t;
    return *this;
  }
  bool has_device_id() const { return device_id_ >= 0; }
  int get_device_id() const { return device_id_; }
  int get_num_threads() const { return num_threads_; }

 private:
  int device_id_ = -1, num_threads_ = -1;
};
// Kokkos::Device<ExecSpace, MemSpace> (core/src/Kokkos_Core_fwd.hpp).
template <class ExecSpace, class MemSpace>
struct Device {
  using execution_space = ExecSpace;
  using memory_space = MemSpace;
  using device_type = Device;
};
// Team scratch memory space tag (the header path's teams use static shared
// memory inside the library skeletons).
struct ScratchMemorySpaceTag {};

namespace Experimental {
// The execution space (core/src/Cuda/Kokkos_Cuda.hpp:95-260 is the device
// model): one CUDA stream; fence() = gbk_stream_check, which also reports
// device conditions (a bounded wait that gave up, a key outside the bins).
class GB300 {
 public:
  using execution_space = GB300;
  using memory_space = GB300Space;
  using device_type = Device<GB300, GB300Space>;
  using array_layout = LayoutLeft;
  using size_type = int64_t;
  using scratch_memory_space = ScratchMemorySpaceTag;
  GB300() = default;
  explicit GB300(cudaStream_t s) : stream_(s) {}
  cudaStream_t stream() const { return stream_; }
  gbk_stream_t handle() const { return (gbk_stream_t)stream_; }
  void fence(const std::string& = std::string()) const { check(gbk_stream_check(handle()), "GB300::fence"); }
  static void impl_static_fence(const std::string& = std::string()) {
    check_cuda(cudaDeviceSynchronize(), "GB300::impl_static_fence");
  }
  int concurrency() const {
    int sm = 0;
    gbk_device_info(&sm, nullptr, nullptr, nullptr);
    return sm * 2048;
  }
  void print_configuration(std::ostream& os, bool = false) const {
    int sm = 0, ma = 0, mi = 0;
    int64_t l2 = 0;
    gbk_device_info(&sm, &ma, &mi, &l2);
    os << "GB300 execution space: " << sm << " SMs, compute capability " << ma << "." << mi << ", L2 " << l2
       << " bytes\n";
  }
  static const char* name() { return "GB300"; }
  // Space registration hooks (core/src/impl/Kokkos_ExecSpaceManager.hpp:17-108):
  // select the device, make the library's per-device state; release it.
  static void impl_initialize(const InitializationSettings& s) {
    if (s.has_device_id()) check_cuda(cudaSetDevice(s.get_device_id()), "GB300::impl_initialize");
    int sm = 0;
    check(gbk_device_info(&sm, nullptr, nullptr, nullptr), "GB300::impl_initialize");
  }
  static void impl_finalize() { check_cuda(cudaDeviceSynchronize(), "GB300::impl_finalize"); }

 private:
  cudaStream_t stream_ = nullptr;
};
}  // namespace Experimental

using DefaultExecutionSpace = Experimental::GB300;

// initialize(): GBK_TUNING_TABLE=<file> loads a tuning table (as written by
// the autotuner) and enables it for every call made without a configuration.
inline void initialize(const InitializationSettings& s) {
  Experimental::GB300::impl_initialize(s);
  Tools::Impl::load_tool();  // KOKKOS_TOOLS_LIBS
  if (const char* p = std::getenv("GBK_TUNING_TABLE")) {
    if (gbk_tuner_load(p) == GBK_OK) gbk_tuner_enable(1);
  }
}
inline void initialize(int = 0, char** = nullptr) { initialize(InitializationSettings()); }
inline void finalize() {
  check_cuda(cudaDeviceSynchronize(), "finalize");
  Tools::Impl::unload_tool();
}
inline void fence(const std::string& = std::string()) { Experimental::GB300::impl_static_fence(); }

// ---------------------------------------------------------------------------
// View: rank 1..6, LayoutLeft / LayoutRight, device (GB300Space) or host.
namespace Impl {
template <class D> struct ViewRank { using value_type = D; static constexpr int rank = 0; };  // View<T>: one value
template <class T> struct ViewRank<T*> { using value_type = T; static constexpr int rank = 1; };
template <class T> struct ViewRank<T**> { using value_type = T; static constexpr int rank = 2; };
template <class T> struct ViewRank<T***> { using value_type = T; static constexpr int rank = 3; };
template <class T> struct ViewRank<T****> { using value_type = T; static constexpr int rank = 4; };
template <class T> struct ViewRank<T*****> { using value_type = T; static constexpr int rank = 5; };
template <class T> struct ViewRank<T******> { using value_type = T; static constexpr int rank = 6; };

template <class... P> struct ViewProps;
template <> struct ViewProps<> { using layout = LayoutLeft; using space = GB300Space; };
template <class... P> struct ViewProps<LayoutLeft, P...> { using layout = LayoutLeft; using space = typename ViewProps<P...>::space; };
template <class... P> struct ViewProps<LayoutRight, P...> { using layout = LayoutRight; using space = typename ViewProps<P...>::space; };
template <class... P> struct ViewProps<HostSpace, P...> { using layout = LayoutRight; using space = HostSpace; };
template <class... P> struct ViewProps<GB300Space, P...> { using layout = typename ViewProps<P...>::layout; using space = GB300Space; };
template <class... P> struct ViewProps<Experimental::GB300, P...> { using layout = typename ViewProps<P...>::layout; using space = GB300Space; };

// Host-side reference count of a View allocation (copies made in device code
// do not touch it).
struct Tracker {
  std::atomic<long> count{1};
  void* ptr = nullptr;
  bool device = true;
  std::string label;
};
}  // namespace Impl

template <class DataType, class... Props>
class View {
 public:
  using traits = Impl::ViewRank<DataType>;
  using value_type = typename traits::value_type;
  using non_const_value_type = std::remove_const_t<value_type>;
  using array_layout = typename Impl::ViewProps<Props...>::layout;
  using memory_space = typename Impl::ViewProps<Props...>::space;
  using pointer_type = value_type*;
  static constexpr int rank = traits::rank;
  static constexpr bool is_device = std::is_same<memory_space, GB300Space>::value;

  KOKKOS_INLINE_FUNCTION View() {}
  // rank 0: one value
  template <int R = rank, std::enable_if_t<R == 0, bool> = true>
  explicit View(const std::string& label) : View(label, 1) {}
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()() const { return ptr_[0]; }
  View(const std::string& label, int64_t n0, int64_t n1 = 1, int64_t n2 = 1, int64_t n3 = 1, int64_t n4 = 1,
       int64_t n5 = 1) {
    set_extents(n0, n1, n2, n3, n4, n5);
    const size_t bytes = sizeof(value_type) * (size_t)size();
    trk_ = new Impl::Tracker();
    trk_->label = label;
    trk_->device = is_device;
    if (bytes) {
      if (is_device) check_cuda(cudaMalloc(&trk_->ptr, bytes), "View allocation");
      else trk_->ptr = std::malloc(bytes);
      if (is_device) check_cuda(cudaMemset(trk_->ptr, 0, bytes), "View initialisation");
      else std::memset(trk_->ptr, 0, bytes);
    }
    ptr_ = (value_type*)trk_->ptr;
  }
  // Unmanaged view of caller memory.
  KOKKOS_INLINE_FUNCTION View(value_type* p, int64_t n0, int64_t n1 = 1, int64_t n2 = 1, int64_t n3 = 1,
                              int64_t n4 = 1, int64_t n5 = 1)
      : ptr_(p) {
    set_extents(n0, n1, n2, n3, n4, n5);
  }
  KOKKOS_INLINE_FUNCTION View(const View& o) : ptr_(o.ptr_), trk_(o.trk_) {
    for (int d = 0; d < kMaxRank; ++d) { ext_[d] = o.ext_[d]; str_[d] = o.str_[d]; }
    retain();
  }
  // Same data type, layout and memory space spelled with other properties
  // (View<T*> and View<T*, LayoutLeft> on the device are the same view).
  template <class... P2,
            std::enable_if_t<std::is_same<typename View<DataType, P2...>::array_layout, array_layout>::value &&
                                 std::is_same<typename View<DataType, P2...>::memory_space, memory_space>::value &&
                                 !std::is_same<View<DataType, P2...>, View>::value,
                             bool> = true>
  KOKKOS_INLINE_FUNCTION View(const View<DataType, P2...>& o) : ptr_(o.ptr_), trk_(o.trk_) {
    for (int d = 0; d < kMaxRank; ++d) { ext_[d] = o.ext_[d]; str_[d] = o.str_[d]; }
    retain();
  }
  template <class D2, class... P2>
  friend class View;

  KOKKOS_INLINE_FUNCTION View& operator=(const View& o) {
    if (this != &o) {
      release();
      ptr_ = o.ptr_;
      trk_ = o.trk_;
      for (int d = 0; d < kMaxRank; ++d) { ext_[d] = o.ext_[d]; str_[d] = o.str_[d]; }
      retain();
    }
    return *this;
  }
  KOKKOS_INLINE_FUNCTION ~View() { release(); }

  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()(int64_t i) const { return ptr_[i * str_[0]]; }
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()(int64_t i, int64_t j) const { return ptr_[i * str_[0] + j * str_[1]]; }
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()(int64_t i, int64_t j, int64_t k) const {
    return ptr_[i * str_[0] + j * str_[1] + k * str_[2]];
  }
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()(int64_t i, int64_t j, int64_t k, int64_t l) const {
    return ptr_[i * str_[0] + j * str_[1] + k * str_[2] + l * str_[3]];
  }
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()(int64_t i, int64_t j, int64_t k, int64_t l, int64_t m) const {
    return ptr_[i * str_[0] + j * str_[1] + k * str_[2] + l * str_[3] + m * str_[4]];
  }
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator()(int64_t i, int64_t j, int64_t k, int64_t l, int64_t m,
                                                     int64_t q) const {
    return ptr_[i * str_[0] + j * str_[1] + k * str_[2] + l * str_[3] + m * str_[4] + q * str_[5]];
  }
  KOKKOS_FORCEINLINE_FUNCTION value_type& operator[](int64_t i) const { return ptr_[i]; }
  KOKKOS_INLINE_FUNCTION value_type* data() const { return ptr_; }
  KOKKOS_INLINE_FUNCTION int64_t extent(int d) const { return d < rank ? ext_[d] : 1; }
  KOKKOS_INLINE_FUNCTION int64_t extent_int(int d) const { return extent(d); }
  KOKKOS_INLINE_FUNCTION int64_t stride(int d) const { return str_[d]; }
  KOKKOS_INLINE_FUNCTION int64_t size() const {
    int64_t s = 1;
    for (int d = 0; d < rank; ++d) s *= ext_[d];
    return s;
  }
  KOKKOS_INLINE_FUNCTION int64_t span() const { return size(); }
  std::string label() const { return trk_ ? trk_->label : std::string(); }
  long use_count() const { return trk_ ? trk_->count.load() : 0; }

 private:
  KOKKOS_INLINE_FUNCTION void set_extents(int64_t n0, int64_t n1, int64_t n2, int64_t n3, int64_t n4, int64_t n5) {
    const int64_t e[kMaxRank] = {n0, n1, n2, n3, n4, n5};
    for (int d = 0; d < kMaxRank; ++d) ext_[d] = d < rank || (rank == 0 && d == 0) ? e[d] : 1;
    if (std::is_same<array_layout, LayoutLeft>::value) {
      int64_t s = 1;
      for (int d = 0; d < kMaxRank; ++d) { str_[d] = s; s *= ext_[d]; }
    } else {
      int64_t s = 1;
      for (int d = rank - 1; d >= 0; --d) { str_[d] = s; s *= ext_[d]; }
      for (int d = rank; d < kMaxRank; ++d) str_[d] = s;
    }
  }
  KOKKOS_INLINE_FUNCTION void retain() {
#ifndef __CUDA_ARCH__
    if (trk_) trk_->count.fetch_add(1);
#endif
  }
  KOKKOS_INLINE_FUNCTION void release() {
#ifndef __CUDA_ARCH__
    if (trk_ && trk_->count.fetch_sub(1) == 1) {
      if (trk_->ptr) {
        if (trk_->device) cudaFree(trk_->ptr);
        else std::free(trk_->ptr);
      }
      delete trk_;
    }
    trk_ = nullptr;
#endif
  }

  static constexpr int kMaxRank = 6;
  value_type* ptr_ = nullptr;
  Impl::Tracker* trk_ = nullptr;
  int64_t ext_[kMaxRank] = {0, 1, 1, 1, 1, 1};
  int64_t str_[kMaxRank] = {1, 1, 1, 1, 1, 1};
};

template <class D, class... P>
auto create_mirror_view(const View<D, P...>& v) {
  using L = typename View<D, P...>::array_layout;
  return View<D, L, HostSpace>(v.label() + "_mirror", v.extent(0), v.extent(1), v.extent(2), v.extent(3), v.extent(4),
                               v.extent(5));
}

// deep_copy between views of equal extents and layout (one contiguous copy)
template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
  static_assert(sizeof(typename View<D1, P1...>::value_type) == sizeof(typename View<D2, P2...>::value_type),
                "deep_copy: element types differ");
  if (dst.size() != src.size()) throw std::runtime_error("deep_copy: extents differ");
  check(gbk_deep_copy(dst.data(), src.data(), (int64_t)(sizeof(typename View<D1, P1...>::value_type) * dst.size()),
                      nullptr),
        "deep_copy");
  check_cuda(cudaStreamSynchronize(nullptr), "deep_copy");
}
// deep_copy(view, value): every element becomes value (the reference's
// ViewFill, core/src/Kokkos_CopyViews.hpp:58-260, 897); device views are
// filled by gbk_fill with 16-byte streaming stores.
template <class D, class... P>
void deep_copy(const View<D, P...>& dst, const typename View<D, P...>::value_type& value) {
  using T = typename View<D, P...>::value_type;
  const int64_t n = (int64_t)dst.size();
  if (View<D, P...>::is_device && (sizeof(T) == 1 || sizeof(T) == 2 || sizeof(T) == 4 || sizeof(T) == 8 ||
                                   sizeof(T) == 16)) {
    check(gbk_fill(dst.data(), &value, (int)sizeof(T), n, nullptr), "deep_copy(view, value)");
    check_cuda(cudaStreamSynchronize(nullptr), "deep_copy(view, value)");
  } else if (View<D, P...>::is_device) {
    throw std::runtime_error("deep_copy(view, value): element size must be 1, 2, 4, 8 or 16 bytes");
  } else {
    for (int64_t i = 0; i < n; ++i) dst.data()[i] = value;
  }
}

// ---------------------------------------------------------------------------
// Policies
struct ChunkSize {
  int value;
  explicit ChunkSize(int v) : value(v) {}
};

template <class ExecSpace = Experimental::GB300, class... Rest>
class RangePolicy {
 public:
  using execution_space = ExecSpace;
  using index_type = int64_t;
  RangePolicy(int64_t b, int64_t e) : begin_(b), end_(e) { validate(); }
  RangePolicy(const ExecSpace& s, int64_t b, int64_t e) : space_(s), begin_(b), end_(e) { validate(); }
  RangePolicy(int64_t b, int64_t e, ChunkSize c) : begin_(b), end_(e), chunk_(c.value) { validate(); }
  int64_t begin() const { return begin_; }
  int64_t end() const { return end_; }
  const ExecSpace& space() const { return space_; }
  int64_t chunk_size() const { return chunk_; }
  RangePolicy& set_chunk_size(int c) { chunk_ = c; return *this; }

 private:
  void validate() {
    if (end_ < begin_) throw std::runtime_error("Kokkos::RangePolicy bounds error: begin > end");
  }
  ExecSpace space_{};
  int64_t begin_ = 0, end_ = 0, chunk_ = 0;
};

enum class Iterate { Default, Left, Right };
template <unsigned N, Iterate OuterDir = Iterate::Default, Iterate InnerDir = Iterate::Default>
struct Rank {
  static_assert(N >= 2 && N <= 6, "Kokkos::Rank: MDRangePolicy ranks 2..6");
  static constexpr int rank = N;
  static constexpr Iterate outer_direction = OuterDir;
  static constexpr Iterate inner_direction = InnerDir;
};
template <class T>
struct IndexType {
  using type = T;
};

namespace Impl {
template <class T> struct is_rank : std::false_type {};
template <unsigned N, Iterate O, Iterate I> struct is_rank<Rank<N, O, I>> : std::true_type {};
template <class T> struct is_index_type : std::false_type {};
template <class T> struct is_index_type<IndexType<T>> : std::true_type {};
// The properties of an MDRangePolicy in any order (the reference's
// PolicyTraits): the Rank, an execution space, an IndexType and a work tag
// (any other class type).
template <class... P> struct MDProps {
  using rank = void;
  using space = Experimental::GB300;
  using tag = void;
  using index = int64_t;
};
template <class P0, class... P> struct MDProps<P0, P...> {
  using rest = MDProps<P...>;
  using rank = std::conditional_t<is_rank<P0>::value, P0, typename rest::rank>;
  using space = std::conditional_t<std::is_same<P0, Experimental::GB300>::value, P0, typename rest::space>;
  using index = typename std::conditional_t<is_index_type<P0>::value, P0, IndexType<typename rest::index>>::type;
  using tag = std::conditional_t<is_rank<P0>::value || std::is_same<P0, Experimental::GB300>::value ||
                                     is_index_type<P0>::value,
                                 typename rest::tag, P0>;
};
}  // namespace Impl

// MDRangePolicy<Rank<N[, outer, inner]>, ...>(lower, upper[, tile])
// (core/src/KokkosExp_MDRangePolicy.hpp:159-458): ranks 2..6, bounds as
// braced lists (their length fixes the rank for the deduction guides) or
// arrays.  Iteration directions default to Iterate::Left on this GPU space
// (dimension 0 fastest, as the reference's CUDA space,
// core/src/Cuda/Kokkos_Cuda_MDRangePolicy.hpp:24-36); the inner direction is
// the dimension that varies fastest between consecutive threads (Right: the
// last).  Tile sizes are checked as the reference checks them (at most 1024
// threads in a tile, the abort of KokkosExp_MDRangePolicy.hpp:416-424) and
// otherwise do not change the walk: every tile shape covers the same
// elements, and the flat walk keeps warps on consecutive addresses.
// (declared as a partial specialisation so that only the guides below deduce
// a braced-list policy, as the reference does, KokkosExp_MDRangePolicy.hpp:168-175)
template <class... Props>
class MDRangePolicy;
template <class P0, class... Props>
class MDRangePolicy<P0, Props...> {
  using props = Impl::MDProps<P0, Props...>;
  static_assert(!std::is_void<typename props::rank>::value, "Kokkos Error: MD iteration pattern not defined");

 public:
  using rank_type = typename props::rank;
  using execution_space = typename props::space;
  using work_tag = typename props::tag;
  using index_type = typename props::index;
  using execution_policy = MDRangePolicy;
  static constexpr int rank = rank_type::rank;
  static constexpr Iterate outer_direction =
      rank_type::outer_direction == Iterate::Default ? Iterate::Left : rank_type::outer_direction;
  static constexpr Iterate inner_direction =
      rank_type::inner_direction == Iterate::Default ? Iterate::Left : rank_type::inner_direction;

  template <class LT, size_t LN, class UT, size_t UN>
  MDRangePolicy(const LT (&lo)[LN], const UT (&up)[UN]) {
    static_assert(LN == rank && UN == rank, "MDRangePolicy: Constructor initializer lists have wrong size");
    set<LT, UT, int64_t>(lo, up, nullptr, 0);
  }
  template <class LT, size_t LN, class UT, size_t UN, class TT, size_t TN>
  MDRangePolicy(const LT (&lo)[LN], const UT (&up)[UN], const TT (&tile)[TN]) {
    static_assert(LN == rank && UN == rank && TN <= rank, "MDRangePolicy: Constructor initializer lists have wrong size");
    set(lo, up, tile, TN);
  }
  template <class LT, size_t LN, class UT, size_t UN>
  MDRangePolicy(const execution_space& s, const LT (&lo)[LN], const UT (&up)[UN]) : space_(s) {
    static_assert(LN == rank && UN == rank, "MDRangePolicy: Constructor initializer lists have wrong size");
    set<LT, UT, int64_t>(lo, up, nullptr, 0);
  }
  template <class LT, size_t LN, class UT, size_t UN, class TT, size_t TN>
  MDRangePolicy(const execution_space& s, const LT (&lo)[LN], const UT (&up)[UN], const TT (&tile)[TN]) : space_(s) {
    static_assert(LN == rank && UN == rank && TN <= rank, "MDRangePolicy: Constructor initializer lists have wrong size");
    set(lo, up, tile, TN);
  }

  // bounds of mixed integer types ({0, n}): the reference's point_type
  // constructors (KokkosExp_MDRangePolicy.hpp:249-259)
  using point_type = std::array<int64_t, rank>;
  MDRangePolicy(const point_type& lo, const point_type& up, const point_type& tile = point_type{}) {
    set<int64_t, int64_t, int64_t>(lo.data(), up.data(), tile.data(), rank);
  }
  MDRangePolicy(const execution_space& s, const point_type& lo, const point_type& up,
                const point_type& tile = point_type{})
      : space_(s) {
    set<int64_t, int64_t, int64_t>(lo.data(), up.data(), tile.data(), rank);
  }

  int64_t lower(int d) const { return lo_[d]; }
  int64_t upper(int d) const { return up_[d]; }
  int64_t tile(int d) const { return tile_[d]; }
  const execution_space& space() const { return space_; }

 private:
  template <class LT, class UT, class TT>
  void set(const LT* lo, const UT* up, const TT* tile, size_t nt) {
    int64_t prod = 1;
    for (int d = 0; d < rank; ++d) {
      lo_[d] = (int64_t)lo[d];
      up_[d] = (int64_t)up[d];
      if (up_[d] < lo_[d])
        throw std::runtime_error("Kokkos::MDRangePolicy bounds error: The lower bound is greater than its upper bound");
      tile_[d] = tile && (size_t)d < nt ? (int64_t)tile[d] : 0;
      prod *= tile_[d] > 0 ? tile_[d] : 1;
    }
    if (prod > 1024)
      throw std::runtime_error(
          "ExecSpace Error: MDRange tile dims exceed maximum number of threads per block - choose smaller tile dims");
  }
  execution_space space_{};
  int64_t lo_[6] = {0, 0, 0, 0, 0, 0}, up_[6] = {0, 0, 0, 0, 0, 0}, tile_[6] = {0, 0, 0, 0, 0, 0};
};

// deduction guides (KokkosExp_MDRangePolicy.hpp:429-458)
template <class LT, size_t N, class UT>
MDRangePolicy(const LT (&)[N], const UT (&)[N]) -> MDRangePolicy<Rank<N>>;
template <class LT, size_t N, class UT, class TT, size_t TN>
MDRangePolicy(const LT (&)[N], const UT (&)[N], const TT (&)[TN]) -> MDRangePolicy<Rank<N>>;
template <class LT, size_t N, class UT>
MDRangePolicy(const Experimental::GB300&, const LT (&)[N], const UT (&)[N]) -> MDRangePolicy<Rank<N>>;
template <class LT, size_t N, class UT, class TT, size_t TN>
MDRangePolicy(const Experimental::GB300&, const LT (&)[N], const UT (&)[N], const TT (&)[TN]) -> MDRangePolicy<Rank<N>>;

// Kokkos::pair (core/src/Kokkos_Pair.hpp): a host-device pair.
template <class T1, class T2>
struct pair {
  using first_type = T1;
  using second_type = T2;
  T1 first;
  T2 second;
  KOKKOS_FORCEINLINE_FUNCTION constexpr pair() : first(), second() {}
  KOKKOS_FORCEINLINE_FUNCTION constexpr pair(const T1& a, const T2& b) : first(a), second(b) {}
};
template <class T1, class T2>
KOKKOS_FORCEINLINE_FUNCTION constexpr pair<T1, T2> make_pair(T1 a, T2 b) {
  return pair<T1, T2>(a, b);
}

struct AUTO_t {};
constexpr AUTO_t AUTO{};

namespace Impl {
// Team collectives of TeamMember, defined in parallel.hpp.
template <class Red, class V> __device__ V team_allreduce(const Red& red, V v);
template <class T> __device__ T team_exclusive_sum(const T& v, T* global_accum);
template <class T> __device__ void team_bcast(T& v, int root);
}  // namespace Impl

// Team member: one team = one CTA (team_size threads), league ranks
// distributed over the grid (core/src/Cuda/Kokkos_Cuda_Team.hpp:72-360 is the
// reference's device member).
// Member functions are host-device (they are called from KOKKOS_LAMBDA
// bodies); they only do work in device code.
class TeamMember {
 public:
  KOKKOS_INLINE_FUNCTION TeamMember(int64_t league_rank, int64_t league_size) : lr_(league_rank), ls_(league_size) {}
  KOKKOS_INLINE_FUNCTION int64_t league_rank() const { return lr_; }
  KOKKOS_INLINE_FUNCTION int64_t league_size() const { return ls_; }
  KOKKOS_INLINE_FUNCTION int team_rank() const {
#ifdef __CUDA_ARCH__
    return threadIdx.x;
#else
    return 0;
#endif
  }
  KOKKOS_INLINE_FUNCTION int team_size() const {
#ifdef __CUDA_ARCH__
    return blockDim.x;
#else
    return 1;
#endif
  }
  KOKKOS_INLINE_FUNCTION void team_barrier() const {
#ifdef __CUDA_ARCH__
    __syncthreads();
#endif
  }
  // Every thread receives the root thread's value
  // (core/src/Cuda/Kokkos_Cuda_Team.hpp:123-170).
  template <class T>
  KOKKOS_INLINE_FUNCTION void team_broadcast(T& val, int root) const {
#ifdef __CUDA_ARCH__
    Impl::team_bcast(val, root);
#endif
  }
  template <class F, class T>
  KOKKOS_INLINE_FUNCTION void team_broadcast(const F& f, T& val, int root) const {
#ifdef __CUDA_ARCH__
    f(val);
    Impl::team_bcast(val, root);
#endif
  }
  // Join of every thread's reducer.reference() (or `value`) over the team;
  // every thread's reducer.reference() receives the result
  // (Kokkos_Cuda_Team.hpp:188-210).
  template <class Red>
  KOKKOS_INLINE_FUNCTION void team_reduce(const Red& red) const {
#ifdef __CUDA_ARCH__
    red.reference() = Impl::team_allreduce(red, red.reference());
#endif
  }
  template <class Red>
  KOKKOS_INLINE_FUNCTION void team_reduce(const Red& red, const typename Red::value_type& value) const {
#ifdef __CUDA_ARCH__
    red.reference() = Impl::team_allreduce(red, value);
#endif
  }
  // Exclusive prefix sum of `value` in team_rank order.  With global_accum,
  // the last thread adds the team's total to *global_accum atomically and
  // every thread's result is offset by the value it held before
  // (Kokkos_Cuda_Team.hpp:223-262; the order of teams is unspecified).
  template <class T>
  KOKKOS_INLINE_FUNCTION T team_scan(const T& value, T* global_accum) const {
#ifdef __CUDA_ARCH__
    return Impl::team_exclusive_sum(value, global_accum);
#else
    (void)value;
    (void)global_accum;
    return T();
#endif
  }
  template <class T>
  KOKKOS_INLINE_FUNCTION T team_scan(const T& value) const {
    return team_scan<T>(value, nullptr);
  }

 private:
  int64_t lr_, ls_;
};

template <class ExecSpace = Experimental::GB300, class... Rest>
class TeamPolicy {
 public:
  using execution_space = ExecSpace;
  using member_type = TeamMember;
  TeamPolicy(int64_t league, int team) : league_(league), team_(team) { validate(); }
  TeamPolicy(int64_t league, AUTO_t) : league_(league), team_(256) { validate(); }
  TeamPolicy(int64_t league, int team, int) : league_(league), team_(team) { validate(); }
  TeamPolicy(const ExecSpace& s, int64_t league, int team) : space_(s), league_(league), team_(team) { validate(); }
  TeamPolicy(const ExecSpace& s, int64_t league, AUTO_t) : space_(s), league_(league), team_(256) { validate(); }
  int64_t league_size() const { return league_; }
  int team_size() const { return team_; }
  const ExecSpace& space() const { return space_; }

 private:
  void validate() {
    if (team_ < 32 || team_ > 1024 || team_ % 32) throw std::runtime_error("TeamPolicy: team size must be 32..1024, multiple of 32");
    if (league_ < 0) throw std::runtime_error("TeamPolicy: negative league size");
  }
  ExecSpace space_{};
  int64_t league_ = 0;
  int team_ = 256;
};

template <class IndexT = int64_t>
struct TeamThreadRangeBoundaries {
  const TeamMember& member;
  int64_t begin, end;
};
KOKKOS_INLINE_FUNCTION TeamThreadRangeBoundaries<> TeamThreadRange(const TeamMember& m, int64_t n) {
  return {m, 0, n};
}
KOKKOS_INLINE_FUNCTION TeamThreadRangeBoundaries<> TeamThreadRange(const TeamMember& m, int64_t b, int64_t e) {
  return {m, b, e};
}

struct PerTeamTag {
  const TeamMember& member;
};
KOKKOS_INLINE_FUNCTION PerTeamTag PerTeam(const TeamMember& m) { return {m}; }
template <class F>
KOKKOS_INLINE_FUNCTION void single(const PerTeamTag& t, const F& f) {
#ifdef __CUDA_ARCH__
  if (t.member.team_rank() == 0) f();
  __syncthreads();
#endif
}

}  // namespace gb300k
