// Kokkos::Experimental::GB300: an execution space on one GB300 GPU, and
// GB300Space, its device memory space.
//
// This is the backend half of the drop-in: with this directory on the include
// path ahead of the Kokkos sources (KokkosCore_config.h here enables it),
// Kokkos' own dispatch (parallel_for / parallel_reduce / parallel_scan,
// Kokkos_Parallel.hpp, Kokkos_Parallel_Reduce.hpp) instantiates the
// Impl::ParallelFor / ParallelReduce / ParallelScan / ParallelScanWithTotal
// specialisations of Kokkos_GB300_Parallel_*.hpp for RangePolicy,
// MDRangePolicy and TeamPolicy (the contract of core/src/Kokkos_Core_fwd.hpp:
// 299-328), View allocation goes through GB300Space, deep_copy through the
// DeepCopy specialisations below, ScatterView picks its defaults from
// Kokkos_GB300_Hooks.hpp and Kokkos::sort / sort_by_key on a GB300 View run
// the library's radix sort.  The space registers itself with Kokkos'
// ExecSpaceManager (Kokkos_GB300.cpp), so Kokkos::initialize / finalize /
// fence cover it like any other space.
//
// The space's requirements are those checked by check_valid_execution_space
// (core/src/impl/Kokkos_ExecSpaceManager.hpp:17-108): default-constructible,
// regular, at most two pointers, the member typedefs, fence() / fence(name) /
// impl_static_fence(name), concurrency(), print_configuration(os, verbose),
// impl_initialize(settings) / impl_finalize().  The device model it follows is
// core/src/Cuda/Kokkos_Cuda.hpp:95-260 and Kokkos_CudaSpace.hpp:59-585; the
// code here is this project's (the library's C ABI, include/gbk.h, does the
// device work).
#ifndef KOKKOS_GB300_HPP_
#define KOKKOS_GB300_HPP_

#include <Kokkos_Macros.hpp>
#if defined(KOKKOS_ENABLE_GB300)

#include <Kokkos_Core_fwd.hpp>

#include <cstddef>
#include <cstdint>
#include <iosfwd>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include <Kokkos_HostSpace.hpp>
#include <Kokkos_Layout.hpp>
#include <Kokkos_MemoryTraits.hpp>
#include <Kokkos_ScratchSpace.hpp>
#include <impl/Kokkos_HostSharedPtr.hpp>
#include <impl/Kokkos_InitializationSettings.hpp>
#include <impl/Kokkos_Profiling_Interface.hpp>
#include <impl/Kokkos_SharedAlloc.hpp>
#include <impl/Kokkos_Tools.hpp>
#include <impl/Kokkos_ZeroMemset_fwd.hpp>

#include <gbk.h>

namespace Kokkos {
namespace Experimental {

// ---------------------------------------------------------------------------
// GB300Space: device memory (cudaMalloc) of the GPU the space runs on.  Not
// host-accessible; deep_copy moves data to and from HostSpace.
class GB300Space {
 public:
  using memory_space = GB300Space;
  using execution_space = Kokkos::Experimental::GB300;
  using device_type = Kokkos::Device<execution_space, memory_space>;
  using size_type = unsigned int;

  GB300Space();
  GB300Space(GB300Space&&) = default;
  GB300Space(const GB300Space&) = default;
  GB300Space& operator=(GB300Space&&) = default;
  GB300Space& operator=(const GB300Space&) = default;
  ~GB300Space() = default;

  void* allocate(const GB300& exec, const size_t arg_alloc_size) const;
  void* allocate(const GB300& exec, const char* arg_label, const size_t arg_alloc_size,
                 const size_t arg_logical_size = 0) const;
  void* allocate(const size_t arg_alloc_size) const;
  void* allocate(const char* arg_label, const size_t arg_alloc_size, const size_t arg_logical_size = 0) const;
  void deallocate(void* const arg_alloc_ptr, const size_t arg_alloc_size) const;
  void deallocate(const char* arg_label, void* const arg_alloc_ptr, const size_t arg_alloc_size,
                  const size_t arg_logical_size = 0) const;

  static constexpr const char* name() { return "GB300"; }

 private:
  int m_device;
};

namespace Impl {
// Per-instance state: one CUDA stream on one device.
struct GB300Internal {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  uint32_t instance_id = 0;
  int sm_count = 1;
  std::mutex mutex;  // serialises host-side set-up of launches on this instance
  ~GB300Internal();
};
}  // namespace Impl

// ---------------------------------------------------------------------------
// GB300: the execution space.  A default-constructed instance runs on the
// stream created by Kokkos::initialize; GB300(stream) wraps a caller's stream
// (the caller keeps ownership).
class GB300 {
 public:
  using execution_space = GB300;
  using memory_space = GB300Space;
  using device_type = Kokkos::Device<execution_space, memory_space>;
  using array_layout = Kokkos::LayoutLeft;
  using size_type = memory_space::size_type;
  using scratch_memory_space = Kokkos::ScratchMemorySpace<GB300>;

  GB300();
  explicit GB300(cudaStream_t stream);

  // Asynchronous work on this instance finishes; device-side errors (a bounded
  // wait that gave up, a key outside a bin range) raise as in the CUDA space
  // (core/src/Cuda/Kokkos_Cuda_Error.hpp:33-67).
  void fence(const std::string& name = "Kokkos::Experimental::GB300::fence: Unnamed Instance Fence") const;
  static void impl_static_fence(const std::string& name);
  // fence() that also copies `bytes` (at most 256) from device memory into
  // host memory behind the same synchronisation (a host-scalar reduce result)
  void impl_fence_read(const std::string& name, const void* device_src, void* host_dst, size_t bytes) const;

  int concurrency() const;  // SMs x 2048 resident threads
  // An index in [0, concurrency()) for the calling device thread: its SM's
  // id x 2048 plus its place among the CTAs of its size that fit on one SM
  // (threads resident on one SM at once can share an index); 0 on the host.
  KOKKOS_INLINE_FUNCTION static int impl_hardware_thread_id() noexcept {
    KOKKOS_IF_ON_DEVICE((unsigned sm; asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
                         const unsigned per = 2048u / blockDim.x;
                         return (int)(sm * 2048u + (blockIdx.x % per) * blockDim.x + threadIdx.x);))
    KOKKOS_IF_ON_HOST((return 0;))
  }
  int impl_max_hardware_threads() const { return concurrency(); }
  void print_configuration(std::ostream& os, bool verbose = false) const;

  static void impl_initialize(InitializationSettings const&);
  static void impl_finalize();
  static bool impl_is_initialized();
  static const char* name() { return "GB300"; }

  cudaStream_t stream() const { return m_space_instance->stream; }
  int device_id() const { return m_space_instance->device; }
  int sm_count() const { return m_space_instance->sm_count; }
  uint32_t impl_instance_id() const noexcept { return m_space_instance->instance_id; }
  Impl::GB300Internal* impl_internal_space_instance() const { return m_space_instance.get(); }

  friend bool operator==(GB300 const& a, GB300 const& b) {
    return a.impl_internal_space_instance() == b.impl_internal_space_instance();
  }
  friend bool operator!=(GB300 const& a, GB300 const& b) { return !(a == b); }

 private:
  Kokkos::Impl::HostSharedPtr<Impl::GB300Internal> m_space_instance;
};

}  // namespace Experimental

// ---------------------------------------------------------------------------
namespace Tools {
namespace Experimental {
template <>
struct DeviceTypeTraits<Kokkos::Experimental::GB300> {
  // Kokkos Tools know the device family as CUDA (a GB300 is a CUDA device).
  static constexpr DeviceType id = DeviceType::Cuda;
  static int device_id(const Kokkos::Experimental::GB300& exec) { return exec.device_id(); }
};
}  // namespace Experimental
}  // namespace Tools

namespace Impl {

// Status of a library call: a device-side timeout or out-of-range key is a
// runtime error, a bad argument an abort-worthy error; both raise the
// reference's runtime exception.
void gb300_check(int status, const char* what);
inline void gb300_check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) gb300_check(GBK_ERR_CUDA, what);
}

// ---- memory space access (the CUDA space's table,
// core/src/Cuda/Kokkos_CudaSpace.hpp:350-384, for a device-only space) ------
template <>
struct MemorySpaceAccess<Kokkos::HostSpace, Kokkos::Experimental::GB300Space> {
  enum : bool { assignable = false };
  enum : bool { accessible = false };
  enum : bool { deepcopy = true };
};
template <>
struct MemorySpaceAccess<Kokkos::Experimental::GB300Space, Kokkos::HostSpace> {
  enum : bool { assignable = false };
  enum : bool { accessible = false };
  enum : bool { deepcopy = true };
};
// A team's scratch is reachable from the code of the space that owns it (a
// managed View over ScratchMemorySpace<GB300> asks this of the space).
template <>
struct MemorySpaceAccess<Kokkos::Experimental::GB300Space, Kokkos::ScratchMemorySpace<Kokkos::Experimental::GB300>> {
  enum : bool { assignable = false };
  enum : bool { accessible = true };
  enum : bool { deepcopy = false };
};

// ---- deep_copy: host<->device and device<->device through the library ----
void gb300_deep_copy(void* dst, const void* src, size_t n);                      // synchronous
void gb300_deep_copy_async(const Kokkos::Experimental::GB300& exec, void* dst, const void* src, size_t n);

template <>
struct DeepCopy<Kokkos::Experimental::GB300Space, Kokkos::Experimental::GB300Space, Kokkos::Experimental::GB300> {
  DeepCopy(void* dst, const void* src, size_t n) { gb300_deep_copy(dst, src, n); }
  DeepCopy(const Kokkos::Experimental::GB300& exec, void* dst, const void* src, size_t n) {
    gb300_deep_copy_async(exec, dst, src, n);
  }
};
template <>
struct DeepCopy<Kokkos::Experimental::GB300Space, HostSpace, Kokkos::Experimental::GB300> {
  DeepCopy(void* dst, const void* src, size_t n) { gb300_deep_copy(dst, src, n); }
  DeepCopy(const Kokkos::Experimental::GB300& exec, void* dst, const void* src, size_t n) {
    gb300_deep_copy_async(exec, dst, src, n);
  }
};
template <>
struct DeepCopy<HostSpace, Kokkos::Experimental::GB300Space, Kokkos::Experimental::GB300> {
  DeepCopy(void* dst, const void* src, size_t n) { gb300_deep_copy(dst, src, n); }
  DeepCopy(const Kokkos::Experimental::GB300& exec, void* dst, const void* src, size_t n) {
    gb300_deep_copy_async(exec, dst, src, n);
  }
};
// Copies ordered by another execution space: fence it, then copy.
template <class ExecutionSpace>
struct DeepCopy<Kokkos::Experimental::GB300Space, Kokkos::Experimental::GB300Space, ExecutionSpace,
                std::enable_if_t<!std::is_same_v<ExecutionSpace, Kokkos::Experimental::GB300>>> {
  DeepCopy(void* dst, const void* src, size_t n) { gb300_deep_copy(dst, src, n); }
  DeepCopy(const ExecutionSpace& exec, void* dst, const void* src, size_t n) {
    exec.fence("Kokkos::Impl::DeepCopy<GB300Space, GB300Space, ExecutionSpace>: fence before copy");
    gb300_deep_copy(dst, src, n);
  }
};
template <class ExecutionSpace>
struct DeepCopy<Kokkos::Experimental::GB300Space, HostSpace, ExecutionSpace,
                std::enable_if_t<!std::is_same_v<ExecutionSpace, Kokkos::Experimental::GB300>>> {
  DeepCopy(void* dst, const void* src, size_t n) { gb300_deep_copy(dst, src, n); }
  DeepCopy(const ExecutionSpace& exec, void* dst, const void* src, size_t n) {
    exec.fence("Kokkos::Impl::DeepCopy<GB300Space, HostSpace, ExecutionSpace>: fence before copy");
    gb300_deep_copy(dst, src, n);
  }
};
template <class ExecutionSpace>
struct DeepCopy<HostSpace, Kokkos::Experimental::GB300Space, ExecutionSpace,
                std::enable_if_t<!std::is_same_v<ExecutionSpace, Kokkos::Experimental::GB300>>> {
  DeepCopy(void* dst, const void* src, size_t n) { gb300_deep_copy(dst, src, n); }
  DeepCopy(const ExecutionSpace& exec, void* dst, const void* src, size_t n) {
    exec.fence("Kokkos::Impl::DeepCopy<HostSpace, GB300Space, ExecutionSpace>: fence before copy");
    gb300_deep_copy(dst, src, n);
  }
};

// ---- View access checks --------------------------------------------------
// Kokkos checks a View access in device code against DefaultExecutionSpace
// and in host code against DefaultHostExecutionSpace
// (core/src/Kokkos_Core_fwd.hpp:230-256, View/Kokkos_ViewAccessPreconditionsCheck.hpp:
// 70-77, View/Kokkos_ViewMapping.hpp:3480-3490).  Kokkos' list of default
// spaces (Kokkos_Core_fwd.hpp:96-121) has no entry for a space added beside
// the built-in ones, so with this backend both are Serial, and the stock checks
// would reject every device access to GB300 memory.  These specialisations
// state the real rule: GB300Space is accessible from device code and not
// from host code; HostSpace is accessible from host code and not from
// device code.
template <class MemorySpace, class AccessSpace, bool>
struct RuntimeCheckBasicViewMemoryAccessViolation;
template <class MemorySpace, class AccessSpace, bool>
struct RuntimeCheckViewMemoryAccessViolation;

// (the same for the space's team scratch, ScratchMemorySpace<GB300>)
template <>
struct RuntimeCheckMemoryAccessViolation<Kokkos::Experimental::GB300Space, Kokkos::DefaultExecutionSpace, false> {
  KOKKOS_FUNCTION RuntimeCheckMemoryAccessViolation(char const* const msg) {
    (void)msg;
    KOKKOS_IF_ON_HOST((Kokkos::abort(msg);))
  }
};
template <>
struct RuntimeCheckMemoryAccessViolation<Kokkos::ScratchMemorySpace<Kokkos::Experimental::GB300>,
                                         Kokkos::DefaultExecutionSpace, false> {
  KOKKOS_FUNCTION RuntimeCheckMemoryAccessViolation(char const* const msg) {
    (void)msg;
    KOKKOS_IF_ON_HOST((Kokkos::abort(msg);))
  }
};
template <>
struct RuntimeCheckMemoryAccessViolation<Kokkos::HostSpace, Kokkos::DefaultExecutionSpace, true> {
  KOKKOS_FUNCTION RuntimeCheckMemoryAccessViolation(char const* const msg) {
    (void)msg;
    KOKKOS_IF_ON_DEVICE((Kokkos::abort(msg);))
  }
};
template <>
struct RuntimeCheckBasicViewMemoryAccessViolation<Kokkos::Experimental::GB300Space, Kokkos::DefaultExecutionSpace,
                                                  false> {
  KOKKOS_FUNCTION RuntimeCheckBasicViewMemoryAccessViolation(SharedAllocationTracker const&) {
    KOKKOS_IF_ON_HOST(
        (Kokkos::abort("Kokkos::View ERROR: attempt to access inaccessible memory space (GB300Space from host code)");))
  }
};
template <>
struct RuntimeCheckBasicViewMemoryAccessViolation<Kokkos::ScratchMemorySpace<Kokkos::Experimental::GB300>,
                                                  Kokkos::DefaultExecutionSpace, false> {
  KOKKOS_FUNCTION RuntimeCheckBasicViewMemoryAccessViolation(SharedAllocationTracker const&) {
    KOKKOS_IF_ON_HOST((Kokkos::abort(
        "Kokkos::View ERROR: attempt to access inaccessible memory space (GB300 team scratch from host code)");))
  }
};
template <>
struct RuntimeCheckBasicViewMemoryAccessViolation<Kokkos::HostSpace, Kokkos::DefaultExecutionSpace, true> {
  KOKKOS_FUNCTION RuntimeCheckBasicViewMemoryAccessViolation(SharedAllocationTracker const&) {
    KOKKOS_IF_ON_DEVICE(
        (Kokkos::abort("Kokkos::View ERROR: attempt to access inaccessible memory space (HostSpace from device code)");))
  }
};
template <>
struct RuntimeCheckViewMemoryAccessViolation<Kokkos::Experimental::GB300Space, Kokkos::DefaultExecutionSpace, false> {
  template <class Track, class Map>
  KOKKOS_FUNCTION RuntimeCheckViewMemoryAccessViolation(char const* const msg, Track const&, Map const&) {
    (void)msg;
    KOKKOS_IF_ON_HOST((Kokkos::abort(msg);))
  }
};
template <>
struct RuntimeCheckViewMemoryAccessViolation<Kokkos::ScratchMemorySpace<Kokkos::Experimental::GB300>,
                                             Kokkos::DefaultExecutionSpace, false> {
  template <class Track, class Map>
  KOKKOS_FUNCTION RuntimeCheckViewMemoryAccessViolation(char const* const msg, Track const&, Map const&) {
    (void)msg;
    KOKKOS_IF_ON_HOST((Kokkos::abort(msg);))
  }
};
template <>
struct RuntimeCheckViewMemoryAccessViolation<Kokkos::HostSpace, Kokkos::DefaultExecutionSpace, true> {
  template <class Track, class Map>
  KOKKOS_FUNCTION RuntimeCheckViewMemoryAccessViolation(char const* const msg, Track const&, Map const&) {
    (void)msg;
    KOKKOS_IF_ON_DEVICE((Kokkos::abort(msg);))
  }
};

// ---- deep_copy(view, 0) on the space's stream --------------------------------
template <>
struct ZeroMemset<Kokkos::Experimental::GB300> {
  ZeroMemset(const Kokkos::Experimental::GB300& exec, void* dst, size_t cnt) {
    gb300_check(gbk_memset(dst, 0, (int64_t)cnt, (gbk_stream_t)exec.stream()), "ZeroMemset<GB300>");
  }
};

}  // namespace Impl
}  // namespace Kokkos

KOKKOS_IMPL_HOST_INACCESSIBLE_SHARED_ALLOCATION_SPECIALIZATION(Kokkos::Experimental::GB300Space);

#endif  // KOKKOS_ENABLE_GB300
#endif  // KOKKOS_GB300_HPP_
