// Out-of-line parts of the GB300 space: instance management, fences, device
// memory, deep_copy, and the registration with Kokkos' ExecSpaceManager
// (core/src/impl/Kokkos_ExecSpaceManager.hpp:157-160; the pattern of
// core/src/Serial/Kokkos_Serial.cpp:183-196).  Compiled with nvcc beside the
// Kokkos core sources and linked with libgbk.so.
#ifndef KOKKOS_IMPL_PUBLIC_INCLUDE
#define KOKKOS_IMPL_PUBLIC_INCLUDE
#endif

#include <Kokkos_Core.hpp>

#include <impl/Kokkos_Error.hpp>
#include <impl/Kokkos_ExecSpaceManager.hpp>
#include <impl/Kokkos_SharedAlloc.hpp>
#include <impl/Kokkos_SharedAlloc_timpl.hpp>

#include <atomic>
#include <ostream>
#include <string>

namespace Kokkos {
namespace Impl {

void gb300_check(int status, const char* what) {
  if (status == GBK_OK) return;
  throw_runtime_exception(std::string("Kokkos::Experimental::GB300: ") + what + ": " + gbk_status_string(status));
}

void gb300_deep_copy(void* dst, const void* src, size_t n) {
  gb300_check(gbk_deep_copy(dst, src, (int64_t)n, nullptr), "deep_copy");
  gb300_check_cuda(cudaStreamSynchronize(nullptr), "deep_copy");
}

void gb300_deep_copy_async(const Kokkos::Experimental::GB300& exec, void* dst, const void* src, size_t n) {
  gb300_check(gbk_deep_copy(dst, src, (int64_t)n, (gbk_stream_t)exec.stream()), "deep_copy");
}

namespace {
std::atomic<uint32_t> g_instance_ids{1};
bool g_initialized = false;
// The instance a default-constructed GB300 refers to (created by initialize).
HostSharedPtr<Kokkos::Experimental::Impl::GB300Internal> g_default;
}  // namespace

}  // namespace Impl

namespace Experimental {
namespace Impl {
GB300Internal::~GB300Internal() {
  if (owns_stream && stream) cudaStreamDestroy(stream);
}
}  // namespace Impl

// ---- GB300 ----------------------------------------------------------------
GB300::GB300() : m_space_instance(Kokkos::Impl::g_default) {
  if (!m_space_instance.get())
    Kokkos::abort("Kokkos::Experimental::GB300 instance constructed before Kokkos::initialize()");
}

GB300::GB300(cudaStream_t stream) {
  auto* in = new Impl::GB300Internal();
  in->device = Kokkos::Impl::g_default.get() ? Kokkos::Impl::g_default->device : 0;
  in->stream = stream;
  in->owns_stream = false;
  in->instance_id = Kokkos::Impl::g_instance_ids++;
  in->sm_count = Kokkos::Impl::g_default.get() ? Kokkos::Impl::g_default->sm_count : 1;
  m_space_instance = Kokkos::Impl::HostSharedPtr<Impl::GB300Internal>(in);
}

void GB300::fence(const std::string& name) const {
  Kokkos::Tools::Experimental::Impl::profile_fence_event<GB300>(
      name, Kokkos::Tools::Experimental::Impl::DirectFenceIDHandle{impl_instance_id()}, [&]() {
        // synchronises the stream and raises any device-side status
        Kokkos::Impl::gb300_check(gbk_stream_check((gbk_stream_t)stream()), "fence");
      });
}

void GB300::impl_fence_read(const std::string& name, const void* device_src, void* host_dst, size_t bytes) const {
  Kokkos::Tools::Experimental::Impl::profile_fence_event<GB300>(
      name, Kokkos::Tools::Experimental::Impl::DirectFenceIDHandle{impl_instance_id()}, [&]() {
        Kokkos::Impl::gb300_check(gbk_fence_read((gbk_stream_t)stream(), device_src, host_dst, (int64_t)bytes),
                                  "fence");
      });
}

void GB300::impl_static_fence(const std::string& name) {
  Kokkos::Tools::Experimental::Impl::profile_fence_event<GB300>(
      name, Kokkos::Tools::Experimental::SpecialSynchronizationCases::GlobalDeviceSynchronization,
      []() { Kokkos::Impl::gb300_check_cuda(cudaDeviceSynchronize(), "static fence"); });
}

int GB300::concurrency() const { return sm_count() * 2048; }

void GB300::print_configuration(std::ostream& os, bool verbose) const {
  int sm = 0, ma = 0, mi = 0;
  int64_t l2 = 0;
  gbk_device_info(&sm, &ma, &mi, &l2);
  os << "Device Execution Space:\n  KOKKOS_ENABLE_GB300: yes\n";
  os << "  device " << device_id() << ": sm_" << ma << mi << ", " << sm << " SMs, L2 " << (l2 >> 20) << " MiB\n";
  if (verbose) os << "  library version " << gbk_version() << "\n";
}

void GB300::impl_initialize(InitializationSettings const& settings) {
  const int dev = settings.has_device_id() ? settings.get_device_id() : 0;
  Kokkos::Impl::gb300_check_cuda(cudaSetDevice(dev), "initialize: cudaSetDevice");
  int sm = 0, ma = 0, mi = 0;
  int64_t l2 = 0;
  Kokkos::Impl::gb300_check(gbk_device_info(&sm, &ma, &mi, &l2), "initialize: device query");
  auto* in = new Impl::GB300Internal();
  in->device = dev;
  in->owns_stream = true;
  in->instance_id = Kokkos::Impl::g_instance_ids++;
  in->sm_count = sm > 0 ? sm : 1;
  Kokkos::Impl::gb300_check_cuda(cudaStreamCreateWithFlags(&in->stream, cudaStreamNonBlocking), "initialize");
  Kokkos::Impl::g_default = Kokkos::Impl::HostSharedPtr<Impl::GB300Internal>(in);
  Kokkos::Impl::g_initialized = true;
}

void GB300::impl_finalize() {
  if (Kokkos::Impl::g_default.get()) cudaStreamSynchronize(Kokkos::Impl::g_default->stream);
  Kokkos::Impl::g_default = Kokkos::Impl::HostSharedPtr<Impl::GB300Internal>();
  Kokkos::Impl::g_initialized = false;
}

bool GB300::impl_is_initialized() { return Kokkos::Impl::g_initialized; }

// ---- GB300Space -------------------------------------------------------------
GB300Space::GB300Space() : m_device(0) { cudaGetDevice(&m_device); }

void* GB300Space::allocate(const size_t n) const { return allocate("[unlabeled]", n); }
void* GB300Space::allocate(const GB300&, const size_t n) const { return allocate("[unlabeled]", n); }
void* GB300Space::allocate(const GB300&, const char* label, const size_t n, const size_t logical) const {
  return allocate(label, n, logical);
}
void* GB300Space::allocate(const char* label, const size_t n, const size_t logical) const {
  void* p = nullptr;
  if (n) {
    const cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      Kokkos::Impl::throw_runtime_exception(std::string("Kokkos::Experimental::GB300Space::allocate(") + label +
                                            "): out of device memory for " + std::to_string(n) + " bytes");
    }
  }
  if (Kokkos::Profiling::profileLibraryLoaded())
    Kokkos::Profiling::allocateData(Kokkos::Tools::make_space_handle(name()), label, p, logical ? logical : n);
  return p;
}
void GB300Space::deallocate(void* const p, const size_t n) const { deallocate("[unlabeled]", p, n); }
void GB300Space::deallocate(const char* label, void* const p, const size_t n, const size_t logical) const {
  if (Kokkos::Profiling::profileLibraryLoaded())
    Kokkos::Profiling::deallocateData(Kokkos::Tools::make_space_handle(name()), label, p, logical ? logical : n);
  if (p) cudaFree(p);
}

}  // namespace Experimental

namespace Impl {
int g_gb300_space_factory_initialized =
    initialize_space_factory<Kokkos::Experimental::GB300>("170_GB300");
}  // namespace Impl
}  // namespace Kokkos

KOKKOS_IMPL_HOST_INACCESSIBLE_SHARED_ALLOCATION_RECORD_EXPLICIT_INSTANTIATION(Kokkos::Experimental::GB300Space);
