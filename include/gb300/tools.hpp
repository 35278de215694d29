// Kokkos Tools profiling hooks of the header path: the dispatch side of
// core/src/impl/Kokkos_Profiling.cpp (loading the tool named by
// KOKKOS_TOOLS_LIBS, kokkosp_init_library / kokkosp_finalize_library) and the
// begin/end calls every parallel_for / parallel_reduce / parallel_scan makes
// (core/src/Kokkos_Parallel.hpp:134-160, 351-365;
// core/src/Kokkos_Parallel_Reduce.hpp:1530-1550), with the C signatures of
// core/src/impl/Kokkos_Profiling_C_Interface.h:48-64 and the device-id
// encoding of core/src/impl/Kokkos_Profiling_Interface.hpp:40-100 (8 bits
// device type, 7 bits device, 17 bits instance).
#pragma once

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <stdint.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <typeinfo>

namespace gb300k {
namespace Tools {

struct KokkosPDeviceInfo {
  size_t deviceID;
};

namespace Impl {
using InitFn = void (*)(const int, const uint64_t, const uint32_t, KokkosPDeviceInfo*);
using FinalizeFn = void (*)();
using BeginFn = void (*)(const char*, const uint32_t, uint64_t*);
using EndFn = void (*)(uint64_t);

enum Kind { kFor = 0, kReduce = 1, kScan = 2 };

struct Hooks {
  void* handle = nullptr;
  FinalizeFn finalize = nullptr;
  BeginFn begin[3] = {nullptr, nullptr, nullptr};
  EndFn end[3] = {nullptr, nullptr, nullptr};
};
inline Hooks& hooks() {
  static Hooks h;
  return h;
}

constexpr uint32_t kInterfaceVersion = 20240906;  // KOKKOSP_INTERFACE_VERSION
constexpr uint32_t kDeviceTypeCuda = 2;          // DeviceType::Cuda
constexpr uint32_t kInstanceBits = 17, kDeviceBits = 7;

// The first library of KOKKOS_TOOLS_LIBS (a ';'-separated list) is loaded and
// initialised; a library that cannot be opened is reported and ignored.
inline void load_tool() {
  Hooks& h = hooks();
  if (h.handle) return;
  const char* env = std::getenv("KOKKOS_TOOLS_LIBS");
  if (!env || !*env) return;
  std::string first(env);
  const size_t semi = first.find(';');
  if (semi != std::string::npos) first = first.substr(0, semi);
  void* lib = dlopen(first.c_str(), RTLD_NOW | RTLD_LOCAL);
  if (!lib) {
    std::fprintf(stderr, "KOKKOS_TOOLS_LIBS: dlopen(%s) failed: %s\n", first.c_str(), dlerror());
    return;
  }
  h.handle = lib;
  auto sym = [&](const char* n) { return dlsym(lib, n); };
  h.finalize = reinterpret_cast<FinalizeFn>(sym("kokkosp_finalize_library"));
  h.begin[kFor] = reinterpret_cast<BeginFn>(sym("kokkosp_begin_parallel_for"));
  h.begin[kReduce] = reinterpret_cast<BeginFn>(sym("kokkosp_begin_parallel_reduce"));
  h.begin[kScan] = reinterpret_cast<BeginFn>(sym("kokkosp_begin_parallel_scan"));
  h.end[kFor] = reinterpret_cast<EndFn>(sym("kokkosp_end_parallel_for"));
  h.end[kReduce] = reinterpret_cast<EndFn>(sym("kokkosp_end_parallel_reduce"));
  h.end[kScan] = reinterpret_cast<EndFn>(sym("kokkosp_end_parallel_scan"));
  if (auto init = reinterpret_cast<InitFn>(sym("kokkosp_init_library"))) init(0, kInterfaceVersion, 0, nullptr);
}
inline void unload_tool() {
  Hooks& h = hooks();
  if (!h.handle) return;
  if (h.finalize) h.finalize();
  dlclose(h.handle);
  h = Hooks();
}

// Device id of a space on `stream` (instance 0: the default stream).
inline uint32_t device_id(cudaStream_t stream) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint32_t inst = stream ? (uint32_t)(((uintptr_t)stream >> 4) % ((1u << kInstanceBits) - 1) + 1) : 0u;
  return (kDeviceTypeCuda << (kInstanceBits + kDeviceBits)) | (((uint32_t)dev & ((1u << kDeviceBits) - 1)) << kInstanceBits) |
         inst;
}

// The label of the innermost labelled call on this thread (set by the
// parallel_*(label, ...) overloads), else the functor's type name, as the
// reference names unlabelled kernels.
inline const std::string*& current_label() {
  thread_local const std::string* l = nullptr;
  return l;
}
struct LabelScope {
  const std::string* prev;
  explicit LabelScope(const std::string& l) : prev(current_label()) { current_label() = &l; }
  ~LabelScope() { current_label() = prev; }
};

// begin_parallel_* on construction, end_parallel_* on destruction, when a
// tool with those callbacks is loaded.
template <class F>
struct Region {
  int kind;
  uint64_t id = 0;
  bool on = false;
  Region(int k, cudaStream_t stream) : kind(k) {
    Hooks& h = hooks();
    if (!h.begin[k]) return;
    const std::string* l = current_label();
    h.begin[k](l ? l->c_str() : typeid(F).name(), device_id(stream), &id);
    on = true;
  }
  ~Region() {
    if (on && hooks().end[kind]) hooks().end[kind](id);
  }
  Region(const Region&) = delete;
  Region& operator=(const Region&) = delete;
};
}  // namespace Impl
}  // namespace Tools
}  // namespace gb300k
