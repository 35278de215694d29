// Internal device/host helpers shared by the libgbk translation units.
//
// Layout of the per-stream workspace (device memory owned by the library,
// never by the caller):
//   counters[64]  u32 slots, zero between launches (each kernel that takes a
//                 ticket resets its slot before it exits)
//   err           i32 device error bits (GBK_EBIT_*), read and cleared by
//                 gbk_stream_check
//   scratch       partials, tile status, sort temporaries (grown on demand
//                 outside stream capture)
//   stage         device copy of host inputs for the *_host entry points
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "../../include/gbk.h"

#define GBK_EBIT_TIMEOUT 1
#define GBK_EBIT_KEY_RANGE 2
#define GBK_EBIT_BAD_STATE 4
#define GBK_EBIT_ABORT 8  /* a kernel instantiated outside the library ran a device-side abort */

namespace gbk {

// ---------------------------------------------------------------------------
// host runtime (gbk_runtime.cu)
struct Workspace {
  cudaStream_t stream = nullptr;
  int device = 0;
  unsigned* counters = nullptr;  // 64 slots
  int* err = nullptr;
  char* scratch = nullptr;
  size_t scratch_bytes = 0;
  char* stage = nullptr;
  size_t stage_bytes = 0;
  // Look-back status words, used only by kernels that tag them with `epoch`
  // (bumped per launch), so no other kernel's data can look like a flag.
  char* flags = nullptr;
  size_t flags_bytes = 0;
  uint32_t epoch = 0;
  std::mutex mu;
  // Pinned host slot for fences: [0, 4) the error word's copy, [256, 512) a
  // small result read back with it (one stream synchronisation for both).
  char* host_slot = nullptr;
  std::mutex slot_mu;
};

Workspace* ws_get(cudaStream_t s, int* status);
// Status-word buffer of at least `count` u32 and the next 30-bit epoch.
unsigned* ws_flags(Workspace* w, size_t count, unsigned* epoch, int* status);
// Ensure at least `bytes` of scratch; returns nullptr (and sets status) on
// failure or when growth is needed while the stream is being captured.
char* ws_scratch(Workspace* w, size_t bytes, int* status);
char* ws_stage(Workspace* w, size_t bytes, int* status);
int sm_count();
// Tuning-table configuration for a call made with tune == NULL (nullptr if
// the table is disabled or has no entry).  Kinds: 0 reduce, 1 scan,
// 2 histogram, 3 segmented.
enum { TUNE_REDUCE = 0, TUNE_SCAN = 1, TUNE_HIST = 2, TUNE_SEG = 3 };
const gbk_tuning_t* tuned_config(int kind, int op, int dtype, int64_t n, int extra, gbk_tuning_t* storage);
int64_t wait_limit();
void note_launch(int64_t k = 1);
int cuda_status(cudaError_t e);
// Counter slots
enum { SLOT_REDUCE = 0, SLOT_SCAN_TILE = 1, SLOT_MISC = 2, SLOT_SEG = 3, SLOT_SEGRED = 5, SLOT_SORT = 8 };

// ---------------------------------------------------------------------------
// dtype mapping
template <int DT> struct dtype_of;
template <> struct dtype_of<GBK_I32> { using type = int32_t; };
template <> struct dtype_of<GBK_I64> { using type = int64_t; };
template <> struct dtype_of<GBK_U32> { using type = uint32_t; };
template <> struct dtype_of<GBK_U64> { using type = uint64_t; };
template <> struct dtype_of<GBK_F32> { using type = float; };
template <> struct dtype_of<GBK_F64> { using type = double; };

inline size_t dtype_size(int dt) { return (dt == GBK_I32 || dt == GBK_U32 || dt == GBK_F32) ? 4 : 8; }

// ---------------------------------------------------------------------------
// identities (core/src/Kokkos_ReductionIdentity.hpp)
template <class T> struct lim;
template <> struct lim<int32_t> { __host__ __device__ static constexpr int32_t hi() { return 2147483647; } __host__ __device__ static constexpr int32_t lo() { return -2147483647 - 1; } };
template <> struct lim<uint32_t> { __host__ __device__ static constexpr uint32_t hi() { return 0xFFFFFFFFu; } __host__ __device__ static constexpr uint32_t lo() { return 0u; } };
template <> struct lim<int64_t> { __host__ __device__ static constexpr int64_t hi() { return 9223372036854775807LL; } __host__ __device__ static constexpr int64_t lo() { return -9223372036854775807LL - 1; } };
template <> struct lim<uint64_t> { __host__ __device__ static constexpr uint64_t hi() { return 0xFFFFFFFFFFFFFFFFull; } __host__ __device__ static constexpr uint64_t lo() { return 0ull; } };
template <> struct lim<float> { __host__ __device__ static constexpr float hi() { return 3.402823466e+38F; } __host__ __device__ static constexpr float lo() { return -3.402823466e+38F; } };
template <> struct lim<double> { __host__ __device__ static constexpr double hi() { return 1.7976931348623158e+308; } __host__ __device__ static constexpr double lo() { return -1.7976931348623158e+308; } };

constexpr int64_t LOC_ID = 9223372036854775807LL;

template <class T> struct ValLoc { T val; int64_t loc; };
template <class T> struct MinMaxV { T min_val, max_val; };
template <class T> struct MinMaxLocV { T min_val, max_val; int64_t min_loc, max_loc; };
template <class T> struct MinMaxLocSumV { T min_val, max_val; int64_t min_loc, max_loc; T sum; };

// ---------------------------------------------------------------------------
// warp shuffles of the value types
template <class T> __device__ __forceinline__ T shx(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
template <class T> __device__ __forceinline__ ValLoc<T> shx(ValLoc<T> v, int m) {
  v.val = shx(v.val, m); v.loc = shx(v.loc, m); return v;
}
template <class T> __device__ __forceinline__ MinMaxV<T> shx(MinMaxV<T> v, int m) {
  v.min_val = shx(v.min_val, m); v.max_val = shx(v.max_val, m); return v;
}
template <class T> __device__ __forceinline__ MinMaxLocV<T> shx(MinMaxLocV<T> v, int m) {
  v.min_val = shx(v.min_val, m); v.max_val = shx(v.max_val, m);
  v.min_loc = shx(v.min_loc, m); v.max_loc = shx(v.max_loc, m); return v;
}
template <class T> __device__ __forceinline__ MinMaxLocSumV<T> shx(MinMaxLocSumV<T> v, int m) {
  v.min_val = shx(v.min_val, m); v.max_val = shx(v.max_val, m);
  v.min_loc = shx(v.min_loc, m); v.max_loc = shx(v.max_loc, m); v.sum = shx(v.sum, m); return v;
}

// ---------------------------------------------------------------------------
// Reducers.  update(v, x, loc) is the element functor of the typed entry
// (v op= x); join(a, b) combines partial results.  ORDERED visits: a thread
// sees its elements in increasing loc, so *Loc updates use a strict compare
// (first occurrence wins, as the reference functor); unordered visits use
// the (value, loc) order.
template <class T> struct RSum {
  using V = T;
  __device__ static V init() { return T(0); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v += x; }
  __device__ static void join(V& a, const V& b) { a += b; }
};
template <class T> struct RProd {
  using V = T;
  __device__ static V init() { return T(1); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v *= x; }
  __device__ static void join(V& a, const V& b) { a *= b; }
};
template <class T> struct RMin {
  using V = T;
  __device__ static V init() { return lim<T>::hi(); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v = (x < v) ? x : v; }
  __device__ static void join(V& a, const V& b) { a = (b < a) ? b : a; }
};
template <class T> struct RMax {
  using V = T;
  __device__ static V init() { return lim<T>::lo(); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v = (x > v) ? x : v; }
  __device__ static void join(V& a, const V& b) { a = (b > a) ? b : a; }
};
template <class T> struct RLAnd {
  using V = T;
  __device__ static V init() { return T(1); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v = (v && x) ? T(1) : T(0); }
  __device__ static void join(V& a, const V& b) { a = (a && b) ? T(1) : T(0); }
};
template <class T> struct RLOr {
  using V = T;
  __device__ static V init() { return T(0); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v = (v || x) ? T(1) : T(0); }
  __device__ static void join(V& a, const V& b) { a = (a || b) ? T(1) : T(0); }
};
template <class T> struct RBAnd {
  using V = T;
  __device__ static V init() { return T(~T(0)); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v &= x; }
  __device__ static void join(V& a, const V& b) { a &= b; }
};
template <class T> struct RBOr {
  using V = T;
  __device__ static V init() { return T(0); }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) { v |= x; }
  __device__ static void join(V& a, const V& b) { a |= b; }
};
template <class T> struct RMinLoc {
  using V = ValLoc<T>;
  __device__ static V init() { return V{lim<T>::hi(), LOC_ID}; }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t l) {
    if (ORD) {
      if (x < v.val) { v.val = x; v.loc = l; }
    } else {
      if (x < v.val || (x == v.val && v.loc != LOC_ID && l < v.loc)) { v.val = x; v.loc = l; }
    }
  }
  __device__ static void join(V& a, const V& b) {
    if (b.val < a.val || (b.val == a.val && b.loc < a.loc)) a = b;
  }
};
template <class T> struct RMaxLoc {
  using V = ValLoc<T>;
  __device__ static V init() { return V{lim<T>::lo(), LOC_ID}; }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t l) {
    if (ORD) {
      if (x > v.val) { v.val = x; v.loc = l; }
    } else {
      if (x > v.val || (x == v.val && v.loc != LOC_ID && l < v.loc)) { v.val = x; v.loc = l; }
    }
  }
  __device__ static void join(V& a, const V& b) {
    if (b.val > a.val || (b.val == a.val && b.loc < a.loc)) a = b;
  }
};
template <class T> struct RMinMax {
  using V = MinMaxV<T>;
  __device__ static V init() { return V{lim<T>::hi(), lim<T>::lo()}; }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t) {
    v.min_val = (x < v.min_val) ? x : v.min_val;
    v.max_val = (x > v.max_val) ? x : v.max_val;
  }
  __device__ static void join(V& a, const V& b) {
    a.min_val = (b.min_val < a.min_val) ? b.min_val : a.min_val;
    a.max_val = (b.max_val > a.max_val) ? b.max_val : a.max_val;
  }
};
template <class T> struct RMinMaxLoc {
  using V = MinMaxLocV<T>;
  __device__ static V init() { return V{lim<T>::hi(), lim<T>::lo(), LOC_ID, LOC_ID}; }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t l) {
    if (ORD) {
      if (x < v.min_val) { v.min_val = x; v.min_loc = l; }
      if (x > v.max_val) { v.max_val = x; v.max_loc = l; }
    } else {
      if (x < v.min_val || (x == v.min_val && v.min_loc != LOC_ID && l < v.min_loc)) { v.min_val = x; v.min_loc = l; }
      if (x > v.max_val || (x == v.max_val && v.max_loc != LOC_ID && l < v.max_loc)) { v.max_val = x; v.max_loc = l; }
    }
  }
  __device__ static void join(V& a, const V& b) {
    if (b.min_val < a.min_val || (b.min_val == a.min_val && b.min_loc < a.min_loc)) { a.min_val = b.min_val; a.min_loc = b.min_loc; }
    if (b.max_val > a.max_val || (b.max_val == a.max_val && b.max_loc < a.max_loc)) { a.max_val = b.max_val; a.max_loc = b.max_loc; }
  }
};
// MinMaxLoc and Sum of the same elements in one pass (two reducers of one
// parallel_reduce); each half behaves exactly as its own reducer.
template <class T> struct RMinMaxLocSum {
  using V = MinMaxLocSumV<T>;
  __device__ static V init() { return V{lim<T>::hi(), lim<T>::lo(), LOC_ID, LOC_ID, T(0)}; }
  template <bool ORD> __device__ static void update(V& v, T x, int64_t l) {
    MinMaxLocV<T> m{v.min_val, v.max_val, v.min_loc, v.max_loc};
    RMinMaxLoc<T>::template update<ORD>(m, x, l);
    v.min_val = m.min_val; v.max_val = m.max_val; v.min_loc = m.min_loc; v.max_loc = m.max_loc;
    v.sum += x;
  }
  __device__ static void join(V& a, const V& b) {
    MinMaxLocV<T> m{a.min_val, a.max_val, a.min_loc, a.max_loc};
    RMinMaxLoc<T>::join(m, MinMaxLocV<T>{b.min_val, b.max_val, b.min_loc, b.max_loc});
    a.min_val = m.min_val; a.max_val = m.max_val; a.min_loc = m.min_loc; a.max_loc = m.max_loc;
    a.sum += b.sum;
  }
};

// Ordered update by one 16-byte vector of consecutive elements at locs l0,
// l0 + 1, ...: the same result as update<true> element by element.  The
// *Loc reducers fold the vector to its extremum first (fminf / fmaxf skip a
// NaN, as the strict comparisons of update<true> do) and touch (val, loc)
// only when that beats the running value, taking the first element equal to
// it (the first occurrence, as the element-wise strict update keeps; -0.0
// and +0.0 compare equal there too).  A running extremum changes rarely, so
// the common cost is VEC - 1 min/max operations and one comparison.
__device__ __forceinline__ float ext_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double ext_min(double a, double b) { return fmin(a, b); }
template <class T> __device__ __forceinline__ T ext_min(T a, T b) { return b < a ? b : a; }
__device__ __forceinline__ float ext_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double ext_max(double a, double b) { return fmax(a, b); }
template <class T> __device__ __forceinline__ T ext_max(T a, T b) { return b > a ? b : a; }

template <class T, int VEC, bool MIN>
__device__ __forceinline__ void vec_extreme(const T* v, T& e) {
  e = v[0];
#pragma unroll
  for (int q = 1; q < VEC; ++q) e = MIN ? ext_min(e, v[q]) : ext_max(e, v[q]);
}
// First q with v[q] == e (e is one of the v[q]), with that element.
template <class T, int VEC>
__device__ __forceinline__ void vec_first_equal(const T* v, T e, T& val, int& q) {
  val = v[VEC - 1];
  q = VEC - 1;
#pragma unroll
  for (int k = VEC - 2; k >= 0; --k)
    if (v[k] == e) { val = v[k]; q = k; }
}

template <class R, class T, int VEC> struct VecUpd {
  __device__ static void run(typename R::V& acc, const T* v, int64_t l0) {
#pragma unroll
    for (int q = 0; q < VEC; ++q) R::template update<true>(acc, v[q], l0 + q);
  }
};
template <class T, int VEC> struct VecUpd<RMinLoc<T>, T, VEC> {
  __device__ static void run(ValLoc<T>& acc, const T* v, int64_t l0) {
    T e;
    vec_extreme<T, VEC, true>(v, e);
    if (e < acc.val) {
      int q;
      vec_first_equal<T, VEC>(v, e, acc.val, q);
      acc.loc = l0 + q;
    }
  }
};
template <class T, int VEC> struct VecUpd<RMaxLoc<T>, T, VEC> {
  __device__ static void run(ValLoc<T>& acc, const T* v, int64_t l0) {
    T e;
    vec_extreme<T, VEC, false>(v, e);
    if (e > acc.val) {
      int q;
      vec_first_equal<T, VEC>(v, e, acc.val, q);
      acc.loc = l0 + q;
    }
  }
};
template <class T, int VEC> struct VecUpd<RMinMaxLoc<T>, T, VEC> {
  __device__ static void run(MinMaxLocV<T>& acc, const T* v, int64_t l0) {
    T lo, hi;
    vec_extreme<T, VEC, true>(v, lo);
    vec_extreme<T, VEC, false>(v, hi);
    if (lo < acc.min_val) {
      int q;
      vec_first_equal<T, VEC>(v, lo, acc.min_val, q);
      acc.min_loc = l0 + q;
    }
    if (hi > acc.max_val) {
      int q;
      vec_first_equal<T, VEC>(v, hi, acc.max_val, q);
      acc.max_loc = l0 + q;
    }
  }
};

template <class T, int VEC> struct VecUpd<RMinMaxLocSum<T>, T, VEC> {
  __device__ static void run(MinMaxLocSumV<T>& acc, const T* v, int64_t l0) {
    MinMaxLocV<T> m{acc.min_val, acc.max_val, acc.min_loc, acc.max_loc};
    VecUpd<RMinMaxLoc<T>, T, VEC>::run(m, v, l0);
    acc.min_val = m.min_val; acc.max_val = m.max_val; acc.min_loc = m.min_loc; acc.max_loc = m.max_loc;
#pragma unroll
    for (int q = 0; q < VEC; ++q) acc.sum += v[q];
  }
};

// Warp tree.  32-bit integer Sum/Min/Max/BAnd/BOr use redux.sync (one
// instruction); everything else a butterfly of shuffles.
template <class R> struct WarpRed {
  __device__ static typename R::V run(typename R::V v) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      typename R::V o = shx(v, m);
      R::join(v, o);
    }
    return v;
  }
};
template <> struct WarpRed<RSum<int32_t>> { __device__ static int32_t run(int32_t v) { return (int32_t)__reduce_add_sync(0xffffffffu, (unsigned)v); } };
template <> struct WarpRed<RSum<uint32_t>> { __device__ static uint32_t run(uint32_t v) { return __reduce_add_sync(0xffffffffu, v); } };
template <> struct WarpRed<RMin<int32_t>> { __device__ static int32_t run(int32_t v) { return __reduce_min_sync(0xffffffffu, v); } };
template <> struct WarpRed<RMin<uint32_t>> { __device__ static uint32_t run(uint32_t v) { return __reduce_min_sync(0xffffffffu, v); } };
template <> struct WarpRed<RMax<int32_t>> { __device__ static int32_t run(int32_t v) { return __reduce_max_sync(0xffffffffu, v); } };
template <> struct WarpRed<RMax<uint32_t>> { __device__ static uint32_t run(uint32_t v) { return __reduce_max_sync(0xffffffffu, v); } };
template <> struct WarpRed<RBAnd<int32_t>> { __device__ static int32_t run(int32_t v) { return (int32_t)__reduce_and_sync(0xffffffffu, (unsigned)v); } };
template <> struct WarpRed<RBAnd<uint32_t>> { __device__ static uint32_t run(uint32_t v) { return __reduce_and_sync(0xffffffffu, v); } };
template <> struct WarpRed<RBOr<int32_t>> { __device__ static int32_t run(int32_t v) { return (int32_t)__reduce_or_sync(0xffffffffu, (unsigned)v); } };
template <> struct WarpRed<RBOr<uint32_t>> { __device__ static uint32_t run(uint32_t v) { return __reduce_or_sync(0xffffffffu, v); } };

// Block tree: result valid in thread 0.  `sm` holds BLOCK/32 values.
template <class R, int BLOCK>
__device__ __forceinline__ typename R::V block_reduce(typename R::V v, typename R::V* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = WarpRed<R>::run(v);
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < BLOCK / 32) ? sm[lane] : R::init();
    v = WarpRed<R>::run(v);
  }
  return v;
}

// ---------------------------------------------------------------------------
// 16-byte streaming load through the non-coherent path without L1
// allocation, with a 256-byte L2 prefetch hint.  Only for data that no
// thread writes during the kernel.
__device__ __forceinline__ uint4 ld_stream16(const void* p) {
  uint4 r;
  asm("ld.global.nc.L1::no_allocate.L2::256B.v4.u32 {%0,%1,%2,%3}, [%4];"
      : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
      : "l"(p));
  return r;
}

template <class T>
union Vec16 {
  uint4 u;
  T v[16 / sizeof(T)];
};

// Release store / acquire load at GPU scope (tile status words).
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ---------------------------------------------------------------------------
// mbarrier + 1-D bulk copy (TMA engine, no tensor map).  The bulk copy wants
// 16-byte aligned source and destination and a size that is a multiple of 16.
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) accesses of the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(b))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Named CTA barriers (ids 1..15; 0 is __syncthreads).  `count` is the
// number of threads taking part, a multiple of 32; bar_arrive does not wait.
__device__ __forceinline__ void bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// Shared -> global bulk copy, tracked by this thread's bulk async-groups.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until the committed stores have read their shared-memory source.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Wait until the committed stores are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Bounded wait for the phase with the given parity; false when it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity, int64_t limit) {
  for (int64_t i = 0; i <= limit; ++i)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}

// Programmatic dependent launch.  A kernel launched with launch_pdl may start
// while the previous kernel of its stream is still finishing: it lets the
// next kernel be scheduled at once (pdl_release), then waits for its
// predecessor's completion and memory (pdl_acquire) before its first global
// memory access, so stream order holds for every buffer it touches.  What it
// gains is the launch and CTA ramp of back-to-back kernels.
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_acquire() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_entry() {
  pdl_release();
  pdl_acquire();
}

// PDL is on unless the environment sets GBK_PDL=0.
bool pdl_enabled();

template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kfn)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kfn, static_cast<Args&&>(args)...);
}

}  // namespace gbk

#define GBK_CUDA_TRY(expr)                      \
  do {                                          \
    cudaError_t e_ = (expr);                    \
    if (e_ != cudaSuccess) return gbk::cuda_status(e_); \
  } while (0)
