// ORACLE — test infrastructure only.
//
// CPU restatement of the reference Kokkos OpenMP backend's reduce / scan /
// ScatterView / sort algorithms, used as the parity checker for the GB300
// kernels and as the timed CPU baseline.  Only the tests, the smoke check
// and the bench's CPU-baseline leg load this library; the product path never
// does.
//
// Parity is pinned: tests/golden/ holds vectors produced by the reference
// itself (built from its own sources by oracle/ref.mk, driven by
// oracle/ref_runner.cpp), and tests/test_oracle_golden.py checks this file
// against them bit for bit.
//
// Codes shared with include/gbk.h:
//   dtype : 0 i32, 1 i64, 2 u32, 3 u64, 4 f32, 5 f64
//   op    : 0 Sum, 1 Prod, 2 Min, 3 Max, 4 LAnd, 5 LOr, 6 BAnd, 7 BOr,
//           8 MinLoc, 9 MaxLoc, 10 MinMax, 11 MinMaxLoc
// Result layouts follow core/src/Kokkos_Parallel_Reduce.hpp:
//   ValLocScalar {T val; int64 loc}            (:406-410)
//   MinMaxScalar {T min_val, max_val}           (:532-535)
//   MinMaxLocScalar {T min_val, max_val; int64 min_loc, max_loc} (:596-600)

#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <type_traits>
#include <utility>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Reduction identities: core/src/Kokkos_ReductionIdentity.hpp:30-398.
// Min identity is the type's maximum (FLT_MAX / DBL_MAX for floating point,
// not +inf), Max identity is the lowest value (-FLT_MAX / -DBL_MAX).
template <class T>
struct ident {
  static T sum() { return T(0); }
  static T prod() { return T(1); }
  static T min() {
    if constexpr (std::is_floating_point_v<T>) return std::numeric_limits<T>::max();
    else return std::numeric_limits<T>::max();
  }
  static T max() {
    if constexpr (std::is_floating_point_v<T>) return -std::numeric_limits<T>::max();
    else return std::numeric_limits<T>::min();
  }
  static T land() { return T(1); }
  static T lor() { return T(0); }
  static T band() { return T(~T(0)); }
  static T bor() { return T(0); }
};
constexpr int64_t LOC_IDENT = std::numeric_limits<int64_t>::max();  // reduction_identity<int64>::min()

template <class T> struct ValLoc { T val; int64_t loc; };
template <class T> struct MinMaxV { T min_val, max_val; };
template <class T> struct MinMaxLocV { T min_val, max_val; int64_t min_loc, max_loc; };

// ---------------------------------------------------------------------------
// Reducers as (init, functor-update, join), restating the built-in reducers
// (core/src/Kokkos_Parallel_Reduce.hpp: Sum :34, Prod :79, Min :124, Max :171,
// LAnd :219, LOr :265, BAnd :312, BOr :359, MinLoc :412, MaxLoc :472,
// MinMax :537, MinMaxLoc :601) together with the element functor a user
// writes for them (update op= x(i); MinLoc: if (x(i) < v.val) {v.val =
// x(i); v.loc = i;}).
template <class T> struct RSum {
  using V = T;
  static V init() { return ident<T>::sum(); }
  static void update(V& v, T x, int64_t) { v += x; }
  static void join(V& d, const V& s) { d += s; }
};
template <class T> struct RProd {
  using V = T;
  static V init() { return ident<T>::prod(); }
  static void update(V& v, T x, int64_t) { v *= x; }
  static void join(V& d, const V& s) { d *= s; }
};
template <class T> struct RMin {
  using V = T;
  static V init() { return ident<T>::min(); }
  static void update(V& v, T x, int64_t) { if (x < v) v = x; }
  static void join(V& d, const V& s) { if (s < d) d = s; }
};
template <class T> struct RMax {
  using V = T;
  static V init() { return ident<T>::max(); }
  static void update(V& v, T x, int64_t) { if (x > v) v = x; }
  static void join(V& d, const V& s) { if (s > d) d = s; }
};
template <class T> struct RLAnd {
  using V = T;
  static V init() { return ident<T>::land(); }
  static void update(V& v, T x, int64_t) { v = (v && x); }
  static void join(V& d, const V& s) { d = (d && s); }
};
template <class T> struct RLOr {
  using V = T;
  static V init() { return ident<T>::lor(); }
  static void update(V& v, T x, int64_t) { v = (v || x); }
  static void join(V& d, const V& s) { d = (d || s); }
};
template <class T> struct RBAnd {
  using V = T;
  static V init() { return ident<T>::band(); }
  static void update(V& v, T x, int64_t) { v = v & x; }
  static void join(V& d, const V& s) { d = d & s; }
};
template <class T> struct RBOr {
  using V = T;
  static V init() { return ident<T>::bor(); }
  static void update(V& v, T x, int64_t) { v = v | x; }
  static void join(V& d, const V& s) { d = d | s; }
};
// MinLoc/MaxLoc join (Kokkos_Parallel_Reduce.hpp:440-447, :500-507): keep
// dest unless src is strictly better, or equal while dest.loc is still the
// identity.
template <class T> struct RMinLoc {
  using V = ValLoc<T>;
  static V init() { return V{ident<T>::min(), LOC_IDENT}; }
  static void update(V& v, T x, int64_t i) { if (x < v.val) { v.val = x; v.loc = i; } }
  static void join(V& d, const V& s) {
    if (s.val < d.val) d = s;
    else if (s.val == d.val && d.loc == LOC_IDENT) d.loc = s.loc;
  }
};
template <class T> struct RMaxLoc {
  using V = ValLoc<T>;
  static V init() { return V{ident<T>::max(), LOC_IDENT}; }
  static void update(V& v, T x, int64_t i) { if (x > v.val) { v.val = x; v.loc = i; } }
  static void join(V& d, const V& s) {
    if (s.val > d.val) d = s;
    else if (s.val == d.val && d.loc == LOC_IDENT) d.loc = s.loc;
  }
};
// MinMax join: Kokkos_Parallel_Reduce.hpp:560-567.
template <class T> struct RMinMax {
  using V = MinMaxV<T>;
  static V init() { return V{ident<T>::min(), ident<T>::max()}; }
  static void update(V& v, T x, int64_t) { if (x < v.min_val) v.min_val = x; if (x > v.max_val) v.max_val = x; }
  static void join(V& d, const V& s) {
    if (s.min_val < d.min_val) d.min_val = s.min_val;
    if (s.max_val > d.max_val) d.max_val = s.max_val;
  }
};
// MinMaxLoc join: Kokkos_Parallel_Reduce.hpp:626-641.
template <class T> struct RMinMaxLoc {
  using V = MinMaxLocV<T>;
  static V init() { return V{ident<T>::min(), ident<T>::max(), LOC_IDENT, LOC_IDENT}; }
  static void update(V& v, T x, int64_t i) {
    if (x < v.min_val) { v.min_val = x; v.min_loc = i; }
    if (x > v.max_val) { v.max_val = x; v.max_loc = i; }
  }
  static void join(V& d, const V& s) {
    if (s.min_val < d.min_val) { d.min_val = s.min_val; d.min_loc = s.min_loc; }
    else if (s.min_val == d.min_val && d.min_loc == LOC_IDENT) d.min_loc = s.min_loc;
    if (s.max_val > d.max_val) { d.max_val = s.max_val; d.max_loc = s.max_loc; }
    else if (s.max_val == d.max_val && d.max_loc == LOC_IDENT) d.max_loc = s.max_loc;
  }
};

// ---------------------------------------------------------------------------
// RangePolicy automatic chunk size: core/src/Kokkos_ExecPolicy.hpp:202-232.
int64_t auto_chunk(int64_t n, int64_t concurrency) {
  if (concurrency == 0) concurrency = 1;
  int64_t c = 1;
  while (c * 100 * concurrency < n) c *= 2;
  if (c < 128) {
    c = 1;
    while (c * 40 * concurrency < n && c < 128) c *= 2;
  }
  return c;
}

// HostThreadTeamData::set_work_partition / get_work_partition:
// core/src/impl/Kokkos_HostThreadTeam.hpp:357-390.  Thread r of P gets
// [part*r*chunk, min(part*(r+1)*chunk, n)).
std::pair<int64_t, int64_t> work_partition(int64_t n, int64_t chunk, int r, int P) {
  const int64_t int_max = std::numeric_limits<int>::max();
  const int64_t chunk_min = (n + int_max) / int_max;
  const int64_t ch = std::max(chunk, chunk_min);
  const int64_t num = (n + ch - 1) / ch;
  const int64_t part = (num + P - 1) / P;
  const int64_t first = part * r * ch;
  const int64_t second = std::min(part * (r + 1) * ch, n);
  return {first, second};
}

// OpenMP ParallelReduce<RangePolicy>::execute:
// core/src/OpenMP/Kokkos_OpenMP_Parallel_Reduce.hpp:69-162.  Each thread
// runs the functor sequentially over its partition into its own value,
// initialised by the reducer; thread 0's value then joins threads 1..P-1 in
// thread order.  With P == 1 the serial path (:98-112) is the same loop.
template <class R, class T>
typename R::V reduce_range(const T* x, int64_t n, int P) {
  using V = typename R::V;
  if (n <= 0) return R::init();
  if (P < 1) P = 1;
  const int64_t chunk = auto_chunk(n, P);
  std::vector<V> part(P, R::init());
#pragma omp parallel num_threads(P)
  {
    const int r = omp_get_thread_num();
    const int np = omp_get_num_threads();
    // When the runtime gives fewer threads than asked, each thread walks
    // the partitions it stands in for, so the result stays that of P.
    for (int q = r; q < P; q += np) {
      auto rg = work_partition(n, chunk, q, P);
      V v = R::init();
      for (int64_t i = rg.first; i < rg.second; ++i) R::update(v, x[i], i);
      part[q] = v;
    }
  }
  V acc = part[0];
  for (int i = 1; i < P; ++i) R::join(acc, part[i]);
  return acc;
}

template <class T>
int reduce_dispatch_T(int op, const T* x, int64_t n, int P, void* out) {
  switch (op) {
    case 0: *(T*)out = reduce_range<RSum<T>>(x, n, P); return 0;
    case 1: *(T*)out = reduce_range<RProd<T>>(x, n, P); return 0;
    case 2: *(T*)out = reduce_range<RMin<T>>(x, n, P); return 0;
    case 3: *(T*)out = reduce_range<RMax<T>>(x, n, P); return 0;
    case 4:  // LAnd / LOr / BAnd / BOr have identities for integers only
      if constexpr (std::is_integral_v<T>) { *(T*)out = reduce_range<RLAnd<T>>(x, n, P); return 0; }
      return 1;
    case 5:
      if constexpr (std::is_integral_v<T>) { *(T*)out = reduce_range<RLOr<T>>(x, n, P); return 0; }
      return 1;
    case 6:
      if constexpr (std::is_integral_v<T>) { *(T*)out = reduce_range<RBAnd<T>>(x, n, P); return 0; }
      return 1;
    case 7:
      if constexpr (std::is_integral_v<T>) { *(T*)out = reduce_range<RBOr<T>>(x, n, P); return 0; }
      return 1;
    case 8: *(ValLoc<T>*)out = reduce_range<RMinLoc<T>>(x, n, P); return 0;
    case 9: *(ValLoc<T>*)out = reduce_range<RMaxLoc<T>>(x, n, P); return 0;
    case 10: *(MinMaxV<T>*)out = reduce_range<RMinMax<T>>(x, n, P); return 0;
    case 11: *(MinMaxLocV<T>*)out = reduce_range<RMinMaxLoc<T>>(x, n, P); return 0;
  }
  return 1;
}

// Neumaier's compensated summation (Neumaier 1974), in FP64.
template <class T>
void neumaier(const T* x, int64_t n, double* sum_out, double* abs_out, double* sq_out) {
  double s = 0.0, c = 0.0, a = 0.0, q = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double v = (double)x[i];
    const double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
    a += std::fabs(v);
    q += v * v;
  }
  if (sum_out) *sum_out = s + c;
  if (abs_out) *abs_out = a;
  if (sq_out) *sq_out = q;
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

int orc_max_threads(void) { return omp_get_max_threads(); }

// parallel_reduce(RangePolicy<OpenMP>(0,n), functor, Reducer(result)) with
// the pool size P; see reduce_range above.
int orc_reduce(int op, int dtype, const void* x, int64_t n, int nthreads, void* out) {
  switch (dtype) {
    case 0: return reduce_dispatch_T<int32_t>(op, (const int32_t*)x, n, nthreads, out);
    case 1: return reduce_dispatch_T<int64_t>(op, (const int64_t*)x, n, nthreads, out);
    case 2: return reduce_dispatch_T<uint32_t>(op, (const uint32_t*)x, n, nthreads, out);
    case 3: return reduce_dispatch_T<uint64_t>(op, (const uint64_t*)x, n, nthreads, out);
    case 4: return reduce_dispatch_T<float>(op, (const float*)x, n, nthreads, out);
    case 5: return reduce_dispatch_T<double>(op, (const double*)x, n, nthreads, out);
  }
  return 1;
}

// Compensated FP64 sums: the tolerance oracle for floating-point Sum.
// Writes {sum, sum|x|, sum x^2}.
int orc_sum_compensated(int dtype, const void* x, int64_t n, double* out3) {
  if (dtype == 4) neumaier((const float*)x, n, out3, out3 + 1, out3 + 2);
  else if (dtype == 5) neumaier((const double*)x, n, out3, out3 + 1, out3 + 2);
  else return 1;
  return 0;
}

}  // extern "C"

// MDRange reduce over an iteration box [lower, upper) of a strided view
// (strides in elements).  Element "loc" is the element's offset from base:
// sum_d i_d * stride_d.  Restates OpenMP ParallelReduce<MDRangePolicy>
// (core/src/OpenMP/Kokkos_OpenMP_Parallel_Reduce.hpp:187-326) with the
// host tile rules of MDRangePolicy::init_helper
// (core/src/KokkosExp_MDRangePolicy.hpp:388-425; host TileSizeProperties
// :145-152: default tile 2, the innermost dimension's tile = its whole
// length), the tile partition set_work_partition(num_tiles, 1) over the
// thread pool, and HostIterateTile's walk
// (core/src/impl/KokkosExp_Host_IterateTile.hpp:2040-2110: tile offsets in
// outer-direction order, partial tiles by check_iteration_bounds, elements in
// inner-direction order), then the thread-order join.  So the result equals
// the reference's bit for bit, floating-point Sums included.
// iter_outer / iter_inner: 0 = Right (last index fastest, the host default),
// 1 = Left.  tile: rank entries, <= 0 = the default for that dimension.
template <class R, class T>
static typename R::V mdrange_tiles(const T* base, int rank, const int64_t* lower, const int64_t* upper,
                                   const int64_t* strides, const int64_t* tile_in, int outer_left,
                                   int inner_left, int P) {
  using V = typename R::V;
  int64_t tile[6], tend[6], num_tiles = 1, prod = 1;
  const int64_t int_max = std::numeric_limits<int>::max();
  const int first = inner_left ? 0 : rank - 1, last = inner_left ? rank : -1, inc = inner_left ? 1 : -1;
  for (int i = first; i != last; i += inc) {
    const int64_t len = upper[i] - lower[i];
    tile[i] = tile_in ? tile_in[i] : 0;
    if (tile[i] <= 0) {
      const bool innermost = inner_left ? (i == 0) : (i == rank - 1);
      if (!innermost) tile[i] = (prod * 2 < int_max) ? 2 : 1;
      else tile[i] = std::max<int64_t>(len, 1);
    }
    tend[i] = (len + tile[i] - 1) / tile[i];
    num_tiles *= tend[i];
    prod *= tile[i];
  }
  if (P < 1) P = 1;
  std::vector<V> part(P, R::init());
  auto run_tiles = [&](int64_t tb, int64_t te, V& v) {
    int64_t off[6], dims[6];
    for (int64_t t = tb; t < te; ++t) {
      int64_t ti = t;
      if (outer_left) {
        for (int i = 0; i < rank; ++i) { off[i] = (ti % tend[i]) * tile[i] + lower[i]; ti /= tend[i]; }
      } else {
        for (int i = rank - 1; i >= 0; --i) { off[i] = (ti % tend[i]) * tile[i] + lower[i]; ti /= tend[i]; }
      }
      for (int i = 0; i < rank; ++i) {
        if (off[i] + tile[i] <= upper[i]) dims[i] = tile[i];
        else dims[i] = (upper[i] - 1 - off[i]) == 0 ? 1
                       : (upper[i] - tile[i]) > 0 ? (upper[i] - off[i]) : (upper[i] - lower[i]);
      }
      // Elements of the tile: the innermost loop runs over dimension
      // rank-1 (Right) or 0 (Left); the counter idx walks the others as an
      // odometer in the same nesting order.
      const int in_d = inner_left ? 0 : rank - 1;
      int64_t idx[6] = {0, 0, 0, 0, 0, 0};
      int64_t outer_cnt = 1;
      for (int i = 0; i < rank; ++i) if (i != in_d) outer_cnt *= dims[i];
      for (int64_t c = 0; c < outer_cnt; ++c) {
        int64_t o = 0;
        for (int i = 0; i < rank; ++i) if (i != in_d) o += (off[i] + idx[i]) * strides[i];
        const int64_t s = strides[in_d];
        int64_t e = o + off[in_d] * s;
        for (int64_t k = 0; k < dims[in_d]; ++k, e += s) R::update(v, base[e], e);
        // advance the odometer: innermost of the remaining dimensions first
        if (inner_left) {
          for (int i = 1; i < rank; ++i) { if (++idx[i] < dims[i]) break; idx[i] = 0; }
        } else {
          for (int i = rank - 2; i >= 0; --i) { if (++idx[i] < dims[i]) break; idx[i] = 0; }
        }
      }
    }
  };
#pragma omp parallel num_threads(P)
  {
    const int r = omp_get_thread_num();
    const int np = omp_get_num_threads();
    for (int q = r; q < P; q += np) {
      auto rg = work_partition(num_tiles, 1, q, P);
      V v = R::init();
      run_tiles(rg.first, rg.second, v);
      part[q] = v;
    }
  }
  V acc = part[0];
  for (int i = 1; i < P; ++i) R::join(acc, part[i]);
  return acc;
}

template <class T>
static int mdrange_dispatch_T(int op, const T* b, int rank, const int64_t* lo, const int64_t* up,
                              const int64_t* st, const int64_t* tile, int ol, int il, int P, void* out) {
  switch (op) {
    case 0: *(T*)out = mdrange_tiles<RSum<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 1: *(T*)out = mdrange_tiles<RProd<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 2: *(T*)out = mdrange_tiles<RMin<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 3: *(T*)out = mdrange_tiles<RMax<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 4:
      if constexpr (std::is_integral_v<T>) { *(T*)out = mdrange_tiles<RLAnd<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0; }
      return 1;
    case 5:
      if constexpr (std::is_integral_v<T>) { *(T*)out = mdrange_tiles<RLOr<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0; }
      return 1;
    case 6:
      if constexpr (std::is_integral_v<T>) { *(T*)out = mdrange_tiles<RBAnd<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0; }
      return 1;
    case 7:
      if constexpr (std::is_integral_v<T>) { *(T*)out = mdrange_tiles<RBOr<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0; }
      return 1;
    case 8: *(ValLoc<T>*)out = mdrange_tiles<RMinLoc<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 9: *(ValLoc<T>*)out = mdrange_tiles<RMaxLoc<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 10: *(MinMaxV<T>*)out = mdrange_tiles<RMinMax<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
    case 11: *(MinMaxLocV<T>*)out = mdrange_tiles<RMinMaxLoc<T>>(b, rank, lo, up, st, tile, ol, il, P); return 0;
  }
  return 1;
}

extern "C" {

// The tile walk above with explicit tiles and iteration directions
// (MDRangePolicy<Rank<N, outer, inner>>(lower, upper, tile)).
int orc_mdrange_reduce_ex(int op, int dtype, const void* base, int rank, const int64_t* lower,
                          const int64_t* upper, const int64_t* strides, const int64_t* tile, int outer_left,
                          int inner_left, int nthreads, void* out) {
  if (rank < 1 || rank > 6) return 1;
  for (int d = 0; d < rank; ++d)
    if (upper[d] < lower[d]) return 1;  // the reference aborts (KokkosExp_MDRangePolicy.hpp:399-411)
  switch (dtype) {
    case 0: return mdrange_dispatch_T<int32_t>(op, (const int32_t*)base, rank, lower, upper, strides, tile, outer_left, inner_left, nthreads, out);
    case 1: return mdrange_dispatch_T<int64_t>(op, (const int64_t*)base, rank, lower, upper, strides, tile, outer_left, inner_left, nthreads, out);
    case 2: return mdrange_dispatch_T<uint32_t>(op, (const uint32_t*)base, rank, lower, upper, strides, tile, outer_left, inner_left, nthreads, out);
    case 3: return mdrange_dispatch_T<uint64_t>(op, (const uint64_t*)base, rank, lower, upper, strides, tile, outer_left, inner_left, nthreads, out);
    case 4: return mdrange_dispatch_T<float>(op, (const float*)base, rank, lower, upper, strides, tile, outer_left, inner_left, nthreads, out);
    case 5: return mdrange_dispatch_T<double>(op, (const double*)base, rank, lower, upper, strides, tile, outer_left, inner_left, nthreads, out);
  }
  return 1;
}

// MDRangePolicy<Rank<N>>(lower, upper) on the host defaults: Iterate::Right
// outer and inner (KokkosExp_MDRangePolicy.hpp:48-58), default tiles.
int orc_mdrange_reduce(int op, int dtype, const void* base, int rank, const int64_t* lower,
                       const int64_t* upper, const int64_t* strides, int nthreads, void* out) {
  return orc_mdrange_reduce_ex(op, dtype, base, rank, lower, upper, strides, nullptr, 0, 0, nthreads, out);
}

// OpenMP ParallelScan: core/src/OpenMP/Kokkos_OpenMP_Parallel_Scan.hpp:69-140
// with WorkRange partition (core/src/Kokkos_ExecPolicy.hpp:315-333), and the
// std-algorithm functors:
//   exclusive: dest[i] = update + init; update += src[i]
//     (algorithms/src/std_algorithms/impl/Kokkos_FunctorsForExclusiveScan.hpp:50-55)
//   inclusive: update += src[i]; dest[i] = update
//     (algorithms/src/std_algorithms/impl/Kokkos_InclusiveScan.hpp:100-106)
// The accumulator type is the output type (int32 in -> int64 out widens).
}  // extern "C"
template <class TI, class TO>
static void scan_impl(int inclusive, const TI* x, int64_t n, TO init, TO* y, int P) {
  if (n <= 0) return;
  if (P < 1) P = 1;
  const int64_t gran = auto_chunk(n, P);
  const int64_t mask = gran - 1;
  const int64_t work_part = (((n + (P - 1)) / P) + mask) & ~mask;
  std::vector<TO> tot(P, TO(0)), base(P, TO(0));
  auto range = [&](int r) {
    int64_t b = work_part * r, e = b + work_part;
    if (n < b) b = n;
    if (n < e) e = n;
    return std::make_pair(b, e);
  };
#pragma omp parallel num_threads(P)
  {
    const int r0 = omp_get_thread_num();
    const int np = omp_get_num_threads();
    for (int r = r0; r < P; r += np) {
      auto rg = range(r);
      TO u = TO(0);
      for (int64_t i = rg.first; i < rg.second; ++i) u += (TO)x[i];
      tot[r] = u;
    }
#pragma omp barrier
#pragma omp single
    {
      // ptr[value_count] of thread i = join of totals of threads < i
      // (Kokkos_OpenMP_Parallel_Scan.hpp:109-130).
      base[0] = TO(0);
      for (int r = 1; r < P; ++r) { base[r] = base[r - 1]; base[r] += tot[r - 1]; }
    }
    for (int r = r0; r < P; r += np) {
      auto rg = range(r);
      TO u = base[r];
      for (int64_t i = rg.first; i < rg.second; ++i) {
        if (inclusive) { u += (TO)x[i]; y[i] = u; }
        else { const TO t = (TO)x[i]; y[i] = u + init; u += t; }
      }
    }
  }
}

extern "C" {
// in_dtype/out_dtype per the codes above; init is read as out_dtype
// (ignored for inclusive).
int orc_scan(int inclusive, int in_dtype, int out_dtype, const void* x, int64_t n, const void* init, void* y,
             int nthreads) {
#define ORC_SCAN_CASE(ci, TI, co, TO)                                                          \
  if (in_dtype == ci && out_dtype == co) {                                                     \
    scan_impl<TI, TO>(inclusive, (const TI*)x, n, init ? *(const TO*)init : TO(0), (TO*)y, nthreads); \
    return 0;                                                                                  \
  }
  ORC_SCAN_CASE(0, int32_t, 0, int32_t)
  ORC_SCAN_CASE(0, int32_t, 1, int64_t)
  ORC_SCAN_CASE(1, int64_t, 1, int64_t)
  ORC_SCAN_CASE(2, uint32_t, 2, uint32_t)
  ORC_SCAN_CASE(2, uint32_t, 3, uint64_t)
  ORC_SCAN_CASE(3, uint64_t, 3, uint64_t)
  ORC_SCAN_CASE(4, float, 4, float)
  ORC_SCAN_CASE(4, float, 5, double)
  ORC_SCAN_CASE(5, double, 5, double)
#undef ORC_SCAN_CASE
  return 1;
}

// ScatterView histogram on OpenMP (Duplicated + NonAtomic defaults,
// containers/src/Kokkos_ScatterView.hpp:84-96): every thread counts into a
// private copy of the bins, then ReduceDuplicates (:596-625) sums the copies
// into the destination, which keeps its previous contents.  Keys outside
// [0, nbins) are skipped and counted in *dropped (the reference leaves them
// undefined).
int orc_histogram_i32_i64(const int32_t* keys, int64_t n, int64_t* bins, int64_t nbins, int nthreads,
                          int64_t* dropped) {
  if (nbins <= 0) return 1;
  if (nthreads < 1) nthreads = 1;
  std::vector<std::vector<int64_t>> dup(nthreads, std::vector<int64_t>((size_t)nbins, 0));
  std::vector<int64_t> drop(nthreads, 0);
#pragma omp parallel num_threads(nthreads)
  {
    const int r = omp_get_thread_num(), np = omp_get_num_threads();
    for (int q = r; q < nthreads; q += np) {
      auto rg = work_partition(n, auto_chunk(n, nthreads), q, nthreads);
      int64_t* h = dup[q].data();
      for (int64_t i = rg.first; i < rg.second; ++i) {
        const int32_t k = keys[i];
        if (k >= 0 && k < nbins) h[k] += 1; else drop[q] += 1;
      }
    }
  }
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t b = 0; b < nbins; ++b) {
    int64_t s = bins[b];
    for (int t = 0; t < nthreads; ++t) s += dup[t][b];
    bins[b] = s;
  }
  if (dropped) {
    int64_t d = 0;
    for (int t = 0; t < nthreads; ++t) d += drop[t];
    *dropped = d;
  }
  return 0;
}

// Kokkos::sort on a host space: std::sort over the view
// (algorithms/src/sorting/Kokkos_SortPublicAPI.hpp:54-58).
int orc_sort_u64(uint64_t* keys, int64_t n) {
  std::sort(keys, keys + n);
  return 0;
}

// Stable sort_by_key: the (key, original position) order.  The reference
// OpenMP sort_by_key is std::sort over an index permutation and therefore
// unstable (algorithms/src/sorting/impl/Kokkos_SortByKeyImpl.hpp:265-347);
// stability is this project's definition of the tie order, equal to the
// reference whenever keys are distinct.
int orc_sort_by_key_stable_u64_i32(uint64_t* keys, int32_t* vals, int64_t n) {
  std::vector<int64_t> perm((size_t)n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) { return keys[a] < keys[b]; });
  std::vector<uint64_t> k2((size_t)n);
  std::vector<int32_t> v2((size_t)n);
  for (int64_t i = 0; i < n; ++i) { k2[i] = keys[perm[i]]; v2[i] = vals[perm[i]]; }
  std::memcpy(keys, k2.data(), sizeof(uint64_t) * (size_t)n);
  std::memcpy(vals, v2.data(), sizeof(int32_t) * (size_t)n);
  return 0;
}

// The reference OpenMP sort_by_key as it runs (for timing): iota permutation,
// std::sort of the permutation by key, then a gather of keys and values
// (Kokkos_SortByKeyImpl.hpp:265-347, applyPermutation :218-233).
int orc_sort_by_key_reference_u64_i32(uint64_t* keys, int32_t* vals, int64_t n, int nthreads) {
  std::vector<int64_t> perm((size_t)n);
  std::iota(perm.begin(), perm.end(), 0);
  std::sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) { return keys[a] < keys[b]; });
  std::vector<uint64_t> k2((size_t)n);
  std::vector<int32_t> v2((size_t)n);
#pragma omp parallel for num_threads(nthreads < 1 ? 1 : nthreads) schedule(static)
  for (int64_t i = 0; i < n; ++i) { k2[i] = keys[perm[i]]; v2[i] = vals[perm[i]]; }
  std::memcpy(keys, k2.data(), sizeof(uint64_t) * (size_t)n);
  std::memcpy(vals, v2.data(), sizeof(int32_t) * (size_t)n);
  return 0;
}

// BinSort with BinOp1D (algorithms/src/sorting/Kokkos_BinOpsPublicAPI.hpp:25-71):
// bin(k) = (int)((double(k) - double(min)) * mul), mul = nbins /
// (double(max) - double(min)) with the reference's rounding guard
// (max_bins * (1 - eps) ... see :43-52); here mul is passed in so the
// checker uses exactly the caller's value.  Writes the per-bin counts, the
// exclusive offsets and the stable permutation (input order kept inside a
// bin) of BinSort::create_permute_vector
// (algorithms/src/sorting/Kokkos_BinSortPublicAPI.hpp:208-238).
int orc_binsort_u64(const uint64_t* keys, int64_t n, int64_t nbins, double kmin, double mul, int32_t* counts,
                    int64_t* offsets, int64_t* perm) {
  if (nbins <= 0) return 1;
  std::vector<int64_t> c((size_t)nbins, 0);
  std::vector<int64_t> bin((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    int64_t b = (int64_t)(((double)keys[i] - kmin) * mul);
    if (b < 0) b = 0;
    if (b >= nbins) b = nbins - 1;
    bin[i] = b;
    c[b] += 1;
  }
  int64_t run = 0;
  for (int64_t b = 0; b < nbins; ++b) {
    counts[b] = (int32_t)c[b];
    offsets[b] = run;
    run += c[b];
  }
  std::vector<int64_t> cur(offsets, offsets + nbins);
  for (int64_t i = 0; i < n; ++i) perm[cur[bin[i]]++] = i;
  return 0;
}

// Per-segment Sum (float accumulation, sequential per segment) and the
// compensated FP64 per-segment sums; offsets has nseg+1 entries.
int orc_seg_sum_f32(const float* x, const int64_t* offsets, int64_t nseg, float* out, double* comp,
                    double* absum, int nthreads) {
#pragma omp parallel for num_threads(nthreads < 1 ? 1 : nthreads) schedule(dynamic, 16)
  for (int64_t s = 0; s < nseg; ++s) {
    const int64_t b = offsets[s], e = offsets[s + 1];
    float acc = 0.0f;
    for (int64_t i = b; i < e; ++i) acc += x[i];
    if (out) out[s] = acc;
    double cs, ca;
    neumaier(x + b, e - b, &cs, &ca, nullptr);
    if (comp) comp[s] = cs;
    if (absum) absum[s] = ca;
  }
  return 0;
}

// Per-segment inclusive_scan of int32 into int32 (exact).
int orc_seg_inclusive_scan_i32(const int32_t* x, const int64_t* offsets, int64_t nseg, int32_t* y, int nthreads) {
#pragma omp parallel for num_threads(nthreads < 1 ? 1 : nthreads) schedule(dynamic, 16)
  for (int64_t s = 0; s < nseg; ++s) {
    int32_t u = 0;
    for (int64_t i = offsets[s]; i < offsets[s + 1]; ++i) { u += x[i]; y[i] = u; }
  }
  return 0;
}

}  // extern "C"
