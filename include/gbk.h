/*
 * gbk.h — C ABI of the GB300 (sm_103a) reduce / scan / scatter / sort
 * library (libgbk.so).
 *
 * Plain pointers, int64_t sizes, an opaque stream handle and an int status.
 * Every data pointer is a device pointer (or memory the GPU can address)
 * unless the function name ends in _host.  Calls are asynchronous on the
 * given stream; results stay in device memory.  Device-side failures (a
 * bounded wait that ran out, a key outside the bin range) are recorded in
 * the stream's error word and returned by gbk_stream_check().
 *
 * Each entry point cites the reference interface it stands in for, by file
 * and line within the Kokkos source tree.
 *
 * Codes:
 *   dtype   : GBK_I32 0, GBK_I64 1, GBK_U32 2, GBK_U64 3, GBK_F32 4, GBK_F64 5
 *   reducer : Sum 0, Prod 1, Min 2, Max 3, LAnd 4, LOr 5, BAnd 6, BOr 7,
 *             MinLoc 8, MaxLoc 9, MinMax 10, MinMaxLoc 11
 *             (core/src/Kokkos_Parallel_Reduce.hpp:34,79,124,171,219,265,
 *              312,359,412,472,537,601).  LAnd/LOr/BAnd/BOr are defined for
 *             the integer dtypes only, as in the reference.
 *
 * Result layouts (core/src/Kokkos_Parallel_Reduce.hpp:406,532,596), with
 * Index = int64_t:
 *   Sum..BOr   : T
 *   MinLoc/Max : struct { T val; int64_t loc; }                  (16 bytes)
 *   MinMax     : struct { T min_val, max_val; }
 *   MinMaxLoc  : struct { T min_val, max_val; int64_t min_loc, max_loc; }
 * Identities follow core/src/Kokkos_ReductionIdentity.hpp: Min starts at the
 * type's maximum (FLT_MAX / DBL_MAX for floating point), Max at its lowest,
 * loc at INT64_MAX.  *Loc reducers: an element replaces the running value
 * only if strictly better, and ties between partial results resolve to the
 * smallest loc.
 */
#ifndef GBK_H_
#define GBK_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GBK_OK 0
#define GBK_ERR_INVALID_ARGUMENT 1
#define GBK_ERR_UNSUPPORTED 2
#define GBK_ERR_CUDA 3
#define GBK_ERR_DEVICE_TIMEOUT 4
#define GBK_ERR_OUT_OF_WORKSPACE 5
#define GBK_ERR_KEY_OUT_OF_RANGE 6
#define GBK_ERR_NO_DEVICE 7
#define GBK_ERR_SCRATCH_LIMIT 8 /* request exceeds the fixed scratch of gbk_reduce_noalloc */
#define GBK_ERR_DEVICE_ABORT 9  /* a kernel of the header paths called Kokkos::abort in device code */

typedef enum { GBK_I32 = 0, GBK_I64 = 1, GBK_U32 = 2, GBK_U64 = 3, GBK_F32 = 4, GBK_F64 = 5 } gbk_dtype_t;

typedef enum {
  GBK_SUM = 0, GBK_PROD = 1, GBK_MIN = 2, GBK_MAX = 3, GBK_LAND = 4, GBK_LOR = 5,
  GBK_BAND = 6, GBK_BOR = 7, GBK_MINLOC = 8, GBK_MAXLOC = 9, GBK_MINMAX = 10, GBK_MINMAXLOC = 11,
  /* MinMaxLoc and Sum in one pass: the parallel_reduce with several reducers
   * (core/src/impl/Kokkos_Combined_Reducer.hpp:533-580) for
   * parallel_reduce(policy, f, MinMaxLoc<T,int64_t>(r1), Sum<T>(r2)).  Result:
   * the MinMaxLoc record, then the sum (gbk_reduce and gbk_mdrange_reduce only). */
  GBK_MINMAXLOC_SUM = 12
} gbk_reducer_t;

/* A cudaStream_t; NULL is the legacy default stream. */
typedef void* gbk_stream_t;

/* Launch configuration.  Zero fields mean "library default / tuned".
 * Stands in for the tuned policy the Kokkos Tools tuning hook may return
 * (core/src/impl/Kokkos_Tools_Generic.hpp:546, Kokkos_Tuners.hpp:600-705). */
typedef struct {
  int32_t block;            /* threads per CTA: 128, 256, 512 or 1024            */
  int32_t items_per_thread; /* 16-byte vectors per thread per tile: 1, 2, 4, 8    */
  int32_t ctas_per_sm;      /* grid = SMs * ctas_per_sm (persistent kernels)      */
  int32_t variant;          /* kernel variant; op specific (0 = default)          */
} gbk_tuning_t;

/* ---- runtime ------------------------------------------------------------ */
/* Library version (major*10000 + minor*100 + patch). */
int gbk_version(void);
/* Text of a status code. */
const char* gbk_status_string(int status);
/* Current device: SM count, compute capability, L2 bytes.  Stands in for
 * the exec-space queries of core/src/Cuda/Kokkos_Cuda.hpp:95-260
 * (concurrency(), print_configuration()). */
int gbk_device_info(int* sm_count, int* cc_major, int* cc_minor, int64_t* l2_bytes);
/* Synchronise the stream, then return and clear the device error status of
 * its workspace (fence(), core/src/Cuda/Kokkos_Cuda.hpp; error convention of
 * core/src/Cuda/Kokkos_Cuda_Error.hpp:33-67). */
int gbk_stream_check(gbk_stream_t stream);
/* gbk_stream_check that also returns `bytes` (at most 256) read from device
 * memory at device_src once the stream's earlier work is done, into
 * host_dst: both reads land in a pinned host slot of the workspace, behind
 * one stream synchronisation.  The host-scalar result of a parallel_reduce:
 * the reference reads it from pinned "unified" scratch after one fence
 * (core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:344-359). */
int gbk_fence_read(gbk_stream_t stream, const void* device_src, void* host_dst, int64_t bytes);
/* Pre-size the stream's workspace (needed before graph capture). */
int gbk_workspace_reserve(gbk_stream_t stream, int64_t bytes);
/* Free every workspace (after all work on them has finished). */
int gbk_workspace_release_all(void);
/* For kernels instantiated in the caller's translation unit (the header
 * template path, include/Kokkos_GB300.hpp): the stream's workspace with at
 * least scratch_bytes of scratch, its 64 ticket counters (slots 32..63 are
 * free for the caller; each kernel resets the slot it takes) and its error
 * word.  Stands in for the per-instance scratch of
 * core/src/Cuda/Kokkos_Cuda_Instance.cpp:508-535 (scratch_space,
 * scratch_flags). */
int gbk_workspace_acquire(gbk_stream_t stream, int64_t scratch_bytes, void** scratch, unsigned** counters,
                          int** error_word);
/* Record `count` kernel launches made by caller-instantiated kernels in the
 * library's launch counter. */
int gbk_note_launches(int64_t count);
/* Bound, in polls, of every device-side wait (lookback, barriers).  The
 * default bounds a wait at roughly a second. */
int gbk_set_wait_limit(int64_t polls);
/* The current bound (for kernels instantiated outside the library). */
int64_t gbk_wait_limit(void);
/* Number of this library's kernels launched so far (all streams). */
int64_t gbk_launch_count(void);
/* deep_copy between any two buffers the runtime can address (host<->device
 * or device<->device), asynchronous on the stream
 * (core/src/Kokkos_CopyViews.hpp deep_copy(dst, src);
 *  DeepCopy<CudaSpace, HostSpace> in core/src/Cuda/Kokkos_CudaSpace.hpp). */
int gbk_deep_copy(void* dst, const void* src, int64_t bytes, gbk_stream_t stream);
/* deep_copy(view, value) for a byte value (e.g. zeroing bins before a
 * ScatterView contribution). */
int gbk_memset(void* dst, int value, int64_t bytes, gbk_stream_t stream);
/* deep_copy(view, value) for a contiguous device view of n elements of
 * elem_bytes (1, 2, 4, 8 or 16) bytes: every element becomes *value (a host
 * pointer to one element).  dst must be aligned to elem_bytes
 * (core/src/Kokkos_CopyViews.hpp:897 deep_copy(const View&, value_type) and
 * its ViewFill functors, Kokkos_CopyViews.hpp:58-260). */
int gbk_fill(void* dst, const void* value, int elem_bytes, int64_t n, gbk_stream_t stream);

/* ---- reduce over a RangePolicy of a contiguous array -------------------- */
/* parallel_reduce(RangePolicy(0,n), [=](i, v){ v op= x[i]; }, Reducer(r))
 * (core/src/Kokkos_Parallel_Reduce.hpp:1684-1790 dispatch,
 *  core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:118-388 CUDA ParallelReduce)
 * and std reduce (algorithms/src/std_algorithms/impl/Kokkos_Reduce.hpp:86-152).
 * result: device pointer to one value of the reducer's layout (above). */
int gbk_reduce(gbk_reducer_t op, gbk_dtype_t dtype, const void* x, int64_t n, void* result,
               gbk_stream_t stream, const gbk_tuning_t* tune);

/* Same, with x and result in HOST memory: copies x to the device, reduces,
 * copies the result back and synchronises (the deep_copy + parallel_reduce +
 * host-scalar result sequence, core/src/Kokkos_CopyViews.hpp and the fence
 * rule of core/src/Kokkos_Parallel_Reduce.hpp:1581-1640). */
int gbk_reduce_host(gbk_reducer_t op, gbk_dtype_t dtype, const void* host_x, int64_t n, void* host_result,
                    gbk_stream_t stream, const gbk_tuning_t* tune);

/* Typed entry points, one per (reducer, dtype):
 *   int gbk_reduce_<op>_<dt>(const T* x, int64_t n, R* result, gbk_stream_t s)
 * op in sum prod min max minloc maxloc minmax minmaxloc (all dtypes) and
 * land lor band bor (integer dtypes); dt in i32 i64 u32 u64 f32 f64. */
#define GBK_DECLARE_TYPED_REDUCE(op, dt, T) \
  int gbk_reduce_##op##_##dt(const T* x, int64_t n, void* result, gbk_stream_t stream);
#define GBK_FOR_EACH_DTYPE(M, op)                                                                  \
  M(op, i32, int32_t) M(op, i64, int64_t) M(op, u32, uint32_t) M(op, u64, uint64_t) M(op, f32, float) \
  M(op, f64, double)
#define GBK_FOR_EACH_INT_DTYPE(M, op) \
  M(op, i32, int32_t) M(op, i64, int64_t) M(op, u32, uint32_t) M(op, u64, uint64_t)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, sum)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, prod)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, min)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, max)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, minloc)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, maxloc)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, minmax)
GBK_FOR_EACH_DTYPE(GBK_DECLARE_TYPED_REDUCE, minmaxloc)
GBK_FOR_EACH_INT_DTYPE(GBK_DECLARE_TYPED_REDUCE, land)
GBK_FOR_EACH_INT_DTYPE(GBK_DECLARE_TYPED_REDUCE, lor)
GBK_FOR_EACH_INT_DTYPE(GBK_DECLARE_TYPED_REDUCE, band)
GBK_FOR_EACH_INT_DTYPE(GBK_DECLARE_TYPED_REDUCE, bor)

/* Reduce that allocates nothing.  No counterpart in the reference: it is
 * for callers that may not allocate device memory — code working inside a
 * device-memory budget owned by someone else (a framework's caching
 * allocator, an application that forbids allocations after start-up) and
 * latency-critical loops that must not hit the device-wide synchronisation
 * cudaMalloc/cudaFree can cause.  Reducers GBK_SUM .. GBK_MINMAXLOC over the
 * six dtypes, with gbk_reduce's result layout; GBK_MINMAXLOC_SUM returns
 * GBK_ERR_UNSUPPORTED.  It always runs the load-pipelined flat kernel with
 * gbk_reduce's default launch shape (grid = SMs * ctas_per_sm CTAs of 256
 * threads, ctas_per_sm 0 = 8), whereas gbk_reduce may pick another kernel
 * for large inputs (the bulk-copy ring kernel, the split fixed-point double
 * Sum): integer results, Min/Max and the *Loc results are identical, but
 * float and double Sums can differ from gbk_reduce's in the last bits.
 * The per-CTA partial values and the ticket live in one fixed device array
 * inside the library: 128 KiB + 256 B per GPU that loads the library, held
 * until the process exits, room for at most 4096 CTAs.  A call that would
 * need more CTAs returns GBK_ERR_SCRATCH_LIMIT.  The caller still provides
 * x and result (device memory).  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) and clears its ticket on the
 * call's stream; that first call should come before any stream capture, and
 * the address is kept until exit, so a process that resets the device
 * (cudaDeviceReset) must not call this entry point afterwards.  All calls on
 * a device share the array: calls whose kernels may overlap on the GPU
 * (different streams not ordered by events) race and must not be issued. */
int gbk_reduce_noalloc(gbk_reducer_t op, gbk_dtype_t dtype, const void* x, int64_t n, void* result,
                       gbk_stream_t stream, int32_t ctas_per_sm);

/* ---- reduce over an MDRangePolicy box of a strided view ------------------ */
/* parallel_reduce(MDRangePolicy<Rank<rank>>(lower, upper),
 *                 [=](i0..ir, v){ v op= x(i0..ir); }, Reducer(r))
 * (core/src/KokkosExp_MDRangePolicy.hpp:159-425,
 *  core/src/Cuda/Kokkos_Cuda_Parallel_MDRange.hpp:248-497).
 * base: element (0,..,0) of the view; strides in elements (LayoutLeft:
 * 1, n0, n0*n1, ...; LayoutRight: reversed).  rank 1..6.  loc of the *Loc
 * reducers = sum_d i_d * strides[d], the element's offset from base. */
int gbk_mdrange_reduce(gbk_reducer_t op, gbk_dtype_t dtype, const void* base, int rank, const int64_t* lower,
                       const int64_t* upper, const int64_t* strides, void* result, gbk_stream_t stream,
                       const gbk_tuning_t* tune);
int gbk_mdrange_reduce_host(gbk_reducer_t op, gbk_dtype_t dtype, const void* host_base, int64_t view_elems,
                            int rank, const int64_t* lower, const int64_t* upper, const int64_t* strides,
                            void* host_result, gbk_stream_t stream, const gbk_tuning_t* tune);

/* ---- scans -------------------------------------------------------------- */
/* Single-pass scan of x[0..n) into y[0..n):
 *   exclusive: y[i] = init + sum_{j<i} x[j]   (std exclusive_scan,
 *     algorithms/src/std_algorithms/impl/Kokkos_ExclusiveScan.hpp:37-90,
 *     functor impl/Kokkos_FunctorsForExclusiveScan.hpp:31-54)
 *   inclusive: y[i] = sum_{j<=i} x[j]         (std inclusive_scan,
 *     algorithms/src/std_algorithms/impl/Kokkos_InclusiveScan.hpp:85-230)
 * which replace parallel_scan over a RangePolicy (core/src/Kokkos_Parallel.hpp:351-458;
 * CUDA ParallelScan core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:390-700).
 * Accumulation is in the OUTPUT type.  Supported (in, out) pairs:
 * (i32,i32) (i32,i64) (i64,i64) (u32,u32) (u32,u64) (u64,u64) (f32,f32)
 * (f32,f64) (f64,f64).  init points to one value of the output type in
 * HOST memory (ignored for inclusive; NULL = 0).  total (may be NULL):
 * device pointer receiving init + the sum of all x, as ParallelScanWithTotal
 * (core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:704-1053).  x and y may be
 * the same array (in place) only when in and out types match. */
int gbk_scan(int inclusive, gbk_dtype_t in_dtype, gbk_dtype_t out_dtype, const void* x, int64_t n,
             const void* init, void* y, void* total, gbk_stream_t stream, const gbk_tuning_t* tune);
/* Typed: exclusive_scan of int32 into int64 (the std-algorithm call with an
 * int64 init), and inclusive scans. */
int gbk_exclusive_scan_i32_i64(const int32_t* x, int64_t n, int64_t init, int64_t* y, gbk_stream_t stream);
int gbk_inclusive_scan_i32(const int32_t* x, int64_t n, int32_t* y, gbk_stream_t stream);
int gbk_inclusive_scan_f64(const double* x, int64_t n, double* y, gbk_stream_t stream);
int gbk_exclusive_scan_i32_i64_host(const int32_t* host_x, int64_t n, int64_t init, int64_t* host_y,
                                    gbk_stream_t stream);

/* ---- scatter (ScatterView contribute) ----------------------------------- */
/* Histogram: bins[keys[i]] += 1 for every i, into existing int64 bins, as
 *   auto sv = create_scatter_view(bins);
 *   parallel_for(n, [=](i){ sv.access()(keys[i]) += 1; }); contribute(bins, sv);
 * (containers/src/Kokkos_ScatterView.hpp:152-165 defaults, :250-286
 *  ScatterValue<ScatterSum,...,ScatterAtomic>, :1532-1580 contribute).
 * Keys outside [0, nbins) are skipped and flag GBK_ERR_KEY_OUT_OF_RANGE at
 * the next gbk_stream_check (the reference leaves them undefined). */
int gbk_histogram_i32_i64(const int32_t* keys, int64_t n, int64_t* bins, int64_t nbins, gbk_stream_t stream,
                          const gbk_tuning_t* tune);
int gbk_histogram_i32_i64_host(const int32_t* host_keys, int64_t n, int64_t* host_bins, int64_t nbins,
                               gbk_stream_t stream, const gbk_tuning_t* tune);
/* General scatter: dest[idx[i]] op= vals[i] with op in Sum (0), Prod (1),
 * Min (2), Max (3) — ScatterSum/ScatterProd/ScatterMin/ScatterMax
 * (containers/src/Kokkos_ScatterView.hpp:41-50, :207-460); dtype of vals
 * and dest in i32 i64 u32 u64 f32 f64 (Prod: integer and float types via
 * compare-and-swap).  Floating-point Sum order is not deterministic. */
int gbk_scatter(gbk_reducer_t op, gbk_dtype_t dtype, const int32_t* idx, const void* vals, int64_t n, void* dest,
                int64_t ndest, gbk_stream_t stream);

/* ---- batched segmented work ------------------------------------------------ */
/* Segments s = [offsets[s], offsets[s+1]) of x[0..n), offsets non-decreasing
 * with offsets[0] = 0 and offsets[nseg] = n (device memory, int64).  All
 * segments are processed in ONE launch, load-balanced over equal shares (or
 * tiles) of the concatenated array whatever the segment lengths.  Stands in for the
 * TeamPolicy league pattern, one team per segment with a TeamThreadRange
 * reduce / scan inside (core/src/Kokkos_ExecPolicy.hpp:366-700,
 * core/src/Cuda/Kokkos_Cuda_Parallel_Team.hpp:589-980,
 * core/src/OpenMP/Kokkos_OpenMP_Parallel_Reduce.hpp:332-530), and for a loop
 * of one parallel_reduce / inclusive_scan per segment.
 * reduce: out[s] = op over segment s (Sum, Min, Max; identity for an empty
 * segment), all six dtypes.  Variant 0 (default): contiguous per-CTA shares
 * for 16-byte aligned x of at least one 16 KiB chunk; variant 1 (and any
 * other x): the tile pipeline, tune->items_per_thread (3 or 7) sets its
 * tile.  NULL = tuning table or default.  Results are deterministic. */
int gbk_segmented_reduce(gbk_reducer_t op, gbk_dtype_t dtype, const void* x, const int64_t* offsets, int64_t nseg,
                         int64_t n, void* out, gbk_stream_t stream, const gbk_tuning_t* tune);
/* scan: per-segment inclusive / exclusive (from 0) prefix sums, (in, out) in
 * (i32,i32) (i32,i64) (i64,i64) (f32,f32) (f64,f64). */
int gbk_segmented_scan(int inclusive, gbk_dtype_t in_dtype, gbk_dtype_t out_dtype, const void* x,
                       const int64_t* offsets, int64_t nseg, int64_t n, void* y, gbk_stream_t stream,
                       const gbk_tuning_t* tune);

/* ---- graphs ----------------------------------------------------------------- */
/* Kokkos::Experimental::Graph for this library's calls
 * (core/src/Kokkos_Graph.hpp:42-183, Kokkos_GraphNode.hpp:227-470; CUDA
 * GraphImpl core/src/Cuda/Kokkos_Cuda_Graph_Impl.hpp:59-215): every gbk_*
 * call issued on `stream` between begin and end becomes a node of a CUDA
 * graph, in issue order (each node depends on the previous one, as a chain
 * of then_parallel_* nodes).  Calls that synchronise the host (*_host,
 * gbk_stream_check) and gbk_binsort_u64 (its staging buffer) cannot be
 * captured; sorts can.  Before capturing, size the stream's workspace with
 * gbk_workspace_reserve and run each call once uncaptured.
 * submit() = gbk_graph_launch. */
typedef struct gbk_graph_s* gbk_graph_t;
int gbk_graph_begin(gbk_stream_t stream);
int gbk_graph_end(gbk_stream_t stream, gbk_graph_t* graph);
int gbk_graph_launch(gbk_graph_t graph, gbk_stream_t stream);
int gbk_graph_destroy(gbk_graph_t graph);

/* ---- sort ----------------------------------------------------------------- */
/* Kokkos::sort(exec, view) for a contiguous view of i32 i64 u32 u64 f32 f64
 * keys, ascending, in place (algorithms/src/sorting/Kokkos_SortPublicAPI.hpp:31-116;
 * the reference's CUDA path is thrust::sort, impl/Kokkos_SortImpl.hpp:204-219).
 * Floating point: -0.0 sorts before +0.0, NaNs after +inf (sign-bit clear)
 * or before -inf (sign-bit set).  Stable LSD radix sort; digit passes whose
 * 8-bit digit is the same for every key are skipped, decided on the device
 * from the digit histogram, so the call never waits for the GPU and can be
 * captured into a graph (its workspace, about n x (key + value) bytes, must
 * exist first: gbk_workspace_reserve or one uncaptured call).  n < 2^30. */
int gbk_sort(gbk_dtype_t key_dtype, void* keys, int64_t n, gbk_stream_t stream);
/* Experimental::sort_by_key(exec, keys, values) (Kokkos_SortByKeyPublicAPI.hpp:30-114,
 * CUDA path thrust::sort_by_key, impl/Kokkos_SortByKeyImpl.hpp:125-138):
 * values of 4 or 8 bytes move with their keys.  STABLE: equal keys keep their
 * input order (the reference's OpenMP sort_by_key is not stable; on distinct
 * keys the results are identical). */
int gbk_sort_by_key(gbk_dtype_t key_dtype, void* keys, int value_bytes, void* values, int64_t n,
                    gbk_stream_t stream);
int gbk_sort_u64(uint64_t* keys, int64_t n, gbk_stream_t stream);
int gbk_sort_by_key_u64_i32(uint64_t* keys, int32_t* values, int64_t n, gbk_stream_t stream);
/* BinSort(keys, BinOp1D(nbins-1, min, max), sort_within_bins)
 * .create_permute_vector() (algorithms/src/sorting/Kokkos_BinSortPublicAPI.hpp:208-238,
 * BinOp1D Kokkos_BinOpsPublicAPI.hpp:25-71): bin(k) = (int)(mul * (double(k)
 * - kmin)) with the caller's mul and kmin (BinOp1D::mul_, min_); nbins =
 * BinOp1D::max_bins().  Writes bin_count[nbins] (int32), bin_offsets[nbins]
 * (exclusive starts, int64) and perm[n] (int64): the stable permutation by
 * bin (by key inside a bin when sort_within_bins).  The reference bins with
 * atomics, so its order inside a bin is arbitrary; bin contents are equal. */
int gbk_binsort_u64(const uint64_t* keys, int64_t n, int64_t nbins, double kmin, double mul, int sort_within_bins,
                    int32_t* bin_count, int64_t* bin_offsets, int64_t* perm, gbk_stream_t stream);
/* BinSort::sort(values) / applyPermutation: dst[i] = src[perm[i]] for
 * elements of value_bytes (1, 2, 4, 8) bytes; dst must not alias src
 * (Kokkos_BinSortPublicAPI.hpp:251-319, impl/Kokkos_SortByKeyImpl.hpp:218-233). */
int gbk_permute(int value_bytes, const void* src, const int64_t* perm, int64_t n, void* dst, gbk_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GBK_H_ */
