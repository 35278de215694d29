// extern "C" reduce / MDRange-reduce entry points (see include/gbk.h).
#include <cstring>
#include <type_traits>

#include "gbk_reduce_impl.cuh"

namespace gbk {
namespace {

size_t result_size(int op, int dt) {
  const size_t e = dtype_size(dt);
  switch (op) {
    case GBK_MINLOC:
    case GBK_MAXLOC: return 16;
    case GBK_MINMAX: return 2 * e;
    case GBK_MINMAXLOC: return (2 * e + 7) / 8 * 8 + 16;
    case GBK_MINMAXLOC_SUM: return (2 * e + 7) / 8 * 8 + 16 + (e + 7) / 8 * 8;
    default: return e;
  }
}

bool valid_op(int op, int dt) {
  if (op < GBK_SUM || op > GBK_MINMAXLOC_SUM) return false;
  if (dt < GBK_I32 || dt > GBK_F64) return false;
  if ((dt == GBK_F32 || dt == GBK_F64) && op >= GBK_LAND && op <= GBK_BOR) return false;
  return true;
}

int reduce_any(int op, int dt, const void* x, int64_t n, int64_t loc0, void* out, Workspace* w,
               const gbk_tuning_t* t) {
  switch (dt) {
    case GBK_I32: return reduce_typed<int32_t>(op, (const int32_t*)x, n, loc0, out, w, t);
    case GBK_I64: return reduce_typed<int64_t>(op, (const int64_t*)x, n, loc0, out, w, t);
    case GBK_U32: return reduce_typed<uint32_t>(op, (const uint32_t*)x, n, loc0, out, w, t);
    case GBK_U64: return reduce_typed<uint64_t>(op, (const uint64_t*)x, n, loc0, out, w, t);
    case GBK_F32: return reduce_typed<float>(op, (const float*)x, n, loc0, out, w, t);
    case GBK_F64: return reduce_typed<double>(op, (const double*)x, n, loc0, out, w, t);
  }
  return GBK_ERR_UNSUPPORTED;
}

int md_any(int op, int dt, const void* base, const MDBox& b, void* out, Workspace* w, const gbk_tuning_t* t) {
  switch (dt) {
    case GBK_I32: return mdreduce_typed<int32_t>(op, (const int32_t*)base, b, out, w, t);
    case GBK_I64: return mdreduce_typed<int64_t>(op, (const int64_t*)base, b, out, w, t);
    case GBK_U32: return mdreduce_typed<uint32_t>(op, (const uint32_t*)base, b, out, w, t);
    case GBK_U64: return mdreduce_typed<uint64_t>(op, (const uint64_t*)base, b, out, w, t);
    case GBK_F32: return mdreduce_typed<float>(op, (const float*)base, b, out, w, t);
    case GBK_F64: return mdreduce_typed<double>(op, (const double*)base, b, out, w, t);
  }
  return GBK_ERR_UNSUPPORTED;
}

// Analyse an MDRange box.  Returns 1 and the contiguous range [off, off+cnt)
// if the box is one contiguous run of memory; otherwise fills the row
// decomposition for the generic kernel.  Returns -1 on invalid input.
int md_plan(int rank, const int64_t* lo, const int64_t* up, const int64_t* st, int64_t* off, int64_t* cnt,
            MDBox* b) {
  if (rank < 1 || rank > 6 || !lo || !up || !st) return -1;
  int64_t ext[6];
  int64_t total = 1;
  for (int d = 0; d < rank; ++d) {
    if (lo[d] < 0) return -1;
    ext[d] = up[d] > lo[d] ? up[d] - lo[d] : 0;
    if (st[d] <= 0 && ext[d] > 1) return -1;
    total *= ext[d];
  }
  int64_t o = 0;
  for (int d = 0; d < rank; ++d) o += lo[d] * st[d];
  *off = o;
  *cnt = total;
  if (total == 0) {
    std::memset(b, 0, sizeof(*b));
    return 1;
  }
  // Order dimensions of extent > 1 by stride; contiguous when each stride is
  // the previous stride times the previous extent, starting from 1.
  int ord[6], m = 0;
  for (int d = 0; d < rank; ++d)
    if (ext[d] > 1) ord[m++] = d;
  for (int i = 1; i < m; ++i)
    for (int j = i; j > 0 && st[ord[j]] < st[ord[j - 1]]; --j) std::swap(ord[j], ord[j - 1]);
  bool contig = true;
  int64_t expect = 1;
  for (int i = 0; i < m; ++i) {
    if (st[ord[i]] != expect) { contig = false; break; }
    expect *= ext[ord[i]];
  }
  if (contig) return 1;
  // Generic: inner = smallest-stride dim, outer dims in stride order.
  std::memset(b, 0, sizeof(*b));
  const int in = ord[0];
  b->inner_lo = lo[in];
  b->inner_ext = ext[in];
  b->inner_stride = st[in];
  b->rank = 0;
  b->rows = 1;
  for (int i = 1; i < m; ++i) {
    const int d = ord[i];
    b->lo[b->rank] = lo[d];
    b->ext[b->rank] = ext[d];
    b->stride[b->rank] = st[d];
    b->rank++;
    b->rows *= ext[d];
  }
  // Dimensions of extent 1 contribute a fixed offset.
  int64_t fixed = 0;
  for (int d = 0; d < rank; ++d)
    if (ext[d] == 1) fixed += lo[d] * st[d];
  // Fold the fixed offset into the inner start (inner stride > 0).
  if (fixed % b->inner_stride == 0) {
    b->inner_lo += fixed / b->inner_stride;
  } else if (b->rank < 6) {
    b->lo[b->rank] = fixed;
    b->ext[b->rank] = 1;
    b->stride[b->rank] = 1;
    b->rank++;
  }
  return 0;
}

int md_launch(int op, int dt, const void* base, int rank, const int64_t* lo, const int64_t* up, const int64_t* st,
              void* out, Workspace* w, const gbk_tuning_t* t) {
  int64_t off = 0, cnt = 0;
  MDBox b;
  const int kind = md_plan(rank, lo, up, st, &off, &cnt, &b);
  if (kind < 0) return GBK_ERR_INVALID_ARGUMENT;
  if (kind == 1) {
    const char* p = (const char*)base + off * (int64_t)dtype_size(dt);
    gbk_tuning_t tt;
    if (!t) t = tuned_config(TUNE_REDUCE, op, dt, cnt, 0, &tt);
    return reduce_any(op, dt, p, cnt, off, out, w, t);
  }
  return md_any(op, dt, base, b, out, w, t);
}

}  // namespace
}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_reduce(gbk_reducer_t op, gbk_dtype_t dt, const void* x, int64_t n, void* result, gbk_stream_t stream,
               const gbk_tuning_t* tune) {
  if (!valid_op(op, dt)) return GBK_ERR_UNSUPPORTED;
  if (n < 0 || !result || (n > 0 && !x)) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)x % dtype_size(dt)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  gbk_tuning_t tt;
  if (!tune) tune = tuned_config(TUNE_REDUCE, op, dt, n, 0, &tt);
  std::lock_guard<std::mutex> lk(w->mu);
  return reduce_any(op, dt, x, n, 0, result, w, tune);
}

int gbk_reduce_host(gbk_reducer_t op, gbk_dtype_t dt, const void* hx, int64_t n, void* hres, gbk_stream_t stream,
                    const gbk_tuning_t* tune) {
  if (!valid_op(op, dt)) return GBK_ERR_UNSUPPORTED;
  if (n < 0 || !hres || (n > 0 && !hx)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Workspace* w = ws_get(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  const size_t bytes = (size_t)n * dtype_size(dt);
  const size_t rpad = (bytes + 255) / 256 * 256;
  char* d = ws_stage(w, rpad + 256, &st);
  if (!d) return st;
  if (bytes) GBK_CUDA_TRY(cudaMemcpyAsync(d, hx, bytes, cudaMemcpyHostToDevice, s));
  st = reduce_any(op, dt, d, n, 0, d + rpad, w, tune);
  if (st) return st;
  GBK_CUDA_TRY(cudaMemcpyAsync(hres, d + rpad, result_size(op, dt), cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  return GBK_OK;
}

int gbk_mdrange_reduce(gbk_reducer_t op, gbk_dtype_t dt, const void* base, int rank, const int64_t* lower,
                       const int64_t* upper, const int64_t* strides, void* result, gbk_stream_t stream,
                       const gbk_tuning_t* tune) {
  if (!valid_op(op, dt)) return GBK_ERR_UNSUPPORTED;
  if (!result || !base) return GBK_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)base % dtype_size(dt)) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  Workspace* w = ws_get((cudaStream_t)stream, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return md_launch(op, dt, base, rank, lower, upper, strides, result, w, tune);
}

int gbk_mdrange_reduce_host(gbk_reducer_t op, gbk_dtype_t dt, const void* hbase, int64_t view_elems, int rank,
                            const int64_t* lower, const int64_t* upper, const int64_t* strides, void* hres,
                            gbk_stream_t stream, const gbk_tuning_t* tune) {
  if (!valid_op(op, dt)) return GBK_ERR_UNSUPPORTED;
  if (!hres || !hbase || view_elems < 0) return GBK_ERR_INVALID_ARGUMENT;
  int st = GBK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Workspace* w = ws_get(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  const size_t bytes = (size_t)view_elems * dtype_size(dt);
  const size_t rpad = (bytes + 255) / 256 * 256;
  char* d = ws_stage(w, rpad + 256, &st);
  if (!d) return st;
  if (bytes) GBK_CUDA_TRY(cudaMemcpyAsync(d, hbase, bytes, cudaMemcpyHostToDevice, s));
  st = md_launch(op, dt, d, rank, lower, upper, strides, d + rpad, w, tune);
  if (st) return st;
  GBK_CUDA_TRY(cudaMemcpyAsync(hres, d + rpad, result_size(op, dt), cudaMemcpyDeviceToHost, s));
  GBK_CUDA_TRY(cudaStreamSynchronize(s));
  return GBK_OK;
}

#define GBK_DEFINE_TYPED_REDUCE(op, dt, T)                                                    \
  int gbk_reduce_##op##_##dt(const T* x, int64_t n, void* result, gbk_stream_t stream) {      \
    return gbk_reduce((gbk_reducer_t)GBK_OPCODE_##op, (gbk_dtype_t)GBK_DT_##dt, x, n, result, stream, nullptr); \
  }
#define GBK_OPCODE_sum GBK_SUM
#define GBK_OPCODE_prod GBK_PROD
#define GBK_OPCODE_min GBK_MIN
#define GBK_OPCODE_max GBK_MAX
#define GBK_OPCODE_land GBK_LAND
#define GBK_OPCODE_lor GBK_LOR
#define GBK_OPCODE_band GBK_BAND
#define GBK_OPCODE_bor GBK_BOR
#define GBK_OPCODE_minloc GBK_MINLOC
#define GBK_OPCODE_maxloc GBK_MAXLOC
#define GBK_OPCODE_minmax GBK_MINMAX
#define GBK_OPCODE_minmaxloc GBK_MINMAXLOC
#define GBK_DT_i32 GBK_I32
#define GBK_DT_i64 GBK_I64
#define GBK_DT_u32 GBK_U32
#define GBK_DT_u64 GBK_U64
#define GBK_DT_f32 GBK_F32
#define GBK_DT_f64 GBK_F64
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, sum)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, prod)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, min)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, max)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, minloc)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, maxloc)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, minmax)
GBK_FOR_EACH_DTYPE(GBK_DEFINE_TYPED_REDUCE, minmaxloc)
GBK_FOR_EACH_INT_DTYPE(GBK_DEFINE_TYPED_REDUCE, land)
GBK_FOR_EACH_INT_DTYPE(GBK_DEFINE_TYPED_REDUCE, lor)
GBK_FOR_EACH_INT_DTYPE(GBK_DEFINE_TYPED_REDUCE, band)
GBK_FOR_EACH_INT_DTYPE(GBK_DEFINE_TYPED_REDUCE, bor)

}  // extern "C"
