// Reduce kernels: contiguous RangePolicy reduce and MDRange box reduce.
//
// Flat kernel (replaces the CUDA ParallelReduce<RangePolicy> of
// core/src/Cuda/Kokkos_Cuda_Parallel_Range.hpp:191-368): a persistent grid
// of SMs x ctas_per_sm CTAs walks tiles of BLOCK*UNROLL 16-byte vectors;
// each thread keeps UNROLL independent 16-byte loads in flight
// (ld.global.nc.L1::no_allocate with an L2 256-byte prefetch hint), folds
// them into one running value with the reducer's element functor, then a
// warp tree (redux.sync for 32-bit integer Sum/Min/Max/BAnd/BOr, shuffles
// otherwise) and a CTA tree produce one partial per CTA.  The last CTA to
// finish (ticket from one atomicAdd) combines the partials in CTA order and
// writes the result: one launch, no second pass, no wait loop.  The
// combine order is fixed by the grid, so results are deterministic for a
// given configuration.
//
// MDRange kernel (replaces core/src/Cuda/Kokkos_Cuda_Parallel_MDRange.hpp:
// 248-497): when the box is one contiguous range of memory (LayoutLeft or
// LayoutRight view, box covering all but the slowest dimension) the host
// collapses it to the flat kernel.  Otherwise each warp walks one row of
// the dimension with the smallest stride at a time, lanes across the row.
#pragma once

#include "gbk_internal.cuh"

namespace gbk {

struct ReduceCfg {
  int block, unroll, ctas_per_sm;
};

template <class V>
__device__ __forceinline__ V ldcg_v(const V* p) {
  static_assert(sizeof(V) % 4 == 0, "value size");
  V r;
  const unsigned* s = reinterpret_cast<const unsigned*>(p);
  unsigned* d = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(V) / 4); ++i) d[i] = __ldcg(s + i);
  return r;
}

// Combine this CTA's value into the grid result with the last-CTA pattern.
template <class R, int BLOCK>
__device__ __forceinline__ void grid_finish(typename R::V acc, typename R::V* partials, unsigned* counter,
                                            typename R::V* out, typename R::V* sm) {
  using V = typename R::V;
  __shared__ unsigned s_ticket;
  acc = block_reduce<R, BLOCK>(acc, sm);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    __threadfence();
    s_ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (s_ticket != gridDim.x - 1) return;
  __threadfence();
  V a = R::init();
  for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) {
    V p = ldcg_v(partials + i);
    R::join(a, p);
  }
  __syncthreads();  // sm is reused by the second tree
  a = block_reduce<R, BLOCK>(a, sm);
  if (threadIdx.x == 0) {
    *out = a;
    *counter = 0u;  // ready for the next launch on this stream
  }
}

template <class R, class T, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK)
    k_reduce_flat(const T* __restrict__ x, int64_t n, int64_t head, int64_t loc0, typename R::V* partials,
                  unsigned* counter, typename R::V* out) {
  using V = typename R::V;
  constexpr int VEC = 16 / sizeof(T);
  __shared__ V sm[BLOCK / 32];
  V acc = R::init();
  const int64_t gtid = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  pdl_entry();
  // Unaligned head [0, head): one element per thread.
  if (gtid < head) R::template update<true>(acc, x[gtid], loc0 + gtid);
  const T* xb = x + head;
  const int64_t nvec = (n - head) / VEC;
  constexpr int64_t TILE = (int64_t)BLOCK * UNROLL;
  const int64_t lb = loc0 + head;
  // Each CTA owns one contiguous, equal share of the whole vectors.
  const int64_t per = nvec / gridDim.x, rem = nvec % gridDim.x;
  const int64_t v0 = (int64_t)blockIdx.x * per + ((int64_t)blockIdx.x < rem ? blockIdx.x : rem);
  const int64_t v1 = v0 + per + ((int64_t)blockIdx.x < rem ? 1 : 0);
  // Software pipeline: the next tile's UNROLL loads are issued before the
  // current tile is folded, so 2*UNROLL 16-byte loads per thread overlap.
  int64_t vb = v0 + threadIdx.x;
  bool have = vb + (int64_t)(UNROLL - 1) * BLOCK < v1;
  Vec16<T> cur[UNROLL], nxt[UNROLL];
  if (have) {
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u].u = ld_stream16(xb + (vb + (int64_t)u * BLOCK) * VEC);
  }
  while (have) {
    const int64_t vn = vb + TILE;
    const bool hn = vn + (int64_t)(UNROLL - 1) * BLOCK < v1;
    if (hn) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) nxt[u].u = ld_stream16(xb + (vn + (int64_t)u * BLOCK) * VEC);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const int64_t e0 = lb + (vb + (int64_t)u * BLOCK) * VEC;
      VecUpd<R, T, VEC>::run(acc, cur[u].v, e0);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = nxt[u];
    vb = vn;
    have = hn;
  }
  for (; vb < v1; vb += BLOCK) {
    Vec16<T> v;
    v.u = ld_stream16(xb + vb * VEC);
    VecUpd<R, T, VEC>::run(acc, v.v, lb + vb * VEC);
  }
  // Tail elements after the last whole vector.
  const int64_t t0 = head + nvec * VEC;
  if (t0 + gtid < n) R::template update<true>(acc, x[t0 + gtid], loc0 + t0 + gtid);
  grid_finish<R, BLOCK>(acc, partials, counter, out, sm);
}

// Flat reduce through a shared-memory ring (TMA engine): each CTA owns one
// contiguous, equal share of the whole vectors and streams it in chunks of
// CV 16-byte vectors by 1-D bulk copies into STAGES stages (mbarrier
// completion), so STAGES - 1 chunks per CTA are in flight while the threads
// fold the current one from shared memory (vector k * BLOCK + tid: striped,
// conflict-free, and increasing per thread, as the ordered *Loc updates
// want).  Head and tail elements and the grid finish are those of the flat
// kernel.  x + head must be 16-byte aligned (it is, by construction of head).
template <class R, class T, int BLOCK, int CV, int STAGES>
__global__ void __launch_bounds__(BLOCK)
    k_reduce_tma(const T* __restrict__ x, int64_t n, int64_t head, int64_t loc0, typename R::V* partials,
                 unsigned* counter, typename R::V* out, int* err, int64_t wait_limit) {
  using V = typename R::V;
  constexpr int VEC = 16 / sizeof(T);
  constexpr unsigned CHUNK_BYTES = (unsigned)CV * 16;
  static_assert(CV % BLOCK == 0, "whole rows of vectors per chunk");
  extern __shared__ __align__(128) unsigned char ring[];
  __shared__ __align__(8) unsigned long long s_bar[STAGES];
  __shared__ V sm[BLOCK / 32];
  V acc = R::init();
  const int64_t gtid = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  pdl_entry();
  if (gtid < head) R::template update<true>(acc, x[gtid], loc0 + gtid);
  const T* xb = x + head;
  const int64_t nvec = (n - head) / VEC;
  const int64_t lb = loc0 + head;
  const int64_t per = nvec / gridDim.x, rem = nvec % gridDim.x;
  const int64_t v0 = (int64_t)blockIdx.x * per + ((int64_t)blockIdx.x < rem ? blockIdx.x : rem);
  const int64_t v1 = v0 + per + ((int64_t)blockIdx.x < rem ? 1 : 0);
  const int64_t nchunks = (v1 - v0 + CV - 1) / CV;
  // Thread 0 only: start the copy of chunk c into its stage.
  auto fill = [&](int64_t c) {
    if (c >= nchunks) return;
    const int s = (int)(c % STAGES);
    const int64_t c0 = v0 + c * CV;
    const int64_t cnt = v1 - c0 < CV ? v1 - c0 : CV;
    mbar_arrive_expect_tx(&s_bar[s], (unsigned)(cnt * 16));
    bulk_g2s(ring + (size_t)s * CHUNK_BYTES, xb + c0 * VEC, (unsigned)(cnt * 16), &s_bar[s]);
  };
  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; ++s) mbar_init(&s_bar[s], 1);
    fence_mbar_init();
    for (int s = 0; s < STAGES; ++s) fill(s);
  }
  __syncthreads();
  bool bad = false;
  for (int64_t c = 0; c < nchunks; ++c) {
    const int s = (int)(c % STAGES);
    if (!mbar_wait(&s_bar[s], (unsigned)(c / STAGES) & 1u, wait_limit)) bad = true;
    const int64_t c0 = v0 + c * CV;
    const int cnt = (int)(v1 - c0 < CV ? v1 - c0 : CV);
    const uint4* sv = reinterpret_cast<const uint4*>(ring + (size_t)s * CHUNK_BYTES);
    if (cnt == CV) {
      // Take the chunk into registers and hand the stage back to the copy
      // engine before folding, so the refill overlaps the fold.
      Vec16<T> u[CV / BLOCK];
#pragma unroll
      for (int k = 0; k < CV / BLOCK; ++k) u[k].u = sv[k * BLOCK + threadIdx.x];
      __syncthreads();  // stage s fully read: refill it
      if (threadIdx.x == 0) fill(c + STAGES);
#pragma unroll
      for (int k = 0; k < CV / BLOCK; ++k)
        VecUpd<R, T, VEC>::run(acc, u[k].v, lb + (c0 + k * BLOCK + threadIdx.x) * VEC);
    } else {
      for (int i = threadIdx.x; i < cnt; i += BLOCK) {
        Vec16<T> u;
        u.u = sv[i];
        const int64_t e0 = lb + (c0 + i) * VEC;
        VecUpd<R, T, VEC>::run(acc, u.v, e0);
      }
      __syncthreads();  // stage s fully read: refill it
      if (threadIdx.x == 0) fill(c + STAGES);
    }
  }
  const int64_t t0 = head + nvec * VEC;
  if (t0 + gtid < n) R::template update<true>(acc, x[t0 + gtid], loc0 + t0 + gtid);
  if (bad) atomicOr(err, GBK_EBIT_TIMEOUT);
  grid_finish<R, BLOCK>(acc, partials, counter, out, sm);
}

template <class R>
__global__ void k_write_identity(typename R::V* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = R::init();
}

struct MDBox {
  int64_t lo[6], ext[6], stride[6];
  int rank;    // number of outer dims in lo/ext/stride (inner dim removed)
  int64_t inner_lo, inner_ext, inner_stride;
  int64_t rows;
};

template <class R, class T, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_reduce_md(const T* __restrict__ base, MDBox b, typename R::V* partials, unsigned* counter,
                typename R::V* out) {
  using V = typename R::V;
  __shared__ V sm[BLOCK / 32];
  V acc = R::init();
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * BLOCK) >> 5;
  for (int64_t r = gw; r < b.rows; r += nw) {
    int64_t rem = r, off = 0;
    for (int d = 0; d < b.rank; ++d) {
      const int64_t i = b.lo[d] + rem % b.ext[d];
      rem /= b.ext[d];
      off += i * b.stride[d];
    }
    for (int64_t i = lane; i < b.inner_ext; i += 32) {
      const int64_t o = off + (b.inner_lo + i) * b.inner_stride;
      R::template update<false>(acc, __ldg(base + o), o);
    }
  }
  grid_finish<R, BLOCK>(acc, partials, counter, out, sm);
}

// ---------------------------------------------------------------------------
// host launchers
template <class R, class T, int BLOCK, int UNROLL>
int launch_flat(const T* x, int64_t n, int64_t loc0, void* out, Workspace* w, int ctas_per_sm) {
  using V = typename R::V;
  cudaStream_t s = w->stream;
  if (n <= 0) {
    k_write_identity<R><<<1, 32, 0, s>>>((V*)out);
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  constexpr int VEC = 16 / sizeof(T);
  const uintptr_t a = (uintptr_t)x;
  int64_t head = (int64_t)(((16 - (a & 15)) & 15) / sizeof(T));
  if (head > n) head = n;
  const int64_t nvec = (n - head) / VEC;
  const int64_t tiles = (nvec + (int64_t)BLOCK * UNROLL - 1) / ((int64_t)BLOCK * UNROLL);
  int64_t grid = (int64_t)sm_count() * (ctas_per_sm > 0 ? ctas_per_sm : 4);
  if (grid > tiles) grid = tiles;
  if (grid < 1) grid = 1;
  // head and tail are handled one element per thread: need enough threads.
  const int64_t tail = (n - head) - nvec * VEC;
  while (grid * BLOCK < head || grid * BLOCK < tail) ++grid;
  int st = GBK_OK;
  char* scr = ws_scratch(w, sizeof(V) * (size_t)grid + 256, &st);
  if (!scr) return st;
  GBK_CUDA_TRY(launch_pdl(k_reduce_flat<R, T, BLOCK, UNROLL>, dim3((unsigned)grid), dim3(BLOCK), 0, s, x, n, head,
                          loc0, (V*)scr, w->counters + SLOT_REDUCE, (V*)out));
  note_launch();
  return GBK_OK;
}

// Ring reduce: 256 threads, chunks of 1024 vectors (16 KiB), 4 stages: three
// CTAs per SM keep about 144 KiB per SM in flight.
template <class R, class T>
int launch_tma(const T* x, int64_t n, int64_t loc0, void* out, Workspace* w, int cps) {
  using V = typename R::V;
  constexpr int BLOCK = 256, CV = 1024, STAGES = 4;
  constexpr int VEC = 16 / sizeof(T);
  cudaStream_t s = w->stream;
  const uintptr_t a = (uintptr_t)x;
  int64_t head = (int64_t)(((16 - (a & 15)) & 15) / sizeof(T));
  if (head > n) head = n;
  const int64_t nvec = (n - head) / VEC;
  auto kfn = k_reduce_tma<R, T, BLOCK, CV, STAGES>;
  constexpr size_t dyn = (size_t)STAGES * CV * 16;
  static std::atomic<int> resident{0};  // CTAs per SM, per instantiation (set once, any host thread)
  if (!resident) {
    GBK_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int r = 0;
    GBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kfn, BLOCK, dyn));
    resident = r > 0 ? r : 1;
  }
  const int per_sm = cps > 0 && cps < resident ? cps : resident.load();
  int64_t grid = (int64_t)sm_count() * per_sm;
  const int64_t chunks = (nvec + CV - 1) / CV;
  if (grid > chunks) grid = chunks;
  if (grid < 1) grid = 1;
  const int64_t tail = (n - head) - nvec * VEC;
  while (grid * BLOCK < head || grid * BLOCK < tail) ++grid;
  int st = GBK_OK;
  char* scr = ws_scratch(w, sizeof(V) * (size_t)grid + 256, &st);
  if (!scr) return st;
  GBK_CUDA_TRY(launch_pdl(kfn, dim3((unsigned)grid), dim3(BLOCK), dyn, s, x, n, head, loc0, (V*)scr,
                          w->counters + SLOT_REDUCE, (V*)out, w->err, wait_limit()));
  note_launch();
  return GBK_OK;
}

// variant 1: the load-pipelined kernel (block, items_per_thread, ctas_per_sm
// from the tuning); variant 2: the ring kernel (ctas_per_sm); variant 0: the
// ring kernel for inputs of 4 MiB and more, else the load-pipelined one.
template <class R, class T>
int launch_flat_cfg(const T* x, int64_t n, int64_t loc0, void* out, Workspace* w, const gbk_tuning_t* t) {
  const int variant = t ? t->variant : 0;
  if (n > 0 && (variant == 2 || (variant == 0 && n * (int64_t)sizeof(T) >= ((int64_t)4 << 20))))
    return launch_tma<R, T>(x, n, loc0, out, w, variant == 2 && t ? t->ctas_per_sm : 0);
  const int blk = t && t->block ? t->block : 256;
  const int un = t && t->items_per_thread ? t->items_per_thread : 4;
  const int cps = t && t->ctas_per_sm ? t->ctas_per_sm : (blk >= 512 ? 4 : 8);
  // The configurations compiled for every reducer; others fall back to 256x4.
  if (blk == 256 && un == 2) return launch_flat<R, T, 256, 2>(x, n, loc0, out, w, cps);
  if (blk == 512 && un == 2) return launch_flat<R, T, 512, 2>(x, n, loc0, out, w, cps);
  if (blk == 512 && un == 4) return launch_flat<R, T, 512, 4>(x, n, loc0, out, w, cps);
  if (blk == 128 && un == 8) return launch_flat<R, T, 128, 8>(x, n, loc0, out, w, cps);
  if (blk == 256 && un == 8) return launch_flat<R, T, 256, 8>(x, n, loc0, out, w, cps);
  if (blk == 1024 && un == 2) return launch_flat<R, T, 1024, 2>(x, n, loc0, out, w, cps);
  return launch_flat<R, T, 256, 4>(x, n, loc0, out, w, cps);
}

template <class R, class T>
int launch_md(const T* base, const MDBox& b, void* out, Workspace* w, const gbk_tuning_t* t) {
  using V = typename R::V;
  cudaStream_t s = w->stream;
  constexpr int BLOCK = 256;
  int64_t total = b.rows * b.inner_ext;
  if (total <= 0) {
    k_write_identity<R><<<1, 32, 0, s>>>((V*)out);
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  const int cps = t && t->ctas_per_sm ? t->ctas_per_sm : 8;
  int64_t grid = (int64_t)sm_count() * cps;
  const int64_t need = (b.rows + (BLOCK / 32) - 1) / (BLOCK / 32);
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  int st = GBK_OK;
  char* scr = ws_scratch(w, sizeof(V) * (size_t)grid + 256, &st);
  if (!scr) return st;
  k_reduce_md<R, T, BLOCK><<<(unsigned)grid, BLOCK, 0, s>>>(base, b, (V*)scr, w->counters + SLOT_REDUCE, (V*)out);
  note_launch();
  return cuda_status(cudaGetLastError());
}

// Sum over doubles split between the FP64 and the integer pipes
// (gbk_sum_f64.cu); tuning variants 3 and 4.
int launch_sum_f64_split(const double* x, int64_t n, void* out, Workspace* w, const gbk_tuning_t* t);

// Dispatch over reducers for one element type.  A double Sum of 2^23
// elements and more takes the split kernel unless the tuning names variant
// 1 or 2 (measured: 2^24 31 us against 41 us, 2^28 6.8 against 4.1 TB/s;
// at 2^22 and below the two are within 10 %).
template <class T>
int reduce_typed(int op, const T* x, int64_t n, int64_t loc0, void* out, Workspace* w, const gbk_tuning_t* t) {
  constexpr bool INT = !(std::is_same<T, float>::value || std::is_same<T, double>::value);
  if constexpr (std::is_same<T, double>::value) {
    const int var = t ? t->variant : 0;
    if (op == GBK_SUM && n > 0 && (var == 3 || var == 4 || (var == 0 && n >= ((int64_t)1 << 23))))
      return launch_sum_f64_split(x, n, out, w, t);
  }
  switch (op) {
    case GBK_SUM: return launch_flat_cfg<RSum<T>, T>(x, n, loc0, out, w, t);
    case GBK_PROD: return launch_flat_cfg<RProd<T>, T>(x, n, loc0, out, w, t);
    case GBK_MIN: return launch_flat_cfg<RMin<T>, T>(x, n, loc0, out, w, t);
    case GBK_MAX: return launch_flat_cfg<RMax<T>, T>(x, n, loc0, out, w, t);
    case GBK_MINLOC: return launch_flat_cfg<RMinLoc<T>, T>(x, n, loc0, out, w, t);
    case GBK_MAXLOC: return launch_flat_cfg<RMaxLoc<T>, T>(x, n, loc0, out, w, t);
    case GBK_MINMAX: return launch_flat_cfg<RMinMax<T>, T>(x, n, loc0, out, w, t);
    case GBK_MINMAXLOC: return launch_flat_cfg<RMinMaxLoc<T>, T>(x, n, loc0, out, w, t);
    case GBK_MINMAXLOC_SUM: return launch_flat_cfg<RMinMaxLocSum<T>, T>(x, n, loc0, out, w, t);
    default: break;
  }
  if constexpr (INT) {
    switch (op) {
      case GBK_LAND: return launch_flat_cfg<RLAnd<T>, T>(x, n, loc0, out, w, t);
      case GBK_LOR: return launch_flat_cfg<RLOr<T>, T>(x, n, loc0, out, w, t);
      case GBK_BAND: return launch_flat_cfg<RBAnd<T>, T>(x, n, loc0, out, w, t);
      case GBK_BOR: return launch_flat_cfg<RBOr<T>, T>(x, n, loc0, out, w, t);
      default: break;
    }
  }
  return GBK_ERR_UNSUPPORTED;
}

template <class T>
int mdreduce_typed(int op, const T* base, const MDBox& b, void* out, Workspace* w, const gbk_tuning_t* t) {
  constexpr bool INT = !(std::is_same<T, float>::value || std::is_same<T, double>::value);
  switch (op) {
    case GBK_SUM: return launch_md<RSum<T>, T>(base, b, out, w, t);
    case GBK_PROD: return launch_md<RProd<T>, T>(base, b, out, w, t);
    case GBK_MIN: return launch_md<RMin<T>, T>(base, b, out, w, t);
    case GBK_MAX: return launch_md<RMax<T>, T>(base, b, out, w, t);
    case GBK_MINLOC: return launch_md<RMinLoc<T>, T>(base, b, out, w, t);
    case GBK_MAXLOC: return launch_md<RMaxLoc<T>, T>(base, b, out, w, t);
    case GBK_MINMAX: return launch_md<RMinMax<T>, T>(base, b, out, w, t);
    case GBK_MINMAXLOC: return launch_md<RMinMaxLoc<T>, T>(base, b, out, w, t);
    case GBK_MINMAXLOC_SUM: return launch_md<RMinMaxLocSum<T>, T>(base, b, out, w, t);
    default: break;
  }
  if constexpr (INT) {
    switch (op) {
      case GBK_LAND: return launch_md<RLAnd<T>, T>(base, b, out, w, t);
      case GBK_LOR: return launch_md<RLOr<T>, T>(base, b, out, w, t);
      case GBK_BAND: return launch_md<RBAnd<T>, T>(base, b, out, w, t);
      case GBK_BOR: return launch_md<RBOr<T>, T>(base, b, out, w, t);
      default: break;
    }
  }
  return GBK_ERR_UNSUPPORTED;
}

// Explicitly instantiated in gbk_reduce_<dtype>.cu.
extern template int reduce_typed<int32_t>(int, const int32_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
extern template int reduce_typed<int64_t>(int, const int64_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
extern template int reduce_typed<uint32_t>(int, const uint32_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
extern template int reduce_typed<uint64_t>(int, const uint64_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
extern template int reduce_typed<float>(int, const float*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
extern template int reduce_typed<double>(int, const double*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
extern template int mdreduce_typed<int32_t>(int, const int32_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
extern template int mdreduce_typed<int64_t>(int, const int64_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
extern template int mdreduce_typed<uint32_t>(int, const uint32_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
extern template int mdreduce_typed<uint64_t>(int, const uint64_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
extern template int mdreduce_typed<float>(int, const float*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
extern template int mdreduce_typed<double>(int, const double*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);

}  // namespace gbk
