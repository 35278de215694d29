// Sum over doubles with the adds split between the FP64 pipe and the
// integer pipes (the Sum<double> of a RangePolicy parallel_reduce /
// std::reduce over a contiguous View<double*>: core/src/Kokkos_Parallel_Reduce.hpp:1496-1560,
// reducer core/src/Kokkos_Parallel_Reduce.hpp:34, default std::reduce functor
// algorithms/src/std_algorithms/impl/Kokkos_Reduce.hpp:31-41).
//
// GB300 adds about 1.2 doubles per SM clock on its FP64 pipe while HBM
// delivers about 2.7, so the plain fold is FP64-bound.  Here each thread's
// tile of UNROLL 16-byte vectors sends FPV vectors to two FP64 accumulators
// and the other UNROLL - FPV to the fixed-point accumulator of
// gbk_fixsum.cuh (exact integer adds, folded into FP64 with one rounding
// at least every 2^14 elements and at the end).  Every thread's value is a
// double again before the warp, CTA and grid trees, which are those of the
// flat reduce (last-CTA finish, one launch, deterministic for a given
// grid).  Nothing is computed in less than FP64 precision: the integer part
// is exact up to far below a double's rounding, so the result is at least
// as accurate as the all-FP64 fold.
#include "gbk_fixsum.cuh"
#include "gbk_reduce_impl.cuh"

namespace gbk {
namespace {

constexpr int FIX_FLUSH = 1 << 14;  // integer-path elements per thread between folds (< 2^(FIX_H - 1))

template <int BLOCK, int UNROLL, int FPV>
__global__ void __launch_bounds__(BLOCK)
    k_sum_f64_split(const double* __restrict__ x, int64_t n, int64_t head, double* partials, unsigned* counter,
                    double* out) {
  static_assert(FPV >= 0 && FPV < UNROLL, "at least one vector per tile on the integer pipes");
  constexpr int IPI = 2 * (UNROLL - FPV);  // integer-path elements per tile
  __shared__ double sm[BLOCK / 32];
  double fa = 0.0, fb = 0.0;
  FixAcc a;
  fix_init(a);
  const int64_t gtid = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  pdl_entry();
  if (gtid < head) fa += x[gtid];  // unaligned head: one element per thread
  const double* xb = x + head;
  const int64_t nvec = (n - head) / 2;
  constexpr int64_t TILE = (int64_t)BLOCK * UNROLL;
  const int64_t per = nvec / gridDim.x, rem = nvec % gridDim.x;
  const int64_t v0 = (int64_t)blockIdx.x * per + ((int64_t)blockIdx.x < rem ? blockIdx.x : rem);
  const int64_t v1 = v0 + per + ((int64_t)blockIdx.x < rem ? 1 : 0);
  int64_t vb = v0 + threadIdx.x;
  bool have = vb + (int64_t)(UNROLL - 1) * BLOCK < v1;
  uint4 cur[UNROLL], nxt[UNROLL];
  if (have) {
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = ld_stream16(xb + (vb + (int64_t)u * BLOCK) * 2);
  }
  int since = 0;
  while (have) {
    const int64_t vn = vb + TILE;
    const bool hn = vn + (int64_t)(UNROLL - 1) * BLOCK < v1;
    if (hn) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) nxt[u] = ld_stream16(xb + (vn + (int64_t)u * BLOCK) * 2);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const uint64_t b0 = ((uint64_t)cur[u].y << 32) | cur[u].x;
      const uint64_t b1 = ((uint64_t)cur[u].w << 32) | cur[u].z;
      if (u < FPV) {
        fa += __longlong_as_double((long long)b0);
        fb += __longlong_as_double((long long)b1);
      } else {
        fix_add2(a, fa, b0, b1);
      }
    }
    since += IPI;
    if (since >= FIX_FLUSH) {
      fb += fix_to_double(a);
      since = 0;
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) cur[u] = nxt[u];
    vb = vn;
    have = hn;
  }
  for (; vb < v1; vb += BLOCK) {  // fewer than UNROLL vectors left for this thread
    const uint4 v = ld_stream16(xb + vb * 2);
    fix_add2(a, fa, ((uint64_t)v.y << 32) | v.x, ((uint64_t)v.w << 32) | v.z);
  }
  const int64_t t0 = head + nvec * 2;
  if (t0 + gtid < n) fb += x[t0 + gtid];  // the odd last element
  const double acc = fa + fb + fix_to_double(a);
  grid_finish<RSum<double>, BLOCK>(acc, partials, counter, out, sm);
}

template <int UNROLL, int FPV>
int launch_split(const double* x, int64_t n, double* out, Workspace* w, int ctas_per_sm) {
  constexpr int BLOCK = 256;
  auto kfn = k_sum_f64_split<BLOCK, UNROLL, FPV>;
  static std::atomic<int> resident{0};  // CTAs per SM, per instantiation (set once, any host thread)
  if (!resident) {
    int r = 0;
    GBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kfn, BLOCK, 0));
    resident = r > 0 ? r : 1;
  }
  const int per_sm = ctas_per_sm > 0 && ctas_per_sm < resident ? ctas_per_sm : resident.load();
  const uintptr_t a = (uintptr_t)x;
  int64_t head = (int64_t)(((16 - (a & 15)) & 15) / sizeof(double));
  if (head > n) head = n;
  const int64_t nvec = (n - head) / 2;
  const int64_t tiles = (nvec + (int64_t)BLOCK * UNROLL - 1) / ((int64_t)BLOCK * UNROLL);
  int64_t grid = (int64_t)sm_count() * per_sm;
  if (grid > tiles) grid = tiles;
  if (grid < 1) grid = 1;
  int st = GBK_OK;
  char* scr = ws_scratch(w, sizeof(double) * (size_t)grid + 256, &st);
  if (!scr) return st;
  GBK_CUDA_TRY(launch_pdl(kfn, dim3((unsigned)grid), dim3(BLOCK), 0, w->stream, x, n, head, (double*)scr,
                          w->counters + SLOT_REDUCE, out));
  note_launch();
  return GBK_OK;
}

}  // namespace

// Variant 3: items_per_thread 3, 4, 5 (default) or 6 vectors per tile, of
// which 1, 1, 2, 2 go to the FP64 pipe; variant 4: all vectors on the
// integer pipes (4 per tile).  Measured over uniform doubles (us, default
// CTAs per SM): 2^24: 32.8 / 31.7 / 31.1 / 30.9, all-integer 35.0;
// 2^28: 324.8 / 324.4 / 315.6 / 317.7, all-integer 394.3 - both pipes
// together beat either alone.
int launch_sum_f64_split(const double* x, int64_t n, void* out, Workspace* w, const gbk_tuning_t* t) {
  double* o = static_cast<double*>(out);
  const int cps = t ? t->ctas_per_sm : 0;
  if (t && t->variant == 4) return launch_split<4, 0>(x, n, o, w, cps);
  switch (t ? t->items_per_thread : 0) {
    case 3: return launch_split<3, 1>(x, n, o, w, cps);
    case 4: return launch_split<4, 1>(x, n, o, w, cps);
    case 6: return launch_split<6, 2>(x, n, o, w, cps);
    default: return launch_split<5, 2>(x, n, o, w, cps);
  }
}

}  // namespace gbk
