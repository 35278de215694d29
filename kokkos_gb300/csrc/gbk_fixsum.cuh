// Fixed-point accumulation of doubles on the integer pipes.
//
// GB300 issues few FP64 additions per SM clock (about 1.2 measured), fewer
// than the HBM delivers doubles (about 2.7 per SM clock), so a Sum over
// doubles folded with DADD alone is FP64-bound at under half of the HBM
// rate.  This accumulator adds doubles exactly, as integers: each thread
// keeps a signed 128-bit fixed-point value A in units of
// 2^(R - 1075 - FIX_F), where R is the largest biased exponent the thread
// has seen so far.  A double with biased exponent e <= R and 53-bit
// significand M adds M * 2^(e - R + FIX_F): exactly when R - e <= FIX_F,
// otherwise truncated below 2^-FIX_F of the unit in the last place of the
// largest element (a loss far below FP64's own rounding).  FIX_H = 127 - 53
// - FIX_F bits of headroom take 2^FIX_H elements of the largest exponent;
// the caller folds A into an FP64 value (fix_to_double, one rounding) at
// least every 2^(FIX_H - 1) elements.  A larger exponent arrives rarely
// (once the thread has seen its largest elements): A is shifted right to
// the new unit.  Infinities and NaNs are not representable and go to the
// caller's FP64 accumulator, which keeps IEEE semantics for them.
//
// Negation: -v = ~v + 1 in two's complement; the kernel adds ~v and counts
// the negatives, whose +1s are added when A is folded or rescaled.
//
// The functions are host/device so the arithmetic can be checked on the
// CPU against exact sums.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

namespace gbk {

constexpr int FIX_F = 58;  // fraction bits below the significand's last bit at exponent R
constexpr int FIX_H = 127 - 53 - FIX_F;  // headroom bits (16)

struct FixAcc {
  uint64_t lo, hi;  // signed 128-bit two's complement
  uint64_t nneg;    // negatives added since the last fold (their +1s)
  int R;            // reference biased exponent, >= 1
};

__host__ __device__ __forceinline__ void fix_init(FixAcc& a) {
  a.lo = 0;
  a.hi = 0;
  a.nneg = 0;
  a.R = 1;
}

__host__ __device__ __forceinline__ void add128(uint64_t& lo, uint64_t& hi, uint64_t alo, uint64_t ahi) {
#ifdef __CUDA_ARCH__
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(alo), "l"(ahi));
#else
  const uint64_t s = lo + alo;
  hi = hi + ahi + (s < lo ? 1u : 0u);
  lo = s;
#endif
}

// Logical shifts that give 0 for amounts of 64 and more (amounts are taken
// as unsigned, so negative amounts give 0 too) - the PTX semantics.
__host__ __device__ __forceinline__ uint64_t shl_c(uint64_t x, int s) {
#ifdef __CUDA_ARCH__
  uint64_t r;
  asm("shl.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
#else
  return (unsigned)s >= 64u ? 0 : x << s;
#endif
}
__host__ __device__ __forceinline__ uint64_t shr_c(uint64_t x, int s) {
#ifdef __CUDA_ARCH__
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
#else
  return (unsigned)s >= 64u ? 0 : x >> s;
#endif
}

__host__ __device__ __forceinline__ double fix_bits_to_double(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}

__host__ __device__ __forceinline__ int fix_exp(uint64_t bits) { return (int)(bits >> 52) & 0x7ff; }

// Add the finite double with bit pattern `bits` and biased exponent e <= a.R.
__host__ __device__ __forceinline__ void fix_add(FixAcc& a, uint64_t bits, int e) {
  const uint64_t M = (bits & 0xFFFFFFFFFFFFFull) | ((uint64_t)(e != 0) << 52);
  const int ee = e > 1 ? e : 1;  // subnormals have the exponent of the smallest normals
  // value = (M << 64) >> t as 128 bits, t = 64 - (FIX_F - (R - ee)) >= 64 - FIX_F
  const int t = (64 - FIX_F) + (a.R - ee);
  const uint64_t vhi = shr_c(M, t);
  const uint64_t vlo = shl_c(M, 64 - t) | shr_c(M, t - 64);
  const uint64_t m = (uint64_t)((int64_t)bits >> 63);  // all ones for a negative value
  add128(a.lo, a.hi, vlo ^ m, vhi ^ m);
  a.nneg += bits >> 63;
}

__host__ __device__ __forceinline__ void fix_fold_neg(FixAcc& a) {
  add128(a.lo, a.hi, a.nneg, 0);
  a.nneg = 0;
}

// Make e (> a.R) the reference exponent: A shifted right (arithmetic) by e - R.
__host__ __device__ __forceinline__ void fix_rescale(FixAcc& a, int e) {
  fix_fold_neg(a);
  int d = e - a.R;
  if (d > 127) d = 127;
  const int64_t h = (int64_t)a.hi;
  if (d >= 64) {
    a.lo = (uint64_t)(h >> (d - 64));
    a.hi = (uint64_t)(h >> 63);
  } else if (d > 0) {
    a.lo = (a.lo >> d) | ((uint64_t)h << (64 - d));
    a.hi = (uint64_t)(h >> d);
  }
  a.R = e;
}

// Add two doubles (one 16-byte vector).  Non-finite values go to the FP64
// accumulator `f`; a larger exponent rescales A first.
__host__ __device__ __forceinline__ void fix_add2(FixAcc& a, double& f, uint64_t b0, uint64_t b1) {
  int e0 = fix_exp(b0), e1 = fix_exp(b1);
  if ((e0 > e1 ? e0 : e1) > a.R) {  // rare once the thread has seen its largest exponent
    if (e0 == 0x7ff) {
      f += fix_bits_to_double(b0);
      b0 = 0;
      e0 = 0;
    }
    if (e1 == 0x7ff) {
      f += fix_bits_to_double(b1);
      b1 = 0;
      e1 = 0;
    }
    const int em = e0 > e1 ? e0 : e1;
    if (em > a.R) fix_rescale(a, em);
  }
  fix_add(a, b0, e0);
  fix_add(a, b1, e1);
}

// The accumulated value, rounded once to the nearest double; A is cleared
// (R is kept).
__host__ __device__ __forceinline__ double fix_to_double(FixAcc& a) {
  fix_fold_neg(a);
  uint64_t lo = a.lo, hi = a.hi;
  a.lo = 0;
  a.hi = 0;
  const bool neg = (int64_t)hi < 0;
  if (neg) {  // magnitude
    lo = ~lo + 1;
    hi = ~hi + (lo == 0 ? 1u : 0u);
  }
  if ((hi | lo) == 0) return 0.0;
#ifdef __CUDA_ARCH__
  const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
#else
  const int lz = hi ? __builtin_clzll(hi) : 64 + __builtin_clzll(lo);
#endif
  uint64_t top, rest;
  if (lz == 0) {
    top = hi;
    rest = lo;
  } else if (lz < 64) {
    top = (hi << lz) | (lo >> (64 - lz));
    rest = lo << lz;
  } else {
    top = lo << (lz - 64);
    rest = 0;
  }
  top |= rest != 0 ? 1u : 0u;  // sticky bit: the 64 -> 53-bit conversion rounds as the full value would
#ifdef __CUDA_ARCH__
  const double d = __ull2double_rn(top);
#else
  const double d = (double)top;  // round-to-nearest-even on IEEE hosts
#endif
  // magnitude = top * 2^(64 - lz) (up to the sticky bit), unit = 2^(R - 1075 - FIX_F)
  const double v = ldexp(d, 64 - lz + a.R - 1075 - FIX_F);
  return neg ? -v : v;
}

}  // namespace gbk
