/*
 * Seeded, deterministic host-side generators for the synthetic workloads of
 * the reduce / scan / scatter / sort path.
 *
 * Random bits: xoshiro256** (Blackman & Vigna, "Scrambled linear pseudorandom
 * number generators", 2018), its 256-bit state filled from splitmix64.  The
 * output is produced in blocks of GBKD_BLOCK elements; block b seeds its own
 * xoshiro state from splitmix64(seed + b * 0x9E3779B97F4A7C15), so the bytes
 * do not depend on how many host threads generate them.
 *
 * Distributions:
 *   uniform double in [0,1)   : (x >> 11) * 2^-53
 *   uniform integer in [lo,hi]: lo + (x >> 32) % (hi - lo + 1)
 *   N(0,1)                    : Box-Muller (u1 in (0,1], u2 in [0,1)),
 *                               one value per draw pair (the cosine branch)
 *   Zipf(s) over [0, nbins)   : inverse CDF over the normalised table of
 *                               k^-s, k = 1..nbins; key = rank - 1
 *   lognormal segment lengths : round(exp(mu + sigma * Z)) clipped to
 *                               [1, max_len]; sigma found by bisection so
 *                               the clipped total is near a target
 *   low-entropy u64 keys      : a seeded 64-bit base pattern with nbits
 *                               seeded bit positions re-drawn per key
 *
 * This file is plain C, compiled for the host only (no device code).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GBKD_BLOCK 65536

static inline uint64_t splitmix64_next(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

typedef struct {
  uint64_t s[4];
} xoshiro_t;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xoshiro_next(xoshiro_t* r) {
  uint64_t* s = r->s;
  const uint64_t result = rotl64(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return result;
}

static inline void xoshiro_seed(xoshiro_t* r, uint64_t seed, uint64_t stream) {
  uint64_t sm = seed + stream * 0x9E3779B97F4A7C15ull;
  for (int i = 0; i < 4; ++i) r->s[i] = splitmix64_next(&sm);
}

static inline double u01(xoshiro_t* r) { return (double)(xoshiro_next(r) >> 11) * 0x1.0p-53; }

static inline double normal01(xoshiro_t* r) {
  const double u1 = 1.0 - u01(r); /* (0,1] */
  const double u2 = u01(r);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925286766559 * u2);
}

#define GBKD_FOR_BLOCKS(n, ...)                                    \
  do {                                                             \
    const int64_t nblk_ = ((n) + GBKD_BLOCK - 1) / GBKD_BLOCK;     \
    _Pragma("omp parallel for schedule(static)")                   \
    for (int64_t b = 0; b < nblk_; ++b) {                          \
      xoshiro_t r;                                                 \
      xoshiro_seed(&r, seed, (uint64_t)b);                         \
      const int64_t lo = b * GBKD_BLOCK;                           \
      const int64_t hi = lo + GBKD_BLOCK < (n) ? lo + GBKD_BLOCK : (n); \
      for (int64_t i = lo; i < hi; ++i) { __VA_ARGS__; }           \
    }                                                              \
  } while (0)

void gbkd_uniform_f64(double* out, int64_t n, uint64_t seed) { GBKD_FOR_BLOCKS(n, out[i] = u01(&r)); }

void gbkd_uniform_f32(float* out, int64_t n, uint64_t seed) { GBKD_FOR_BLOCKS(n, out[i] = (float)u01(&r)); }

void gbkd_normal_f32(float* out, int64_t n, uint64_t seed) { GBKD_FOR_BLOCKS(n, out[i] = (float)normal01(&r)); }

void gbkd_normal_f64(double* out, int64_t n, uint64_t seed) { GBKD_FOR_BLOCKS(n, out[i] = normal01(&r)); }

void gbkd_uniform_i32(int32_t* out, int64_t n, int32_t lo_v, int32_t hi_v, uint64_t seed) {
  const uint64_t range = (uint64_t)((int64_t)hi_v - (int64_t)lo_v + 1);
  GBKD_FOR_BLOCKS(n, out[i] = (int32_t)((int64_t)lo_v + (int64_t)((xoshiro_next(&r) >> 32) % range)));
}

void gbkd_uniform_i64(int64_t* out, int64_t n, int64_t lo_v, int64_t hi_v, uint64_t seed) {
  const uint64_t range = (uint64_t)(hi_v - lo_v) + 1u;
  GBKD_FOR_BLOCKS(n, out[i] = range == 0 ? (int64_t)xoshiro_next(&r)
                                         : lo_v + (int64_t)(xoshiro_next(&r) % range));
}

void gbkd_bits_u64(uint64_t* out, int64_t n, uint64_t seed) { GBKD_FOR_BLOCKS(n, out[i] = xoshiro_next(&r)); }

void gbkd_bits_u32(uint32_t* out, int64_t n, uint64_t seed) {
  GBKD_FOR_BLOCKS(n, out[i] = (uint32_t)(xoshiro_next(&r) >> 32));
}

/* Zipf(s) keys over [0, nbins): inverse CDF by binary search in the
 * normalised cumulative table of k^-s. */
int gbkd_zipf_i32(int32_t* out, int64_t n, int32_t nbins, double s, uint64_t seed) {
  if (nbins <= 0) return 1;
  double* cdf = (double*)malloc(sizeof(double) * (size_t)nbins);
  if (!cdf) return 2;
  double acc = 0.0;
  for (int32_t k = 0; k < nbins; ++k) {
    acc += pow((double)(k + 1), -s);
    cdf[k] = acc;
  }
  for (int32_t k = 0; k < nbins; ++k) cdf[k] /= acc;
  cdf[nbins - 1] = 1.0;
  GBKD_FOR_BLOCKS(n, {
    const double u = u01(&r);
    int32_t lo = 0, hi = nbins - 1; /* first k with cdf[k] > u */
    while (lo < hi) {
      const int32_t mid = lo + (hi - lo) / 2;
      if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    out[i] = lo;
  });
  free(cdf);
  return 0;
}

/* Low-entropy u64 keys: a seeded base pattern with `nbits` distinct seeded
 * bit positions re-drawn for every key.  positions_out (may be NULL)
 * receives the chosen positions. */
int gbkd_lowentropy_u64(uint64_t* out, int64_t n, int nbits, uint64_t seed, int* positions_out) {
  if (nbits < 0 || nbits > 64) return 1;
  uint64_t sm = seed ^ 0xA5A5A5A5DEADBEEFull;
  const uint64_t base = splitmix64_next(&sm);
  int pos[64];
  int used[64];
  memset(used, 0, sizeof(used));
  for (int j = 0; j < nbits; ++j) {
    int p;
    do { p = (int)(splitmix64_next(&sm) % 64u); } while (used[p]);
    used[p] = 1;
    pos[j] = p;
    if (positions_out) positions_out[j] = p;
  }
  uint64_t mask = 0;
  for (int j = 0; j < nbits; ++j) mask |= 1ull << pos[j];
  GBKD_FOR_BLOCKS(n, {
    const uint64_t rb = xoshiro_next(&r);
    uint64_t k = base & ~mask;
    for (int j = 0; j < nbits; ++j) k |= ((rb >> j) & 1ull) << pos[j];
    out[i] = k;
  });
  return 0;
}

/* Lognormal segment lengths: len_i = clip(round(exp(mu + sigma Z_i)), 1,
 * max_len).  Z_i are drawn once (seeded); sigma is bisected in [0.01, 8] so
 * the clipped total is as close as bisection gets to `target_total`.  Writes
 * lengths to `len` and returns the chosen sigma through sigma_out. */
static int64_t seg_total(const double* z, int64_t nseg, double mu, double sigma, int64_t max_len) {
  int64_t tot = 0;
  for (int64_t i = 0; i < nseg; ++i) {
    double v = floor(exp(mu + sigma * z[i]) + 0.5);
    if (v < 1.0) v = 1.0;
    if (v > (double)max_len) v = (double)max_len;
    tot += (int64_t)v;
  }
  return tot;
}

int gbkd_lognormal_lengths(int64_t* len, int64_t nseg, double median, int64_t max_len, int64_t target_total,
                           uint64_t seed, double* sigma_out) {
  if (nseg <= 0 || median <= 0.0 || max_len <= 0) return 1;
  double* z = (double*)malloc(sizeof(double) * (size_t)nseg);
  if (!z) return 2;
  xoshiro_t r;
  xoshiro_seed(&r, seed, 0x5E6u);
  for (int64_t i = 0; i < nseg; ++i) z[i] = normal01(&r);
  const double mu = log(median);
  double lo = 0.01, hi = 8.0;
  for (int it = 0; it < 60; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (seg_total(z, nseg, mu, mid, max_len) < target_total) lo = mid; else hi = mid;
  }
  const double sigma = 0.5 * (lo + hi);
  for (int64_t i = 0; i < nseg; ++i) {
    double v = floor(exp(mu + sigma * z[i]) + 0.5);
    if (v < 1.0) v = 1.0;
    if (v > (double)max_len) v = (double)max_len;
    len[i] = (int64_t)v;
  }
  if (sigma_out) *sigma_out = sigma;
  free(z);
  return 0;
}

void gbkd_iota_i32(int32_t* out, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) out[i] = (int32_t)i;
}
