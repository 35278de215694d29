// Host driver for the fixed-point double accumulator of
// kokkos_gb300/csrc/gbk_fixsum.cuh (the arithmetic of the split Sum kernel).
// Reads doubles from stdin; each run of `per` values is summed the way one
// kernel thread sums its share: pairs through fix_add2, a fold into FP64
// every 2^14 values, an odd last value added in FP64, then the per-run
// results added in FP64.  Prints the sum with 17 significant digits.
#define __host__
#define __device__
#define __forceinline__ inline
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../kokkos_gb300/csrc/gbk_fixsum.cuh"

int main(int argc, char** argv) {
  const long per = argc > 1 ? atol(argv[1]) : 1L << 40;
  std::vector<double> x;
  double v;
  while (fread(&v, sizeof v, 1, stdin) == 1) x.push_back(v);
  double total = 0;
  for (size_t s = 0; s < x.size(); s += per) {
    gbk::FixAcc a;
    gbk::fix_init(a);
    double f = 0;
    long since = 0;
    const size_t e = s + per < x.size() ? s + per : x.size();
    size_t i = s;
    for (; i + 1 < e; i += 2) {
      uint64_t b0, b1;
      memcpy(&b0, &x[i], 8);
      memcpy(&b1, &x[i + 1], 8);
      gbk::fix_add2(a, f, b0, b1);
      if ((since += 2) >= (1 << 14)) {
        f += gbk::fix_to_double(a);
        since = 0;
      }
    }
    if (i < e) f += x[i];
    total += f + gbk::fix_to_double(a);
  }
  printf("%.17g\n", total);
  return 0;
}
