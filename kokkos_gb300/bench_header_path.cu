// Throughput of the header-template path (include/Kokkos_GB300.hpp) for user
// functors, beside the library's typed entry points on the same data (used
// by bench.py's other_configs; prints one JSON line).  CUDA events around
// `reps` back-to-back calls after 3 warm-up calls, inputs alternating over two
// copies (each copy is at least 128 MiB, so a call starts with most of its
// input out of the 129 MB L2):
//   range_sum_f64:   parallel_reduce(RangePolicy(0, 2^24), x(i) summed) vs gbk_reduce
//   mdrange_sum_f32: parallel_reduce(MDRangePolicy<Rank<3>> over a LayoutLeft
//                    512x512x256 float view) vs gbk_mdrange_reduce
//   team_sum_f32:    TeamPolicy league, one team per segment, TeamThreadRange
//                    reduce, single(PerTeam) store, over the lognormal
//                    segments whose int64 offsets are in argv[1]; vs
//                    gbk_segmented_reduce
//   umap_insert_u32: UnorderedMap<uint32_t, uint32_t> AtomicAdd inserts of
//                    2^24 keys drawn from 2^23 values (table of 2^24 slots,
//                    emptied before each call), then a find of each key;
//                    the size is checked against the distinct keys counted
//                    on the host
//   bitset_set:      Bitset of 2^27 bits, 2^24 set() calls at hashed bits
//   bench_header_path <offsets.bin> <nseg> <reps>
#include <Kokkos_GB300.hpp>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

// keys of the UnorderedMap and Bitset runs (splitmix64 finaliser of i)
__host__ __device__ inline uint32_t bench_key(uint64_t i, uint32_t mask) {
  uint64_t z = i + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return (uint32_t)(z ^ (z >> 31)) & mask;
}

template <class F>
static double time_us(int reps, F&& f) {
  for (int r = 0; r < 3; ++r) f(r);
  cudaDeviceSynchronize();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, nullptr);
  for (int r = 0; r < reps; ++r) f(r);
  cudaEventRecord(b, nullptr);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return 1000.0 * ms / reps;
}

int main(int argc, char** argv) {
  if (argc < 4) return 1;
  const int64_t nseg = std::atoll(argv[2]);
  const int reps = std::atoi(argv[3]);
  std::vector<int64_t> offs(nseg + 1);
  FILE* fo = std::fopen(argv[1], "rb");
  if (!fo || std::fread(offs.data(), 8, offs.size(), fo) != offs.size()) return 2;
  std::fclose(fo);
  Kokkos::initialize();
  {
    Kokkos::Experimental::GB300 ex;
    cudaStream_t s = ex.stream();
    // ---- RangePolicy Sum over 2^24 doubles -------------------------------
    const int64_t n = 1 << 24;
    Kokkos::View<double*> x0("x0", n), x1("x1", n);
    Kokkos::parallel_for(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i) {
      x0(i) = (double)((i * 2654435761u) % 1000) * 1e-3;
      x1(i) = (double)((i * 40503u) % 1000) * 1e-3;
    });
    double sum = 0;
    const double t_range = time_us(reps, [&](int r) {
      const Kokkos::View<double*>& x = (r & 1) ? x1 : x0;
      Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, double& u) { u += x(i); }, sum);
    });
    Kokkos::View<double> dres("dres");
    const double t_range_lib = time_us(reps, [&](int r) {
      const Kokkos::View<double*>& x = (r & 1) ? x1 : x0;
      gbk_reduce(GBK_SUM, GBK_F64, x.data(), n, dres.data(), (gbk_stream_t)s, nullptr);
    });
    // the same through a View result (no host fence per call)
    const double t_range_dev = time_us(reps, [&](int r) {
      const Kokkos::View<double*>& x = (r & 1) ? x1 : x0;
      Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, double& u) { u += x(i); },
                              Kokkos::Sum<double>(dres));
    });
    // ---- MDRange Sum over a 512x512x256 float box --------------------------
    const int64_t n0 = 512, n1 = 512, n2 = 256;
    Kokkos::View<float***, Kokkos::LayoutLeft> b0("b0", n0, n1, n2), b1("b1", n0, n1, n2);
    Kokkos::parallel_for(Kokkos::MDRangePolicy<Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                         KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k) {
                           b0(i, j, k) = (float)((i + j + k) % 7);
                           b1(i, j, k) = (float)((i * 3 + j + k) % 5);
                         });
    Kokkos::View<float> fres("fres");
    const double t_md = time_us(reps, [&](int r) {
      const auto& b = (r & 1) ? b1 : b0;
      Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                              KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, float& u) { u += b(i, j, k); },
                              Kokkos::Sum<float>(fres));
    });
    const int64_t lo[3] = {0, 0, 0}, up[3] = {n0, n1, n2}, st[3] = {1, n0, n0 * n1};
    const double t_md_lib = time_us(reps, [&](int r) {
      const auto& b = (r & 1) ? b1 : b0;
      gbk_mdrange_reduce(GBK_SUM, GBK_F32, b.data(), 3, lo, up, st, fres.data(), (gbk_stream_t)s, nullptr);
    });
    // ---- TeamPolicy league reduce over lognormal segments ------------------
    const int64_t ns = offs[nseg];
    Kokkos::View<int64_t*> doff("doff", nseg + 1);
    Kokkos::View<int64_t*, Kokkos::HostSpace> hoff(offs.data(), nseg + 1);
    Kokkos::deep_copy(doff, hoff);
    Kokkos::View<float*> v("v", ns), segs("segs", nseg);
    Kokkos::parallel_for(Kokkos::RangePolicy<>(0, ns), KOKKOS_LAMBDA(int64_t i) { v(i) = (float)(i % 11); });
    using TP = Kokkos::TeamPolicy<>;
    const double t_team = time_us(reps, [&](int) {
      Kokkos::parallel_for(TP((int)nseg, 256), KOKKOS_LAMBDA(const TP::member_type& t) {
        const int64_t sg = t.league_rank();
        float u = 0;
        Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, doff(sg), doff(sg + 1)),
                                [&](int64_t i, float& w) { w += v(i); }, u);
        Kokkos::single(Kokkos::PerTeam(t), [&]() { segs(sg) = u; });
      });
    });
    const double t_team_lib = time_us(reps, [&](int) {
      gbk_segmented_reduce(GBK_SUM, GBK_F32, v.data(), doff.data(), nseg, ns, segs.data(), (gbk_stream_t)s, nullptr);
    });
    // ---- UnorderedMap inserts and finds, Bitset sets ---------------------
    const uint32_t nk = 1u << 24, nu = 1u << 23;
    Kokkos::View<uint32_t*> ks("ks", nk), fidx("fidx", nk);
    Kokkos::parallel_for(Kokkos::RangePolicy<>(0, (int64_t)nk),
                         KOKKOS_LAMBDA(int64_t i) { ks(i) = bench_key((uint64_t)i, nu - 1); });
    Kokkos::UnorderedMap<uint32_t, uint32_t> map(nu);
    using AddOp = Kokkos::UnorderedMapInsertOpTypes<Kokkos::View<uint32_t*>, uint32_t>::AtomicAdd;
    cudaEvent_t ea, eb;
    cudaEventCreate(&ea);
    cudaEventCreate(&eb);
    double t_ins = 0;
    for (int r = 0; r < 3 + reps; ++r) {
      map.clear();
      cudaDeviceSynchronize();
      cudaEventRecord(ea, nullptr);
      Kokkos::parallel_for(Kokkos::RangePolicy<>(0, (int64_t)nk),
                           KOKKOS_LAMBDA(int64_t i) { map.insert(ks(i), 1u, AddOp()); });
      cudaEventRecord(eb, nullptr);
      cudaEventSynchronize(eb);
      float ms = 0;
      cudaEventElapsedTime(&ms, ea, eb);
      if (r >= 3) t_ins += 1000.0 * ms / reps;
    }
    const double t_find = time_us(reps, [&](int) {
      Kokkos::parallel_for(Kokkos::RangePolicy<>(0, (int64_t)nk), KOKKOS_LAMBDA(int64_t i) { fidx(i) = map.find(ks(i)); });
    });
    std::vector<uint32_t> hk(nk);
    for (uint32_t i = 0; i < nk; ++i) hk[i] = bench_key(i, nu - 1);
    std::sort(hk.begin(), hk.end());
    const uint32_t distinct = (uint32_t)(std::unique(hk.begin(), hk.end()) - hk.begin());
    int64_t missing = 0;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, (int64_t)nk), KOKKOS_LAMBDA(int64_t i, int64_t& u) {
      u += (map.valid_at(fidx(i)) && map.key_at(fidx(i)) == ks(i)) ? 0 : 1;
    }, missing);
    const bool map_ok = map.size() == distinct && !map.failed_insert() && missing == 0;
    const unsigned nbits = 1u << 27;
    Kokkos::Bitset<> bits(nbits);
    double t_bits = 0;
    for (int r = 0; r < 3 + reps; ++r) {
      bits.reset();
      cudaDeviceSynchronize();
      cudaEventRecord(ea, nullptr);
      Kokkos::parallel_for(Kokkos::RangePolicy<>(0, (int64_t)nk),
                           KOKKOS_LAMBDA(int64_t i) { bits.set(bench_key((uint64_t)i + 77, nbits - 1)); });
      cudaEventRecord(eb, nullptr);
      cudaEventSynchronize(eb);
      float ms = 0;
      cudaEventElapsedTime(&ms, ea, eb);
      if (r >= 3) t_bits += 1000.0 * ms / reps;
    }
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
    ex.fence();
    auto gbs = [](double bytes, double us) { return bytes / (us * 1e-6) / 1e9; };
    const double rb = (double)n * 8, mb = (double)n0 * n1 * n2 * 4, tb = (double)ns * 4 + (nseg + 1) * 8.0 + nseg * 4.0;
    std::printf(
        "{\"range_sum_f64_2^24\": {\"us\": %.2f, \"GB/s\": %.1f, \"view_result_us\": %.2f, \"library_us\": %.2f, "
        "\"library_GB/s\": %.1f}, "
        "\"mdrange_sum_f32_512x512x256\": {\"us\": %.2f, \"GB/s\": %.1f, \"library_us\": %.2f, \"library_GB/s\": %.1f}, "
        "\"team_sum_f32_lognormal_segments\": {\"segments\": %lld, \"elements\": %lld, \"us\": %.2f, \"GB/s\": %.1f, "
        "\"library_us\": %.2f, \"library_GB/s\": %.1f}, "
        "\"umap_insert_u32\": {\"inserts\": %u, \"distinct\": %u, \"capacity\": %u, \"insert_us\": %.2f, "
        "\"G_inserts_per_s\": %.3f, \"find_us\": %.2f, \"G_finds_per_s\": %.3f, \"ok\": %s}, "
        "\"bitset_set\": {\"bits\": %u, \"sets\": %u, \"us\": %.2f, \"G_sets_per_s\": %.3f}}\n",
        t_range, gbs(rb, t_range), t_range_dev, t_range_lib, gbs(rb, t_range_lib), t_md, gbs(mb, t_md), t_md_lib,
        gbs(mb, t_md_lib), (long long)nseg, (long long)ns, t_team, gbs(tb, t_team), t_team_lib, gbs(tb, t_team_lib),
        nk, distinct, map.capacity(), t_ins, nk / t_ins * 1e-3, t_find, nk / t_find * 1e-3, map_ok ? "true" : "false",
        nbits, nk, t_bits, nk / t_bits * 1e-3);
  }
  Kokkos::finalize();
  return 0;
}
