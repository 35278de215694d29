// Throughput of the reference's own Kokkos API on the GB300 execution space
// (the backend in include/gb300_backend, built by tests/backend/Makefile):
// plain Kokkos user code, timed with CUDA events on the instance's stream
// after 3 warm-up calls, inputs alternating over two copies of at least
// 128 MiB each (a call starts with most of its input out of the 129 MB L2).
// Prints one JSON line.
//   range_sum_f64:   parallel_reduce(RangePolicy<GB300>(0, 2^24), x(i) summed)
//                    into a host double and into a device View
//   mdrange_sum_f32: parallel_reduce(MDRangePolicy<GB300, Rank<3>> over a
//                    LayoutLeft 512x512x256 float View, Sum into a View)
//   team_sum_f32:    TeamPolicy<GB300>(segments, 256), TeamThreadRange reduce
//                    per league rank over the lognormal segments whose int64
//                    offsets are in argv[1], single(PerTeam) store
//   scatter_hist:    ScatterView (defaults: non-duplicated, atomic) histogram
//                    of 2^26 int32 keys (x * 2654435761 mod 2^16) into 2^16
//                    int64 bins, contribute; and the same with log-uniform keys
//                    (exp2(16 u) - 1: a few bins take most of them)
//   sort_u64:        Kokkos::sort of 2^27 uint64 keys (refilled each call)
//   graph:           Experimental::Graph of 8 dependent parallel_for nodes over
//                    2^16 int64 (y = x + 1) submitted, against the same 8
//                    parallel_for launched directly
//   umap_insert_u32: Kokkos::UnorderedMap<uint32_t, uint32_t, GB300> AtomicAdd
//                    inserts of 2^24 keys drawn from 2^23 values (the map
//                    emptied before each call), then a find of each key; the
//                    size is checked against the distinct keys counted on the
//                    host
//   backend_bench <offsets.bin> <nseg> <reps>
#include <Kokkos_Core.hpp>
#include <Kokkos_ScatterView.hpp>
#include <Kokkos_Sort.hpp>
#include <Kokkos_Graph.hpp>
#include <Kokkos_UnorderedMap.hpp>
#include <GB300/Kokkos_GB300_Graph_Impl.hpp>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

using ES = Kokkos::Experimental::GB300;
using MS = Kokkos::Experimental::GB300Space;

// graph nodes: y = x + 1, chained (functors: no extended lambda inside the
// generic lambda that builds the graph)
struct AddOne {
  Kokkos::View<int64_t*, MS> x, y;
  KOKKOS_INLINE_FUNCTION void operator()(int64_t i) const { y(i) = x(i) + 1; }
};

// keys of the UnorderedMap run (splitmix64 finaliser of i)
KOKKOS_INLINE_FUNCTION uint32_t bench_key(uint64_t i, uint32_t mask) {
  uint64_t z = i + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return (uint32_t)(z ^ (z >> 31)) & mask;
}

template <class F>
static double time_us(const ES& ex, int reps, F&& f) {
  for (int r = 0; r < 3; ++r) f(r);
  ex.fence();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, ex.stream());
  for (int r = 0; r < reps; ++r) f(r);
  cudaEventRecord(b, ex.stream());
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
  Kokkos::initialize(argc, argv);
  {
    ES ex;
    auto gbs = [](double bytes, double us) { return bytes / (us * 1e-6) / 1e9; };
    // ---- RangePolicy Sum over 2^24 doubles -------------------------------
    const int64_t n = 1 << 24;
    Kokkos::View<double*, MS> x0("x0", n), x1("x1", n);
    Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, n), KOKKOS_LAMBDA(int64_t i) {
      x0(i) = (double)((i * 2654435761u) % 1000) * 1e-3;
      x1(i) = (double)((i * 40503u) % 1000) * 1e-3;
    });
    double hsum = 0;
    const double t_range_host = time_us(ex, reps, [&](int r) {
      auto x = (r & 1) ? x1 : x0;
      Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(ex, 0, n), KOKKOS_LAMBDA(int64_t i, double& u) { u += x(i); },
                              hsum);
    });
    Kokkos::View<double, MS> dsum("dsum");
    const double t_range_dev = time_us(ex, reps, [&](int r) {
      auto x = (r & 1) ? x1 : x0;
      Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(ex, 0, n), KOKKOS_LAMBDA(int64_t i, double& u) { u += x(i); },
                              dsum);
    });
    // ---- MDRange Sum over a 512x512x256 float box --------------------------
    const int64_t n0 = 512, n1 = 512, n2 = 256;
    Kokkos::View<float***, Kokkos::LayoutLeft, MS> b0("b0", n0, n1, n2), b1("b1", n0, n1, n2);
    using MD = Kokkos::MDRangePolicy<ES, Kokkos::Rank<3>>;
    Kokkos::parallel_for(MD(ex, {0, 0, 0}, {n0, n1, n2}), KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k) {
      b0(i, j, k) = (float)((i + j + k) % 7);
      b1(i, j, k) = (float)((i * 3 + j + k) % 5);
    });
    Kokkos::View<float, MS> fsum("fsum");
    const double t_md = time_us(ex, reps, [&](int r) {
      auto b = (r & 1) ? b1 : b0;
      Kokkos::parallel_reduce(MD(ex, {0, 0, 0}, {n0, n1, n2}),
                              KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, float& u) { u += b(i, j, k); }, fsum);
    });
    // ---- TeamPolicy league reduce over lognormal segments ------------------
    const int64_t ns = offs[nseg];
    Kokkos::View<int64_t*, MS> doff("doff", nseg + 1);
    Kokkos::View<int64_t*, Kokkos::HostSpace> hoff(offs.data(), nseg + 1);
    Kokkos::deep_copy(ex, doff, hoff);
    Kokkos::View<float*, MS> v("v", ns), segs("segs", nseg);
    Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, ns), KOKKOS_LAMBDA(int64_t i) { v(i) = (float)(i % 11); });
    using TP = Kokkos::TeamPolicy<ES>;
    const double t_team = time_us(ex, reps, [&](int) {
      Kokkos::parallel_for(TP(ex, (int)nseg, 256), KOKKOS_LAMBDA(const TP::member_type& t) {
        const int64_t sg = t.league_rank();
        float u = 0;
        Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, doff(sg), doff(sg + 1)),
                                [&](int64_t i, float& w) { w += v(i); }, u);
        Kokkos::single(Kokkos::PerTeam(t), [&]() { segs(sg) = u; });
      });
    });
    // ---- ScatterView histogram -------------------------------------------
    const int64_t nk = 1 << 26, nb = 1 << 16;
    Kokkos::View<int32_t*, MS> keys("keys", nk);
    Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, nk), KOKKOS_LAMBDA(int64_t i) {
      keys(i) = (int32_t)(((uint64_t)i * 2654435761ull) & (uint64_t)(nb - 1));
    });
    Kokkos::View<int64_t*, MS> bins("bins", nb);
    const double t_hist = time_us(ex, reps, [&](int) {
      auto sv = Kokkos::Experimental::create_scatter_view(bins);
      Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, nk), KOKKOS_LAMBDA(int64_t i) {
        auto a = sv.access();
        a(keys(i)) += 1;
      });
      Kokkos::Experimental::contribute(bins, sv);
    });
    // skewed keys: log-uniform over the bins (a few bins take most keys)
    Kokkos::View<int32_t*, MS> skeys("skeys", nk);
    Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, nk), KOKKOS_LAMBDA(int64_t i) {
      const double u = (double)(((uint64_t)i * 0x9E3779B97F4A7C15ull) >> 11) * (1.0 / 9007199254740992.0);
      const int64_t k = (int64_t)exp2(u * 16.0) - 1;
      skeys(i) = (int32_t)(k < nb ? k : nb - 1);
    });
    const double t_hist_skew = time_us(ex, reps, [&](int) {
      auto sv = Kokkos::Experimental::create_scatter_view(bins);
      Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, nk), KOKKOS_LAMBDA(int64_t i) {
        auto a = sv.access();
        a(skeys(i)) += 1;
      });
      Kokkos::Experimental::contribute(bins, sv);
    });
    // ---- Kokkos::sort of 2^27 uint64 keys -----------------------------------
    const int64_t nsort = 1 << 27;
    Kokkos::View<uint64_t*, MS> sk("sk", nsort);
    auto fill = [&](int r) {
      Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, nsort), KOKKOS_LAMBDA(int64_t i) {
        uint64_t z = (uint64_t)i + 0x9E3779B97F4A7C15ull * (uint64_t)(r + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        sk(i) = z ^ (z >> 31);
      });
    };
    const double t_fill = time_us(ex, 3, fill);
    const double t_sort_fill = time_us(ex, 3, [&](int r) {
      fill(r);
      Kokkos::sort(ex, sk);
    });
    // ---- Graph of 8 dependent parallel_for nodes over 2^16 elements ----------
    const int64_t gn = 1 << 16;
    std::vector<Kokkos::View<int64_t*, MS>> gv;
    for (int i = 0; i < 9; ++i) gv.emplace_back("gv", gn);
    auto chain = [&]() {
      for (int i = 0; i < 8; ++i) Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, gn), AddOne{gv[i], gv[i + 1]});
    };
    auto graph = Kokkos::Experimental::create_graph(ex, [&](auto root) {
      // type-erased node handle, so that each link can be assigned to it
      Kokkos::Experimental::GraphNodeRef<ES> node = root.then_parallel_for(Kokkos::RangePolicy<ES>(0, gn), AddOne{gv[0], gv[1]});
      for (int i = 1; i < 8; ++i) node = node.then_parallel_for(Kokkos::RangePolicy<ES>(0, gn), AddOne{gv[i], gv[i + 1]});
    });
    graph.instantiate();
    const double t_chain = time_us(ex, reps * 10, [&](int) { chain(); });
    const double t_graph = time_us(ex, reps * 10, [&](int) { graph.submit(); });
    // ---- UnorderedMap: AtomicAdd inserts, then finds --------------------------
    const uint32_t unk = 1u << 24, unu = 1u << 23;
    Kokkos::View<uint32_t*, MS> uks("uks", unk), ufx("ufx", unk);
    Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, unk),
                         KOKKOS_LAMBDA(int64_t i) { uks(i) = bench_key((uint64_t)i, unu - 1); });
    using UMap = Kokkos::UnorderedMap<uint32_t, uint32_t, ES>;
    using UAdd =
        Kokkos::UnorderedMapInsertOpTypes<Kokkos::View<uint32_t*, typename UMap::device_type>, uint32_t>::AtomicAdd;
    UMap umap(unu);
    cudaEvent_t ua, ub;
    cudaEventCreate(&ua);
    cudaEventCreate(&ub);
    double t_uins = 0;
    for (int r = 0; r < 3 + reps; ++r) {
      umap.clear();
      ex.fence();
      cudaEventRecord(ua, ex.stream());
      Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, unk), KOKKOS_LAMBDA(int64_t i) { umap.insert(uks(i), 1u, UAdd()); });
      cudaEventRecord(ub, ex.stream());
      cudaEventSynchronize(ub);
      float ms = 0;
      cudaEventElapsedTime(&ms, ua, ub);
      if (r >= 3) t_uins += 1000.0 * ms / reps;
    }
    cudaEventDestroy(ua);
    cudaEventDestroy(ub);
    const double t_ufind = time_us(ex, reps, [&](int) {
      Kokkos::parallel_for(Kokkos::RangePolicy<ES>(ex, 0, unk), KOKKOS_LAMBDA(int64_t i) { ufx(i) = umap.find(uks(i)); });
    });
    std::vector<uint32_t> hks(unk);
    for (uint32_t i = 0; i < unk; ++i) hks[i] = bench_key(i, unu - 1);
    std::sort(hks.begin(), hks.end());
    const uint32_t udistinct = (uint32_t)(std::unique(hks.begin(), hks.end()) - hks.begin());
    int64_t umissing = 0;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(ex, 0, unk), KOKKOS_LAMBDA(int64_t i, int64_t& u) {
      u += (umap.valid_at(ufx(i)) && umap.key_at(ufx(i)) == uks(i)) ? 0 : 1;
    }, umissing);
    const bool umap_ok = umap.size() == udistinct && !umap.failed_insert() && umissing == 0;
    ex.fence();
    const double rb = (double)n * 8, mb = (double)n0 * n1 * n2 * 4, tb = (double)ns * 4 + (nseg + 1) * 8.0 + nseg * 4.0;
    const double hb = (double)nk * 4 + nb * 8.0;
    std::printf(
        "{\"range_sum_f64_2^24\": {\"host_result_us\": %.2f, \"view_result_us\": %.2f, \"GB/s\": %.1f}, "
        "\"mdrange_sum_f32_512x512x256\": {\"us\": %.2f, \"GB/s\": %.1f}, "
        "\"team_sum_f32_lognormal_segments\": {\"segments\": %lld, \"elements\": %lld, \"us\": %.2f, \"GB/s\": %.1f}, "
        "\"scatterview_hist_2^26_keys_2^16_bins\": {\"us\": %.2f, \"GB/s\": %.1f, \"log_uniform_keys_us\": %.2f}, "
        "\"sort_u64_2^27\": {\"ms\": %.3f, \"Gkeys_per_s\": %.2f}, "
        "\"graph_8_parallel_for_2^16\": {\"graph_us\": %.2f, \"launches_us\": %.2f}, "
        "\"umap_insert_u32\": {\"inserts\": %u, \"distinct\": %u, \"capacity\": %u, \"insert_us\": %.2f, "
        "\"G_inserts_per_s\": %.3f, \"find_us\": %.2f, \"G_finds_per_s\": %.3f, \"ok\": %s}}\n",
        t_range_host, t_range_dev, gbs(rb, t_range_dev), t_md, gbs(mb, t_md), (long long)nseg, (long long)ns, t_team,
        gbs(tb, t_team), t_hist, gbs(hb, t_hist), t_hist_skew, (t_sort_fill - t_fill) / 1000.0,
        (double)nsort / ((t_sort_fill - t_fill) * 1e-6) / 1e9, t_graph, t_chain, unk, udistinct,
        (unsigned)umap.capacity(), t_uins, unk / t_uins * 1e-3, t_ufind, unk / t_ufind * 1e-3,
        umap_ok ? "true" : "false");
  }
  Kokkos::finalize();
  return 0;
}
