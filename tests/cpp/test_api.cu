// Tests of the header-template path (include/Kokkos_GB300.hpp), in the style
// of the reference's unit tests (core/unit_test/TestReduce.hpp,
// TestReducers.hpp, TestMDRangeReduce.hpp, TestTeamReductionScan.hpp,
// TestParallelScanRangePolicy.hpp, containers/unit_tests/TestScatterView.hpp,
// algorithms/unit_tests/TestSort*.hpp, TestGraph.hpp): closed forms and host
// loops, bit-exact for integers and Loc results, float sums within the
// project's stated tolerances.  Prints one PASS/FAIL line per check and exits
// non-zero on any failure.
#include <Kokkos_GB300.hpp>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <vector>

static int g_fail = 0;
static void report(bool ok, const char* name, const char* detail = "") {
  std::printf("%s %s %s\n", ok ? "PASS" : "FAIL", name, detail);
  if (!ok) ++g_fail;
}

// splitmix64: seeded test data
struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * 0x1.0p-53; }
};

template <class T>
static Kokkos::View<T*> to_device(const std::vector<T>& h) {
  Kokkos::View<T*> d("d", (int64_t)h.size());
  Kokkos::View<T*, Kokkos::HostSpace> m((T*)h.data(), (int64_t)h.size());
  Kokkos::deep_copy(d, m);
  return d;
}
template <class T>
static std::vector<T> to_host(const Kokkos::View<T*>& d) {
  std::vector<T> h(d.size());
  Kokkos::View<T*, Kokkos::HostSpace> m(h.data(), (int64_t)h.size());
  Kokkos::deep_copy(m, d);
  return h;
}

static double comp_sum(const double* x, size_t n, double* abs_out) {
  double s = 0, c = 0, a = 0;
  for (size_t i = 0; i < n; ++i) {
    const double t = s + x[i];
    c += std::fabs(s) >= std::fabs(x[i]) ? (s - t) + x[i] : (x[i] - t) + s;
    s = t;
    a += std::fabs(x[i]);
  }
  *abs_out = a;
  return s + c;
}

static void test_range_reducers() {
  // TestReduce.hpp-style closed form: sum of i over [0, n)
  for (int64_t n : {0L, 1L, 31L, 1000L, 1000003L}) {
    int64_t s = -1;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, int64_t& u) { u += i; }, s);
    char buf[64];
    std::snprintf(buf, sizeof buf, "n=%lld", (long long)n);
    report(s == n * (n - 1) / 2, "range_sum_closed_form", buf);
  }
  Rng r{7};
  const int64_t n = (1 << 20) + 17;
  std::vector<double> hx(n);
  std::vector<int32_t> hi(n);
  for (int64_t i = 0; i < n; ++i) {
    hx[i] = r.u01() * 2 - 1;
    hi[i] = (int32_t)(r.next() % 2001) - 1000;
  }
  hi[n / 3] = -5000;  // unique extrema, as the reference tests arrange
  hi[n / 5] = 7000;
  auto dx = to_device(hx);
  auto di = to_device(hi);
  double s = 0;
  Kokkos::parallel_reduce("sum", Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, double& u) { u += dx(i); },
                          Kokkos::Sum<double>(s));
  double a = 0;
  const double cs = comp_sum(hx.data(), n, &a);
  report(std::fabs(s - cs) <= 1e-12 * a, "range_sum_f64_tolerance");
  using VL = Kokkos::MinLoc<int32_t, int64_t>::value_type;
  VL mn;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, VL& u) {
    if (di(i) < u.val) { u.val = di(i); u.loc = i; }
  }, Kokkos::MinLoc<int32_t, int64_t>(mn));
  report(mn.val == -5000 && mn.loc == n / 3, "range_minloc_i32");
  VL mx;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, VL& u) {
    if (di(i) > u.val) { u.val = di(i); u.loc = i; }
  }, Kokkos::MaxLoc<int32_t, int64_t>(mx));
  report(mx.val == 7000 && mx.loc == n / 5, "range_maxloc_i32");
  Kokkos::MinMaxScalar<int32_t> mm;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, Kokkos::MinMaxScalar<int32_t>& u) {
    if (di(i) < u.min_val) u.min_val = di(i);
    if (di(i) > u.max_val) u.max_val = di(i);
  }, Kokkos::MinMax<int32_t>(mm));
  report(mm.min_val == -5000 && mm.max_val == 7000, "range_minmax_i32");
  int32_t band = 0, land = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, int32_t& u) { u &= (di(i) | 0x10000); },
                          Kokkos::BAnd<int32_t>(band));
  int32_t hband = ~0;
  for (int64_t i = 0; i < n; ++i) hband &= (hi[i] | 0x10000);
  report(band == hband, "range_band_i32");
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, int32_t& u) { u = u && (di(i) != 12345); },
                          Kokkos::LAnd<int32_t>(land));
  report(land == 1, "range_land_i32");
  // empty range: the reducer's identity (Min of float starts at FLT_MAX)
  float emin = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(5, 5), KOKKOS_LAMBDA(int64_t, float& u) { u = u; },
                          Kokkos::Min<float>(emin));
  report(emin == 3.402823466e+38F, "range_empty_identity");
  // result into a device View (no fence)
  Kokkos::View<double*> dres("dres", 1);
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, double& u) { u += dx(i); },
                          Kokkos::Sum<double>(dres));
  auto hres = to_host(dres);
  report(std::fabs(hres[0] - cs) <= 1e-12 * a, "range_sum_into_view");
}

static void test_mdrange() {
  // TestMDRangeReduce.hpp-style: LayoutLeft View<float***>, loc = i + n0*(j + n1*k)
  const int64_t n0 = 96, n1 = 80, n2 = 33;
  Rng r{11};
  std::vector<float> h(n0 * n1 * n2);
  for (auto& v : h) v = (float)(r.u01() * 2 - 1);
  const int64_t imin = 12345, imax = 54321;
  h[imin] = -3.f;
  h[imax] = 3.f;
  Kokkos::View<float***, Kokkos::LayoutLeft> x("x", n0, n1, n2);
  Kokkos::check_cuda(cudaMemcpy(x.data(), h.data(), h.size() * 4, cudaMemcpyHostToDevice), "copy");
  using V = Kokkos::MinLoc<float, int64_t>::value_type;
  V mn, mx;
  Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                          KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, V& u) {
                            if (x(i, j, k) < u.val) { u.val = x(i, j, k); u.loc = i + n0 * (j + n1 * k); }
                          },
                          Kokkos::MinLoc<float, int64_t>(mn));
  Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                          KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, V& u) {
                            if (x(i, j, k) > u.val) { u.val = x(i, j, k); u.loc = i + n0 * (j + n1 * k); }
                          },
                          Kokkos::MaxLoc<float, int64_t>(mx));
  report(mn.val == -3.f && mn.loc == imin, "mdrange_minloc_f32");
  report(mx.val == 3.f && mx.loc == imax, "mdrange_maxloc_f32");
  // LOr over a sub-box, rank 2 (TestMDRangeReduce: bounds {0,1,7,32,65,7000})
  for (int64_t e : {0L, 1L, 7L, 32L, 65L, 7000L}) {
    int32_t lor = 0;
    Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<2>>({0, 0}, {e, 3}),
                            KOKKOS_LAMBDA(int64_t i, int64_t j, int32_t& u) { u = u || (i == e - 1 && j == 2); },
                            Kokkos::LOr<int32_t>(lor));
    report(lor == (e > 0 ? 1 : 0), "mdrange_lor_bounds");
  }
  double s = 0;
  Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<3>>({1, 2, 3}, {n0, n1, n2}),
                          KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, double& u) { u += x(i, j, k); }, s);
  double hs = 0;
  for (int64_t k = 3; k < n2; ++k)
    for (int64_t j = 2; j < n1; ++j)
      for (int64_t i = 1; i < n0; ++i) hs += h[i + n0 * (j + n1 * k)];
  report(std::fabs(s - hs) <= 1e-9 * std::fabs(hs) + 1e-9, "mdrange_subbox_sum");
}

static void test_team() {
  // TeamPolicy league of segments: per-team TeamThreadRange reduce written by
  // single(PerTeam), plus the league-level reduce (TestTeamReductionScan.hpp)
  const int64_t league = 777;
  std::vector<int64_t> off(league + 1, 0);
  for (int64_t s = 0; s < league; ++s) off[s + 1] = off[s] + (s * 37) % 1500;
  std::vector<int32_t> v(off[league]);
  for (size_t i = 0; i < v.size(); ++i) v[i] = (int32_t)(i % 97);
  auto dv = to_device(v);
  auto doff = to_device(off);
  Kokkos::View<int64_t*> sums("sums", league);
  using TP = Kokkos::TeamPolicy<>;
  Kokkos::parallel_for(TP(league, 128), KOKKOS_LAMBDA(const TP::member_type& t) {
    const int64_t s = t.league_rank();
    int64_t ts = 0;
    Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, doff(s), doff(s + 1)),
                            [&](int64_t i, int64_t& u) { u += dv(i); }, ts);
    Kokkos::single(Kokkos::PerTeam(t), [&]() { sums(s) = ts; });
  });
  auto hs = to_host(sums);
  bool ok = true;
  int64_t tot = 0;
  for (int64_t s = 0; s < league; ++s) {
    int64_t e = 0;
    for (int64_t i = off[s]; i < off[s + 1]; ++i) e += v[i];
    ok = ok && hs[s] == e;
    tot += e;
  }
  report(ok, "team_per_segment_sums");
  int64_t lsum = 0;
  Kokkos::parallel_reduce(TP(league, 256), KOKKOS_LAMBDA(const TP::member_type& t, int64_t& u) {
    const int64_t s = t.league_rank();
    int64_t ts = 0;
    Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, doff(s), doff(s + 1)),
                            [&](int64_t i, int64_t& w) { w += dv(i); }, ts);
    if (t.team_rank() == 0) u += ts;
  }, lsum);
  report(lsum == tot, "team_league_reduce");
  // team scan: per-segment exclusive prefix inside each team
  Kokkos::View<int64_t*> pre("pre", (int64_t)v.size());
  Kokkos::parallel_for(TP(league, 64), KOKKOS_LAMBDA(const TP::member_type& t) {
    const int64_t s = t.league_rank();
    Kokkos::parallel_scan(Kokkos::TeamThreadRange(t, doff(s), doff(s + 1)),
                          [&](int64_t i, int64_t& u, bool fin) {
                            if (fin) pre(i) = u;
                            u += dv(i);
                          });
  });
  auto hp = to_host(pre);
  ok = true;
  for (int64_t s = 0; s < league; ++s) {
    int64_t u = 0;
    for (int64_t i = off[s]; i < off[s + 1]; ++i) { ok = ok && hp[i] == u; u += v[i]; }
  }
  report(ok, "team_thread_range_scan");
}

static void test_scan() {
  // TestParallelScanRangePolicy.hpp-style: exclusive prefix of i with total
  for (int64_t n : {1L, 100L, 2049L, 1000003L}) {
    Kokkos::View<int64_t*> y("y", n);
    int64_t total = 0;
    Kokkos::parallel_scan(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, int64_t& u, bool fin) {
      if (fin) y(i) = u;
      u += i;
    }, total);
    auto h = to_host(y);
    bool ok = total == n * (n - 1) / 2;
    for (int64_t i = 0; i < n && ok; ++i) ok = h[i] == i * (i - 1) / 2;
    report(ok, "range_scan_with_total");
  }
  // inclusive, int32 -> int64 via the functor
  Rng r{3};
  const int64_t n = (1 << 22) + 5;
  std::vector<int32_t> hx(n);
  for (auto& v : hx) v = (int32_t)(r.next() % 16);
  auto dx = to_device(hx);
  Kokkos::View<int64_t*> y("y", n);
  Kokkos::parallel_scan(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, int64_t& u, bool fin) {
    u += dx(i);
    if (fin) y(i) = u;
  });
  auto h = to_host(y);
  int64_t run = 0;
  bool ok = true;
  for (int64_t i = 0; i < n && ok; ++i) { run += hx[i]; ok = h[i] == run; }
  report(ok, "range_scan_inclusive_widening");
}

static void test_scatter() {
  // ScatterView histogram (TestScatterView.hpp): sv.access()(k) += 1
  const int64_t n = 3000017, nb = 4096;
  Rng r{5};
  std::vector<int32_t> k(n);
  for (auto& v : k) { const double u = r.u01(); v = (int32_t)(nb * u * u * u); }
  auto dk = to_device(k);
  Kokkos::View<int64_t*> bins("bins", nb);
  auto sv = Kokkos::Experimental::create_scatter_view(bins);
  Kokkos::parallel_for(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i) {
    auto acc = sv.access();
    acc(dk(i)) += 1;
  });
  Kokkos::Experimental::contribute(bins, sv);
  auto hb = to_host(bins);
  std::vector<int64_t> want(nb, 0);
  for (auto v : k) want[v]++;
  report(hb == want, "scatterview_histogram");
  // ScatterMax / ScatterMin contributions
  Kokkos::View<int32_t*> mx("mx", nb);
  auto svm = Kokkos::Experimental::create_scatter_view<Kokkos::Experimental::ScatterMax>(mx);
  Kokkos::parallel_for(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i) {
    svm.access()(dk(i)).update((int32_t)(i % 1000));
  });
  auto hm = to_host(mx);
  std::vector<int32_t> wm(nb, 0);
  for (int64_t i = 0; i < n; ++i) wm[k[i]] = std::max(wm[k[i]], (int32_t)(i % 1000));
  report(hm == wm, "scatterview_max");
}

static void test_sorts() {
  Rng r{9};
  const int64_t n = 1000003;
  std::vector<uint64_t> keys(n);
  for (auto& v : keys) v = r.next() & 0xFFFF0000000000FFull;  // many equal keys
  auto dk = to_device(keys);
  std::vector<int32_t> iota(n);
  std::iota(iota.begin(), iota.end(), 0);
  auto dv = to_device(iota);
  Kokkos::Experimental::sort_by_key(dk, dv);
  auto hk = to_host(dk);
  auto hv = to_host(dv);
  std::vector<int32_t> perm(iota);
  std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) { return keys[a] < keys[b]; });
  report(hv == perm, "sort_by_key_stable_permutation");
  std::vector<uint64_t> sk(keys);
  std::sort(sk.begin(), sk.end());
  report(hk == sk, "sort_by_key_keys");
  std::vector<double> d(n);
  for (auto& v : d) v = r.u01() - 0.5;
  auto dd = to_device(d);
  Kokkos::sort(dd);
  auto hd = to_host(dd);
  std::sort(d.begin(), d.end());
  report(hd == d, "sort_f64");
  // BinSort with BinOp1D (TestBinSortA.hpp)
  std::vector<uint64_t> bk(200003);
  for (auto& v : bk) v = r.next() % 1000000;
  auto dbk = to_device(bk);
  const uint64_t kmin = *std::min_element(bk.begin(), bk.end()), kmax = *std::max_element(bk.begin(), bk.end());
  using KV = Kokkos::View<uint64_t*>;
  Kokkos::BinOp1D<KV> op(5000, kmin, kmax);
  Kokkos::BinSort<KV, Kokkos::BinOp1D<KV>> bs(dbk, op, true);
  bs.create_permute_vector();
  bs.sort(dbk);
  auto hbk = to_host(dbk);
  std::vector<uint64_t> sbk(bk);
  std::sort(sbk.begin(), sbk.end());
  report(hbk == sbk, "binsort_sort_within_bins");
  auto cnt = to_host(bs.get_bin_count());
  int64_t tot = 0;
  for (auto c : cnt) tot += c;
  report(tot == (int64_t)bk.size() && (int64_t)cnt.size() == 5001, "binsort_counts");
}

static void test_std_algorithms() {
  namespace KE = Kokkos::Experimental;
  Rng r{13};
  const int64_t n = 1 << 20;
  std::vector<int32_t> x(n);
  for (auto& v : x) v = (int32_t)(r.next() % 16);
  auto dx = to_device(x);
  Kokkos::View<int64_t*> y("y", n);
  KE::GB300 ex;
  KE::exclusive_scan(ex, KE::cbegin(dx), KE::cend(dx), KE::begin(y), (int64_t)7);
  auto h = to_host(y);
  int64_t run = 7;
  bool ok = true;
  for (int64_t i = 0; i < n && ok; ++i) { ok = h[i] == run; run += x[i]; }
  report(ok, "std_exclusive_scan_i32_i64_init");
  const int64_t s = KE::reduce(ex, KE::cbegin(y), KE::cend(y), (int64_t)0);
  int64_t hs = 0;
  for (auto v : h) hs += v;
  report(s == hs, "std_reduce_i64");
  Kokkos::View<int32_t*> z("z", n);
  KE::inclusive_scan(ex, KE::cbegin(dx), KE::cend(dx), KE::begin(z));
  auto hz = to_host(z);
  int32_t ri = 0;
  ok = true;
  for (int64_t i = 0; i < n && ok; ++i) { ri += x[i]; ok = hz[i] == ri; }
  report(ok, "std_inclusive_scan_i32");
}

static void test_graph() {
  // TestGraph.hpp-style: a chain of nodes, submitted more than once
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  Kokkos::Experimental::GB300 ex(st);
  const int64_t n = 1 << 20;
  Kokkos::View<int64_t*> a("a", n), b("b", n);
  Kokkos::View<int64_t*> out("out", 2);
  auto o0 = Kokkos::View<int64_t*>(out.data(), 1), o1 = Kokkos::View<int64_t*>(out.data() + 1, 1);
  // (nvcc does not allow extended lambdas inside a generic lambda, so the
  // closure names the node type instead of `auto`)
  auto graph = Kokkos::Experimental::create_graph(ex, [&](Kokkos::Experimental::GraphNodeRef root) {
    auto n1 = root.then_parallel_for(n, KOKKOS_LAMBDA(int64_t i) { a(i) = i % 10; });
    auto n2 = n1.then_parallel_scan(n, KOKKOS_LAMBDA(int64_t i, int64_t& u, bool fin) {
      if (fin) b(i) = u;
      u += a(i);
    });
    auto n3 = n2.then_parallel_reduce(n, KOKKOS_LAMBDA(int64_t i, int64_t& u) { u += b(i) % 3; },
                                      Kokkos::Sum<int64_t>(o0));
    n3.then_parallel_reduce(n, KOKKOS_LAMBDA(int64_t i, int64_t& u) { if (b(i) > u) u = b(i); },
                            Kokkos::Max<int64_t>(o1));
  });
  int64_t want0 = 0, want1 = 0, run = 0;
  for (int64_t i = 0; i < n; ++i) { want0 += run % 3; want1 = std::max(want1, run); run += i % 10; }
  bool ok = true;
  for (int rep = 0; rep < 3; ++rep) {
    cudaMemsetAsync(out.data(), 0, 16, st);
    graph.submit();
    ex.fence();
    auto h = to_host(out);
    ok = ok && h[0] == want0 && h[1] == want1;
  }
  report(ok, "graph_chain_submitted_three_times");
  cudaStreamDestroy(st);
}

static void test_errors() {
  bool threw = false;
  try {
    Kokkos::RangePolicy<> p(5, 2);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  report(threw, "rangepolicy_bounds_error");
  threw = false;
  try {
    Kokkos::View<uint64_t*> k("k", 10);
    Kokkos::View<int32_t*> v("v", 9);
    Kokkos::Experimental::sort_by_key(k, v);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  report(threw, "sort_by_key_extent_mismatch");
}

int main(int argc, char** argv) {
  Kokkos::initialize(argc, argv);
  {
    test_range_reducers();
    test_mdrange();
    test_team();
    test_scan();
    test_scatter();
    test_sorts();
    test_std_algorithms();
    test_graph();
    test_errors();
  }
  Kokkos::finalize();
  std::printf("%s (%d failures)\n", g_fail ? "SOME FAILED" : "ALL PASS", g_fail);
  return g_fail ? 1 : 0;
}
