// The reference's own Kokkos API on the GB300 execution space: this program
// is compiled against the Kokkos headers with include/gb300_backend ahead of
// them (tests/backend/Makefile), so every call below goes through Kokkos'
// generic dispatch into the GB300 pattern specialisations, memory space,
// ScatterView defaults and sort overloads.  Each check compares with a plain
// host computation and prints "ok <name>" or "FAIL <name> ...".
//
//   backend_api              run every check on cuda:0 (exit status = failures)
//   backend_api --no-device  on a machine without a GPU: show that the space is
//                            registered (Kokkos::initialize reaches
//                            GB300::impl_initialize, which reports the missing
//                            device) and exit 0
#include <Kokkos_Core.hpp>
#include <Kokkos_ScatterView.hpp>
#include <Kokkos_Sort.hpp>
#include <Kokkos_StdAlgorithms.hpp>
#include <Kokkos_Graph.hpp>
#include <GB300/Kokkos_GB300_Graph_Impl.hpp>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <numeric>
#include <string>
#include <vector>

using ES = Kokkos::Experimental::GB300;
using MS = Kokkos::Experimental::GB300Space;
// (Kokkos' execution-space concept check, check_valid_execution_space, runs
// where the space registers itself: include/gb300_backend/GB300/Kokkos_GB300.cpp.)
static_assert(Kokkos::is_execution_space_v<ES> && Kokkos::is_memory_space_v<MS>);
static_assert(!Kokkos::SpaceAccessibility<Kokkos::HostSpace, MS>::accessible);
static_assert(Kokkos::SpaceAccessibility<ES, MS>::accessible);

static int g_fail = 0;
static void report(bool ok, const char* name, const std::string& detail = "") {
  if (ok) std::printf("ok %s\n", name);
  else {
    std::printf("FAIL %s %s\n", name, detail.c_str());
    ++g_fail;
  }
}

// array reduction: value_type[] with a runtime count (sum, sum of squares, count)
struct ArrayMoments {
  using value_type = double[];
  using size_type = int;
  Kokkos::View<const double*, MS> x;
  size_type value_count = 3;
  KOKKOS_INLINE_FUNCTION void operator()(int i, value_type v) const {
    v[0] += x(i);
    v[1] += x(i) * x(i);
    v[2] += 1.0;
  }
  KOKKOS_INLINE_FUNCTION void init(value_type v) const { v[0] = v[1] = v[2] = 0.0; }
  KOKKOS_INLINE_FUNCTION void join(value_type d, const value_type s) const {
    for (int k = 0; k < 3; ++k) d[k] += s[k];
  }
};

// functor with init / join / final: mean of x (final divides by the count)
struct Mean {
  struct value_type {
    double s;
    double c;
  };
  Kokkos::View<const double*, MS> x;
  KOKKOS_INLINE_FUNCTION void operator()(int i, value_type& v) const {
    v.s += x(i);
    v.c += 1.0;
  }
  KOKKOS_INLINE_FUNCTION void init(value_type& v) const { v.s = v.c = 0.0; }
  KOKKOS_INLINE_FUNCTION void join(value_type& d, const value_type& s) const {
    d.s += s.s;
    d.c += s.c;
  }
  KOKKOS_INLINE_FUNCTION void final(value_type& v) const { v.s = v.c > 0 ? v.s / v.c : 0.0; }
};

struct TagA {};
struct Tagged {
  Kokkos::View<int64_t*, MS> y;
  KOKKOS_INLINE_FUNCTION void operator()(TagA, int i) const { y(i) = 3 * i; }
  KOKKOS_INLINE_FUNCTION void operator()(TagA, int i, int64_t& s) const { s += y(i); }
};

static void range_checks() {
  const int n = (1 << 20) + 77;
  Kokkos::View<double*, MS> x("x", n);
  Kokkos::parallel_for("fill", Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) { x(i) = 0.5 * (i % 7); });
  double s = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i, double& u) { u += x(i); }, s);
  double want = 0;
  for (int i = 0; i < n; ++i) want += 0.5 * (i % 7);
  report(s == want, "range_reduce_sum", std::to_string(s) + " vs " + std::to_string(want));

  // offset range, Sum reducer into a device View result
  Kokkos::View<double, MS> dres("r");
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(100, n - 5), KOKKOS_LAMBDA(int i, double& u) { u += x(i); },
                          Kokkos::Sum<double, MS>(dres));
  double r = 0;
  Kokkos::deep_copy(r, dres);
  double w2 = 0;
  for (int i = 100; i < n - 5; ++i) w2 += 0.5 * (i % 7);
  report(r == w2, "range_reduce_view_result");

  // MinLoc / MaxLoc with a unique extremum
  Kokkos::View<int*, MS> v("v", n);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) { v(i) = (int)((i * 7919L) % 1000003) + 5; });
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(777, 778), KOKKOS_LAMBDA(int i) { v(i) = -4; });
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(n - 3, n - 2), KOKKOS_LAMBDA(int i) { v(i) = 5000000; });
  Kokkos::MinLoc<int, int>::value_type mn;
  Kokkos::MaxLoc<int, int>::value_type mx;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(0, n),
                          KOKKOS_LAMBDA(int i, Kokkos::MinLoc<int, int>::value_type& u) {
                            if (v(i) < u.val) { u.val = v(i); u.loc = i; }
                          },
                          Kokkos::MinLoc<int, int>(mn));
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(0, n),
                          KOKKOS_LAMBDA(int i, Kokkos::MaxLoc<int, int>::value_type& u) {
                            if (v(i) > u.val) { u.val = v(i); u.loc = i; }
                          },
                          Kokkos::MaxLoc<int, int>(mx));
  report(mn.val == -4 && mn.loc == 777 && mx.val == 5000000 && mx.loc == n - 3, "range_minloc_maxloc");

  // two reducers in one pass (Kokkos_Combined_Reducer.hpp)
  double s2 = 0;
  int mxv = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(0, n),
                          KOKKOS_LAMBDA(int i, double& a, int& b) {
                            a += x(i);
                            if (v(i) > b) b = v(i);
                          },
                          s2, Kokkos::Max<int>(mxv));
  report(s2 == want && mxv == 5000000, "range_combined_reducers");

  // array reduction (runtime value count) and a functor with final()
  double mom[3] = {0, 0, 0};
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(0, n), ArrayMoments{x}, mom);
  double sq = 0;
  for (int i = 0; i < n; ++i) sq += 0.25 * (i % 7) * (i % 7);
  report(mom[0] == want && mom[1] == sq && mom[2] == n, "range_array_reduction");
  Mean::value_type mean;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(0, n), Mean{x}, mean);
  report(std::fabs(mean.s - want / n) <= 1e-12 * (want / n), "range_functor_final");

  // work tags
  Kokkos::View<int64_t*, MS> y("y", 1000);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES, TagA>(0, 1000), Tagged{y});
  int64_t ts = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES, TagA>(0, 1000), Tagged{y}, ts);
  report(ts == 3 * 999 * 1000 / 2, "range_work_tag");

  // empty range: the identity
  double e = 1.0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<ES>(5, 5), KOKKOS_LAMBDA(int i, double& u) { u += x(i); }, e);
  report(e == 0.0, "range_reduce_empty");
}

static void scan_checks() {
  const int n = 3 * 2048 * 5 + 123;
  Kokkos::View<int64_t*, MS> x("x", n), y("y", n);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) { x(i) = (i * 37) % 16; });
  int64_t total = 0;
  Kokkos::parallel_scan(Kokkos::RangePolicy<ES>(0, n),
                        KOKKOS_LAMBDA(int i, int64_t& u, bool fin) {
                          if (fin) y(i) = u;  // exclusive
                          u += x(i);
                        },
                        total);
  auto hy = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), y);
  int64_t run = 0;
  bool ok = true;
  for (int i = 0; i < n; ++i) {
    ok &= hy(i) == run;
    run += (i * 37) % 16;
  }
  report(ok && total == run, "parallel_scan_exclusive_with_total");
  Kokkos::parallel_scan(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i, int64_t& u, bool fin) {
    u += x(i);
    if (fin) y(i) = u;  // inclusive
  });
  Kokkos::deep_copy(hy, y);
  run = 0;
  ok = true;
  for (int i = 0; i < n; ++i) {
    run += (i * 37) % 16;
    ok &= hy(i) == run;
  }
  report(ok, "parallel_scan_inclusive");
  // std algorithms on the space
  namespace KE = Kokkos::Experimental;
  Kokkos::View<int32_t*, MS> a("a", n);
  Kokkos::View<int64_t*, MS> b("b", n);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) { a(i) = i % 16; });
  KE::exclusive_scan(ES(), KE::cbegin(a), KE::cend(a), KE::begin(b), int64_t{0});
  Kokkos::deep_copy(hy, b);
  run = 0;
  ok = true;
  for (int i = 0; i < n; ++i) {
    ok &= hy(i) == run;
    run += i % 16;
  }
  report(ok, "std_exclusive_scan");
  const int64_t red = KE::reduce(ES(), KE::cbegin(b), KE::cend(b), int64_t{0});
  int64_t wr = 0;
  for (int i = 0; i < n; ++i) wr += hy(i);
  report(red == wr, "std_reduce");
}

static void mdrange_checks() {
  const int n0 = 67, n1 = 33, n2 = 21;
  Kokkos::View<float***, Kokkos::LayoutLeft, MS> v("v", n0, n1, n2);
  Kokkos::parallel_for(Kokkos::MDRangePolicy<ES, Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                       KOKKOS_LAMBDA(int i, int j, int k) { v(i, j, k) = (float)((i + 2 * j + 3 * k) % 11); });
  double want = 0;
  for (int i = 0; i < n0; ++i)
    for (int j = 0; j < n1; ++j)
      for (int k = 0; k < n2; ++k) want += (i + 2 * j + 3 * k) % 11;
  float s = 0;
  Kokkos::parallel_reduce(Kokkos::MDRangePolicy<ES, Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                          KOKKOS_LAMBDA(int i, int j, int k, float& u) { u += v(i, j, k); }, s);
  report((double)s == want, "mdrange_rank3_sum");
  // tiles and Iterate::Right, the reference's tile constructor
  float s2 = 0;
  Kokkos::parallel_reduce(
      Kokkos::MDRangePolicy<ES, Kokkos::Rank<3, Kokkos::Iterate::Right, Kokkos::Iterate::Right>>({1, 2, 3},
                                                                                                 {n0, n1, n2}, {4, 4, 8}),
      KOKKOS_LAMBDA(int i, int j, int k, float& u) { u += v(i, j, k); }, s2);
  double w2 = 0;
  for (int i = 1; i < n0; ++i)
    for (int j = 2; j < n1; ++j)
      for (int k = 3; k < n2; ++k) w2 += (i + 2 * j + 3 * k) % 11;
  report((double)s2 == w2, "mdrange_tiled_iterate_right");
  // rank 6
  Kokkos::View<int******, MS> z("z", 3, 4, 2, 5, 3, 2);
  Kokkos::parallel_for(Kokkos::MDRangePolicy<ES, Kokkos::Rank<6>>({0, 0, 0, 0, 0, 0}, {3, 4, 2, 5, 3, 2}),
                       KOKKOS_LAMBDA(int a, int b, int c, int d, int e, int f) {
                         z(a, b, c, d, e, f) = a + 10 * b + 100 * c + 1000 * d + 10000 * e + 100000 * f;
                       });
  long t = 0;
  Kokkos::parallel_reduce(Kokkos::MDRangePolicy<ES, Kokkos::Rank<6>>({0, 0, 0, 0, 0, 0}, {3, 4, 2, 5, 3, 2}),
                          KOKKOS_LAMBDA(int a, int b, int c, int d, int e, int f, long& u) { u += z(a, b, c, d, e, f); },
                          t);
  long wt = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 4; ++b)
      for (int c = 0; c < 2; ++c)
        for (int d = 0; d < 5; ++d)
          for (int e = 0; e < 3; ++e)
            for (int f = 0; f < 2; ++f) wt += a + 10 * b + 100 * c + 1000 * d + 10000 * e + 100000 * f;
  report(t == wt, "mdrange_rank6");
  // deep_copy of a strided (rank-3 LayoutLeft) view to the host mirror
  auto hv = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), v);
  report(hv(5, 7, 9) == (float)((5 + 14 + 27) % 11), "mdrange_mirror");
}

static void team_checks() {
  using TP = Kokkos::TeamPolicy<ES>;
  using member = TP::member_type;
  const int league = 1000, len = 777;
  Kokkos::View<double**, Kokkos::LayoutRight, MS> a("a", league, len);
  Kokkos::parallel_for(Kokkos::MDRangePolicy<ES, Kokkos::Rank<2>>({0, 0}, {league, len}),
                       KOKKOS_LAMBDA(int i, int j) { a(i, j) = (i + j) % 5; });
  Kokkos::View<double*, MS> rows("rows", league);
  for (int ts : {128, 100}) {
    Kokkos::parallel_for(TP(league, ts), KOKKOS_LAMBDA(const member& m) {
      const int i = m.league_rank();
      double s = 0;
      Kokkos::parallel_reduce(Kokkos::TeamThreadRange(m, len), [&](int j, double& u) { u += a(i, j); }, s);
      Kokkos::single(Kokkos::PerTeam(m), [&]() { rows(i) = s; });
    });
    auto hr = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), rows);
    bool ok = true;
    for (int i = 0; i < league; ++i) {
      double w = 0;
      for (int j = 0; j < len; ++j) w += (i + j) % 5;
      ok &= hr(i) == w;
    }
    report(ok, ts == 128 ? "team_thread_range_reduce" : "team_thread_range_reduce_team100");
  }
  double tot = 0;
  Kokkos::parallel_reduce(TP(league, Kokkos::AUTO), KOKKOS_LAMBDA(const member& m, double& u) {
    Kokkos::parallel_for(Kokkos::TeamThreadRange(m, len), [&](int j) { u += a(m.league_rank(), j); });
  }, tot);
  double want = 0;
  for (int i = 0; i < league; ++i)
    for (int j = 0; j < len; ++j) want += (i + j) % 5;
  report(tot == want, "team_policy_reduce");
  // team_scan and a TeamThreadRange scan
  Kokkos::View<int*, MS> out("out", league * 64);
  Kokkos::parallel_for(TP(league, 64), KOKKOS_LAMBDA(const member& m) {
    const int p = m.team_scan(m.team_rank() + 1);
    out(m.league_rank() * 64 + m.team_rank()) = p;
  });
  auto ho = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), out);
  bool ok = true;
  for (int t = 0; t < 64; ++t) ok &= ho(3 * 64 + t) == t * (t + 1) / 2;
  report(ok, "team_scan");
  Kokkos::View<int*, MS> sc("sc", league * len);
  Kokkos::parallel_for(TP(league, 96), KOKKOS_LAMBDA(const member& m) {
    const int i = m.league_rank();
    Kokkos::parallel_scan(Kokkos::TeamThreadRange(m, len), [&](int j, int& u, bool fin) {
      if (fin) sc(i * len + j) = u;
      u += (i + j) % 3;
    });
  });
  auto hs = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), sc);
  ok = true;
  for (int i : {0, 17, league - 1}) {
    int run = 0;
    for (int j = 0; j < len; ++j) {
      ok &= hs(i * len + j) == run;
      run += (i + j) % 3;
    }
  }
  report(ok, "team_thread_range_scan");
  // level-0 team scratch
  using ScratchV = Kokkos::View<double*, ES::scratch_memory_space, Kokkos::MemoryUnmanaged>;
  Kokkos::parallel_for(TP(league, 64).set_scratch_size(0, Kokkos::PerTeam(ScratchV::shmem_size(64))),
                       KOKKOS_LAMBDA(const member& m) {
                         ScratchV buf(m.team_scratch(0), 64);
                         buf(m.team_rank()) = m.team_rank();
                         m.team_barrier();
                         double s = 0;
                         for (int k = 0; k < 64; ++k) s += buf(k);
                         Kokkos::single(Kokkos::PerTeam(m), [&]() { rows(m.league_rank()) = s; });
                       });
  auto hr = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), rows);
  report(hr(0) == 2016 && hr(league - 1) == 2016, "team_scratch");
}

static void scatter_sort_checks() {
  const int n = 1 << 20, nb = 4096;
  Kokkos::View<int*, MS> keys("keys", n);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) {
    keys(i) = (i % 3 == 0) ? 7 : (int)((i * 2654435761u) % nb);  // a hot bin
  });
  Kokkos::View<int64_t*, MS> bins("bins", nb);
  auto sv = Kokkos::Experimental::create_scatter_view(bins);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) {
    auto acc = sv.access();
    acc(keys(i)) += 1;
  });
  Kokkos::Experimental::contribute(bins, sv);
  auto hb = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), bins);
  std::vector<int64_t> want(nb, 0);
  for (int i = 0; i < n; ++i) ++want[(i % 3 == 0) ? 7 : (int)((i * 2654435761u) % nb)];
  bool ok = true;
  for (int b = 0; b < nb; ++b) ok &= hb(b) == want[b];
  report(ok, "scatter_view_histogram");

  Kokkos::View<uint64_t*, MS> k("k", n);
  Kokkos::View<int*, MS> val("val", n);
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) {
    uint64_t z = (uint64_t)i * 0x9E3779B97F4A7C15ull;
    z ^= z >> 31;
    k(i) = z % 100000;  // duplicates: the stable order is checked by the payload
    val(i) = i;
  });
  auto hk0 = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), k);
  Kokkos::Experimental::sort_by_key(ES(), k, val);
  auto hk = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), k);
  auto hvv = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace(), val);
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int p, int q) { return hk0(p) < hk0(q); });
  ok = true;
  for (int i = 0; i < n; ++i) ok &= hvv(i) == idx[i] && hk(i) == hk0(idx[i]);
  report(ok, "sort_by_key_stable");
  Kokkos::parallel_for(Kokkos::RangePolicy<ES>(0, n), KOKKOS_LAMBDA(int i) { k(i) = (uint64_t)(n - i) * 977; });
  Kokkos::sort(ES(), k);
  Kokkos::deep_copy(hk, k);
  ok = true;
  for (int i = 0; i < n; ++i) ok &= hk(i) == (uint64_t)(i + 1) * 977;
  report(ok, "sort");
}

// Experimental::Graph on the GB300 space (GraphImpl<GB300>: the nodes are
// captured into one CUDA graph at instantiate): a chain of two parallel_for
// and a parallel_reduce into a device View, submitted three times; then a
// diamond through when_all (an aggregate node) submitted twice, once on
// another instance.
// (functors, not lambdas: nvcc takes no extended lambda inside the generic
// lambda that builds the graph)
struct GraphFill {
  Kokkos::View<int64_t*, MS> a;
  KOKKOS_INLINE_FUNCTION void operator()(int i) const { a(i) = i % 7; }
};
struct GraphMap {
  Kokkos::View<int64_t*, MS> a, b;
  KOKKOS_INLINE_FUNCTION void operator()(int i) const { b(i) = 2 * a(i) + 1; }
};
struct GraphSum {
  Kokkos::View<int64_t*, MS> b;
  KOKKOS_INLINE_FUNCTION void operator()(int i, int64_t& u) const { u += b(i); }
};
struct GraphShift {
  Kokkos::View<int64_t*, MS> a, c;
  KOKKOS_INLINE_FUNCTION void operator()(int i) const { c(i) = a(i) + 5; }
};
struct GraphSum2 {
  Kokkos::View<int64_t*, MS> b, c;
  KOKKOS_INLINE_FUNCTION void operator()(int i, int64_t& u) const { u += b(i) + c(i); }
};
static void graph_checks() {
  const int n = 1 << 20;
  ES ex;
  Kokkos::View<int64_t*, MS> a("a", n), b("b", n);
  Kokkos::View<int64_t, MS> s("s");
  auto graph = Kokkos::Experimental::create_graph(ex, [&](auto root) {
    auto f1 = root.then_parallel_for(Kokkos::RangePolicy<ES>(0, n), GraphFill{a});
    auto f2 = f1.then_parallel_for(Kokkos::RangePolicy<ES>(0, n), GraphMap{a, b});
    f2.then_parallel_reduce(Kokkos::RangePolicy<ES>(0, n), GraphSum{b}, s);
  });
  int64_t want = 0;
  for (int i = 0; i < n; ++i) want += 2 * (i % 7) + 1;
  bool ok = true;
  for (int rep = 0; rep < 3; ++rep) {
    Kokkos::deep_copy(ex, s, int64_t(0));
    Kokkos::deep_copy(ex, b, int64_t(0));
    graph.submit();
    int64_t got = -1;
    Kokkos::deep_copy(ex, got, s);
    ex.fence();
    ok = ok && got == want;
  }
  report(ok, "graph_chain_submit_three_times");
  // diamond: fill a; b = 2a + 1 and c = a + 5 both after it; sum of b + c after both
  Kokkos::View<int64_t*, MS> c("c", n);
  Kokkos::View<int64_t, MS> s2("s2");
  auto diamond = Kokkos::Experimental::create_graph(ex, [&](auto root) {
    auto f1 = root.then_parallel_for(Kokkos::RangePolicy<ES>(0, n), GraphFill{a});
    auto fb = f1.then_parallel_for(Kokkos::RangePolicy<ES>(0, n), GraphMap{a, b});
    auto fc = f1.then_parallel_for(Kokkos::RangePolicy<ES>(0, n), GraphShift{a, c});
    Kokkos::Experimental::when_all(fb, fc).then_parallel_reduce(Kokkos::RangePolicy<ES>(0, n), GraphSum2{b, c}, s2);
  });
  int64_t want2 = want;
  for (int i = 0; i < n; ++i) want2 += i % 7 + 5;
  cudaStream_t other_stream = nullptr;
  cudaStreamCreateWithFlags(&other_stream, cudaStreamNonBlocking);
  ES other(other_stream);
  bool ok2 = true;
  for (int rep = 0; rep < 2; ++rep) {
    const ES& on = rep ? other : ex;
    Kokkos::deep_copy(on, s2, int64_t(0));
    Kokkos::deep_copy(on, b, int64_t(0));
    Kokkos::deep_copy(on, c, int64_t(0));
    diamond.submit(on);
    int64_t got = -1;
    Kokkos::deep_copy(on, got, s2);
    on.fence();
    ok2 = ok2 && got == want2;
  }
  report(ok2, "graph_diamond_when_all");
  other.fence();
  cudaStreamDestroy(other_stream);
}

static void copy_checks() {
  const int n = 1000003;
  std::vector<double> h(n);
  for (int i = 0; i < n; ++i) h[i] = i * 0.25;
  Kokkos::View<double*, Kokkos::HostSpace, Kokkos::MemoryUnmanaged> hu(h.data(), n);
  Kokkos::View<double*, MS> d("d", n);
  Kokkos::deep_copy(d, hu);
  Kokkos::View<double*, MS> d2("d2", n);
  Kokkos::deep_copy(ES(), d2, d);
  ES().fence();
  std::vector<double> back(n, -1);
  Kokkos::View<double*, Kokkos::HostSpace, Kokkos::MemoryUnmanaged> bu(back.data(), n);
  Kokkos::deep_copy(bu, d2);
  report(back == h, "deep_copy_roundtrip");
  Kokkos::deep_copy(d2, 3.5);
  Kokkos::deep_copy(bu, d2);
  report(std::all_of(back.begin(), back.end(), [](double v) { return v == 3.5; }), "deep_copy_value");
}

int main(int argc, char** argv) {
  if (argc > 1 && std::string(argv[1]) == "--no-device") {
    try {
      Kokkos::initialize(argc, argv);
    } catch (std::exception& e) {
      const bool ours = std::string(e.what()).find("Kokkos::Experimental::GB300: initialize") != std::string::npos;
      std::printf("%s: %s\n", ours ? "registered" : "unexpected", e.what());
      return ours ? 0 : 1;
    }
    std::printf("unexpected: initialize succeeded without a device\n");
    return 1;
  }
  Kokkos::initialize(argc, argv);
  {
    ES().print_configuration(std::cout);
    range_checks();
    scan_checks();
    mdrange_checks();
    team_checks();
    scatter_sort_checks();
    graph_checks();
    copy_checks();
    ES().fence();
  }
  Kokkos::finalize();
  std::printf("%d failures\n", g_fail);
  return g_fail;
}
