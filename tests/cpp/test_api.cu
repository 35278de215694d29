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
#include <limits>
#include <numeric>
#include <vector>

// The execution-space concept a Kokkos space must model
// (core/src/impl/Kokkos_ExecSpaceManager.hpp:17-108): typedefs, regular and
// at most two pointers in size.
using ESpace = Kokkos::Experimental::GB300;
static_assert(std::is_same<ESpace::execution_space, ESpace>::value, "execution_space");
static_assert(std::is_same<ESpace::device_type::execution_space, ESpace>::value, "device_type");
static_assert(std::is_same<ESpace::device_type::memory_space, ESpace::memory_space>::value, "memory_space");
static_assert(sizeof(ESpace::size_type) == 8 && sizeof(ESpace::array_layout) >= 1, "size_type / array_layout");
static_assert(sizeof(ESpace::scratch_memory_space) >= 1, "scratch_memory_space");
static_assert(std::is_default_constructible<ESpace>::value && std::is_copy_assignable<ESpace>::value, "regular");
static_assert(sizeof(ESpace) <= 2 * sizeof(void*), "at most two pointers");

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
  {  // several reducers in one pass (Kokkos_Combined_Reducer.hpp): MinLoc, MaxLoc, a Sum and a plain count
    VL cmn, cmx;
    double cs2 = 0;
    int64_t pos = 0;
    Kokkos::parallel_reduce("combined", Kokkos::RangePolicy<>(0, n),
                            KOKKOS_LAMBDA(int64_t i, VL& a, VL& b, double& su, int64_t& c) {
                              if (di(i) < a.val) { a.val = di(i); a.loc = i; }
                              if (di(i) > b.val) { b.val = di(i); b.loc = i; }
                              su += dx(i);
                              if (di(i) > 0) c += 1;
                            },
                            Kokkos::MinLoc<int32_t, int64_t>(cmn), Kokkos::MaxLoc<int32_t, int64_t>(cmx),
                            Kokkos::Sum<double>(cs2), pos);
    int64_t hpos = 0;
    for (int64_t i = 0; i < n; ++i) hpos += hi[i] > 0;
    report(cmn.val == -5000 && cmn.loc == n / 3 && cmx.val == 7000 && cmx.loc == n / 5 &&
               std::fabs(cs2 - cs) <= 1e-12 * a && pos == hpos,
           "range_combined_minloc_maxloc_sum_count");
    Kokkos::View<double*> dsum("dsum", 1);
    int64_t pos2 = 0;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, double& su, int64_t& c) {
      su += dx(i);
      c += di(i) > 0;
    }, Kokkos::Sum<double>(dsum), pos2);
    double hsum = 0;
    Kokkos::check_cuda(cudaMemcpy(&hsum, dsum.data(), sizeof(double), cudaMemcpyDeviceToHost), "copy");
    report(std::fabs(hsum - cs) <= 1e-12 * a && pos2 == hpos, "range_combined_view_result");
    Kokkos::View<int64_t*> dcount("dcount", 1);
    int64_t neg4 = 0;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, int64_t& p, int64_t& q) {
      p += di(i) > 0;
      q += di(i) < 0;
    }, dcount, neg4);  // a View result stands for a Sum into it, as a scalar does
    int64_t hcount = -1;
    Kokkos::check_cuda(cudaMemcpy(&hcount, dcount.data(), sizeof(int64_t), cudaMemcpyDeviceToHost), "copy");
    int64_t pos3 = 0, neg3 = 0;
    Kokkos::parallel_reduce("count", n, KOKKOS_LAMBDA(int64_t i, int64_t& p, int64_t& q) {
      p += di(i) > 0;
      q += di(i) < 0;
    }, pos3, neg3);
    int64_t hneg = 0;
    for (int64_t i = 0; i < n; ++i) hneg += hi[i] < 0;
    report(pos3 == hpos && neg3 == hneg, "range_combined_count_form");
    report(hcount == hpos && neg4 == hneg, "range_combined_view_as_sum");
  }
  {  // FirstLoc / LastLoc of a predicate, alone and as two reducers of one pass
    using FL = Kokkos::FirstLoc<int64_t>;
    using LL = Kokkos::LastLoc<int64_t>;
    FL::value_type f1;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, FL::value_type& u) {
      if (di(i) > 900 && i < u.min_loc_true) u.min_loc_true = i;
    }, FL(f1));
    FL::value_type f2;
    LL::value_type l2;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n),
                            KOKKOS_LAMBDA(int64_t i, FL::value_type& u, LL::value_type& w) {
                              if (di(i) > 900) {
                                if (i < u.min_loc_true) u.min_loc_true = i;
                                if (i > w.max_loc_true) w.max_loc_true = i;
                              }
                            },
                            FL(f2), LL(l2));
    int64_t hf = -1, hl = -1;
    for (int64_t i = 0; i < n; ++i)
      if (hi[i] > 900) {
        if (hf < 0) hf = i;
        hl = i;
      }
    FL::value_type none;
    Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i, FL::value_type& u) {
      if (di(i) > 100000 && i < u.min_loc_true) u.min_loc_true = i;
    }, FL(none));
    report(f1.min_loc_true == hf && f2.min_loc_true == hf && l2.max_loc_true == hl &&
               none.min_loc_true == std::numeric_limits<int64_t>::max(),
           "range_firstloc_lastloc");
  }
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

// a tagged MDRange functor (kernel template arguments may not be local types)
struct TagSq {};
struct Sq {
  KOKKOS_INLINE_FUNCTION void operator()(TagSq, int64_t i, int64_t j, int64_t& u) const { u += i * j; }
};

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
  {
    V cmn, cmx;
    double cs3 = 0;
    Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<3>>({0, 0, 0}, {n0, n1, n2}),
                            KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, V& a, V& b, double& su) {
                              const float v = x(i, j, k);
                              const int64_t l = i + n0 * (j + n1 * k);
                              if (v < a.val) { a.val = v; a.loc = l; }
                              if (v > b.val) { b.val = v; b.loc = l; }
                              su += v;
                            },
                            Kokkos::MinLoc<float, int64_t>(cmn), Kokkos::MaxLoc<float, int64_t>(cmx), cs3);
    double hs3 = 0;
    for (float v : h) hs3 += v;
    report(cmn.val == -3.f && cmn.loc == imin && cmx.val == 3.f && cmx.loc == imax &&
               std::fabs(cs3 - hs3) <= 1e-9 * std::fabs(hs3) + 1e-9,
           "mdrange_combined_minloc_maxloc_sum");
  }
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
  // the reference's tile-list constructor with Iterate::Right on a LayoutRight
  // view, and the deduction guide of a braced-list policy
  // (KokkosExp_MDRangePolicy.hpp:283-307, 429-458)
  {
    Kokkos::View<int32_t***, Kokkos::LayoutRight> z("z", 33, 17, 65);
    Kokkos::parallel_for(
        Kokkos::MDRangePolicy<Kokkos::Rank<3, Kokkos::Iterate::Right, Kokkos::Iterate::Right>>({0, 0, 0}, {33, 17, 65},
                                                                                            {2, 4, 32}),
        KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k) { z(i, j, k) = (int32_t)(i * 10000 + j * 100 + k); });
    int64_t zs = 0;
    Kokkos::parallel_reduce(Kokkos::MDRangePolicy({0, 0, 0}, {33, 17, 65}),
                            KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, int64_t& u) { u += z(i, j, k); }, zs);
    int64_t hz = 0;
    for (int64_t i = 0; i < 33; ++i)
      for (int64_t j = 0; j < 17; ++j)
        for (int64_t k = 0; k < 65; ++k) hz += i * 10000 + j * 100 + k;
    report(zs == hz, "mdrange_tiles_iterate_right_ctad");
    bool threw = false;
    try {
      Kokkos::MDRangePolicy<Kokkos::Rank<3>> bad({0, 0, 0}, {8, 8, 8}, {16, 16, 16});  // 4096 threads in a tile
    } catch (const std::runtime_error&) {
      threw = true;
    }
    report(threw, "mdrange_tile_too_large_rejected");
  }
  // ranks 5 and 6 (the reference's maximum, KokkosExp_MDRangePolicy.hpp:196)
  {
    Kokkos::View<int32_t*****> a5("a5", 3, 4, 5, 6, 7);
    Kokkos::parallel_for(Kokkos::MDRangePolicy<Kokkos::Rank<5>>({0, 0, 0, 0, 0}, {3, 4, 5, 6, 7}),
                         KOKKOS_LAMBDA(int64_t a, int64_t b, int64_t c, int64_t d, int64_t e) {
                           a5(a, b, c, d, e) = (int32_t)(a + 3 * b + 5 * c + 7 * d + 11 * e);
                         });
    Kokkos::View<double******, Kokkos::LayoutRight> a6("a6", 2, 3, 4, 3, 2, 5);
    Kokkos::parallel_for(
        Kokkos::MDRangePolicy<Kokkos::Rank<6, Kokkos::Iterate::Right, Kokkos::Iterate::Right>>({0, 0, 0, 0, 0, 0},
                                                                                            {2, 3, 4, 3, 2, 5}),
        KOKKOS_LAMBDA(int64_t a, int64_t b, int64_t c, int64_t d, int64_t e, int64_t f) {
          a6(a, b, c, d, e, f) = (double)(a + b * 2 + c * 4 + d * 8 + e * 16 + f * 32);
        });
    int64_t s5 = 0;
    double s6 = 0;
    Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<5>>({1, 0, 2, 0, 3}, {3, 4, 5, 6, 7}),
                            KOKKOS_LAMBDA(int64_t a, int64_t b, int64_t c, int64_t d, int64_t e, int64_t& u) {
                              u += a5(a, b, c, d, e);
                            },
                            s5);
    Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<6>>({0, 0, 0, 0, 0, 0}, {2, 3, 4, 3, 2, 5}),
                            KOKKOS_LAMBDA(int64_t a, int64_t b, int64_t c, int64_t d, int64_t e, int64_t f, double& u) {
                              u += a6(a, b, c, d, e, f);
                            },
                            s6);
    int64_t h5 = 0;
    for (int64_t a = 1; a < 3; ++a)
      for (int64_t b = 0; b < 4; ++b)
        for (int64_t c = 2; c < 5; ++c)
          for (int64_t d = 0; d < 6; ++d)
            for (int64_t e = 3; e < 7; ++e) h5 += a + 3 * b + 5 * c + 7 * d + 11 * e;
    double h6 = 0;
    for (int64_t a = 0; a < 2; ++a)
      for (int64_t b = 0; b < 3; ++b)
        for (int64_t c = 0; c < 4; ++c)
          for (int64_t d = 0; d < 3; ++d)
            for (int64_t e = 0; e < 2; ++e)
              for (int64_t f = 0; f < 5; ++f) h6 += (double)(a + b * 2 + c * 4 + d * 8 + e * 16 + f * 32);
    report(s5 == h5 && s6 == h6, "mdrange_rank5_rank6");
  }
  // a work tag among the policy's properties
  {
    int64_t t = 0;
    Kokkos::parallel_reduce(Kokkos::MDRangePolicy<Kokkos::Rank<2>, TagSq>({0, 0}, {100, 50}), Sq{}, t);
    report(t == (int64_t)(99 * 100 / 2) * (49 * 50 / 2), "mdrange_work_tag");
  }
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
  // A league longer than one CTA per rank allows (2^20 CTAs; the rest stride
  // over them) and long TeamThreadRange ranges (the 32-, 8- and 1-call steps).
  {
    const int64_t big = (int64_t(1) << 20) + 37;
    Kokkos::View<int64_t*> marks("marks", big);
    Kokkos::parallel_for(TP(big, 32), KOKKOS_LAMBDA(const TP::member_type& t) {
      Kokkos::single(Kokkos::PerTeam(t), [&]() { marks(t.league_rank()) = t.league_rank() * 3 + 1; });
    });
    int64_t msum = 0;
    Kokkos::parallel_reduce(TP(big, 64), KOKKOS_LAMBDA(const TP::member_type& t, int64_t& u) {
      if (t.team_rank() == 0) u += marks(t.league_rank());
    }, msum);
    const int64_t want = 3 * (big * (big - 1) / 2) + big;
    auto hm = to_host(marks);
    bool okm = msum == want;
    for (int64_t r = 0; r < big; r += 4093) okm = okm && hm[r] == r * 3 + 1;
    okm = okm && hm[big - 1] == (big - 1) * 3 + 1;
    report(okm, "team_league_beyond_grid");
    const int64_t len = 1000003;
    Kokkos::View<int64_t*> lv("lv", len);
    Kokkos::parallel_for(Kokkos::RangePolicy<>(0, len), KOKKOS_LAMBDA(int64_t i) { lv(i) = i % 1013; });
    Kokkos::View<int64_t*> ls("ls", 3);
    Kokkos::parallel_for(TP(3, 256), KOKKOS_LAMBDA(const TP::member_type& t) {
      const int64_t b = t.league_rank() * 7, e = len - t.league_rank() * 5;
      int64_t acc = 0;
      Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, b, e), [&](int64_t i, int64_t& w) { w += lv(i); }, acc);
      Kokkos::single(Kokkos::PerTeam(t), [&]() { ls(t.league_rank()) = acc; });
    });
    auto hl = to_host(ls);
    bool okl = true;
    for (int64_t r = 0; r < 3; ++r) {
      int64_t e = 0;
      for (int64_t i = r * 7; i < len - r * 5; ++i) e += i % 1013;
      okl = okl && hl[r] == e;
    }
    report(okl, "team_thread_range_long");
  }
  int64_t lsum2 = 0, lcnt = 0;
  Kokkos::parallel_reduce(TP(league, 128), KOKKOS_LAMBDA(const TP::member_type& t, int64_t& u, int64_t& c) {
    const int64_t s = t.league_rank();
    int64_t ts = 0;
    Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, doff(s), doff(s + 1)),
                            [&](int64_t i, int64_t& w) { w += dv(i); }, ts);
    if (t.team_rank() == 0) {
      u += ts;
      c += 1;
    }
  }, lsum2, lcnt);
  report(lsum2 == tot && lcnt == league, "team_combined_reduce");
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

static void test_team_collectives() {
  // TestTeamScan.hpp / TestTeamReductionScan.hpp style: member team_reduce
  // (Sum and MaxLoc), team_scan with and without a global accumulator,
  // team_broadcast
  using TP = Kokkos::TeamPolicy<>;
  const int64_t league = 300;
  const int ts = 128;
  Kokkos::View<int64_t*> red("red", league), mloc("mloc", league), scan("scan", league * ts),
      gscan("gscan", league * ts), bc("bc", league * ts), gacc("gacc", 1);
  Kokkos::parallel_for(TP(league, ts), KOKKOS_LAMBDA(const TP::member_type& t) {
    const int64_t lr = t.league_rank();
    const int r = t.team_rank();
    const int64_t v = (lr * 7 + r * 3) % 11;
    int64_t s = v;
    t.team_reduce(Kokkos::Sum<int64_t>(s));
    Kokkos::ValLocScalar<int64_t, int> vl{v, r};
    t.team_reduce(Kokkos::MaxLoc<int64_t, int>(vl));
    if (r == 0) {
      red(lr) = s;
      mloc(lr) = vl.loc;
    }
    scan(lr * ts + r) = t.team_scan(v);
    gscan(lr * ts + r) = t.team_scan(v, &gacc(0));
    int64_t b = r * 10 + lr;
    t.team_broadcast(b, 5);
    bc(lr * ts + r) = b;
  });
  auto hred = to_host(red), hml = to_host(mloc), hs = to_host(scan), hg = to_host(gscan), hb = to_host(bc),
       ha = to_host(gacc);
  bool ok_red = true, ok_ml = true, ok_scan = true, ok_bc = true, ok_g = true;
  int64_t total = 0;
  std::vector<std::pair<int64_t, int64_t>> bases;  // (global base, team total) per team
  for (int64_t lr = 0; lr < league; ++lr) {
    int64_t run = 0, best = -1, bl = 0;
    for (int r = 0; r < ts; ++r) {
      const int64_t v = (lr * 7 + r * 3) % 11;
      ok_scan = ok_scan && hs[lr * ts + r] == run;
      ok_bc = ok_bc && hb[lr * ts + r] == 50 + lr;
      // global: the team's base plus the in-team exclusive prefix
      ok_g = ok_g && hg[lr * ts + r] - hg[lr * ts] == run;
      if (v > best) { best = v; bl = r; }
      run += v;
    }
    ok_red = ok_red && hred[lr] == run;
    ok_ml = ok_ml && hml[lr] == bl;
    total += run;
    bases.push_back({hg[lr * ts], run});
  }
  // the team bases are the exclusive prefix of the team totals in some order
  std::sort(bases.begin(), bases.end());
  int64_t acc = 0;
  for (auto& p : bases) { ok_g = ok_g && p.first == acc; acc += p.second; }
  report(ok_red, "team_reduce_sum");
  report(ok_ml, "team_reduce_maxloc_first");
  report(ok_scan, "team_scan_exclusive");
  report(ok_g && ha[0] == total, "team_scan_global_accum");
  report(ok_bc, "team_broadcast");
}

static void test_std_more() {
  // TestStdAlgorithmsMinMaxElementOps.cpp / TestStdAlgorithmsTransformReduce /
  // TestStdAlgorithmsTransform{Inclusive,Exclusive}Scan style: host std:: results
  namespace KE = Kokkos::Experimental;
  KE::GB300 ex;
  Rng r{21};
  const int64_t n = (1 << 20) + 3;
  std::vector<int32_t> x(n);
  for (auto& v : x) v = (int32_t)(r.next() % 1000) - 500;
  std::vector<float> f(n);
  for (auto& v : f) v = (float)((int)(r.next() % 200) - 100);
  auto dx = to_device(x);
  auto df = to_device(f);
  const int64_t imin = KE::min_element(ex, KE::cbegin(dx), KE::cend(dx)) - KE::cbegin(dx);
  const int64_t imax = KE::max_element(ex, KE::cbegin(dx), KE::cend(dx)) - KE::cbegin(dx);
  report(imin == std::min_element(x.begin(), x.end()) - x.begin(), "std_min_element_first");
  report(imax == std::max_element(x.begin(), x.end()) - x.begin(), "std_max_element_first");
  auto absless = KOKKOS_LAMBDA(float a, float b) { return (a < 0 ? -a : a) < (b < 0 ? -b : b); };
  auto habsless = [](float a, float b) { return std::fabs(a) < std::fabs(b); };
  const int64_t cmin = KE::min_element(ex, KE::cbegin(df), KE::cend(df), absless) - KE::cbegin(df);
  report(cmin == std::min_element(f.begin(), f.end(), habsless) - f.begin(), "std_min_element_comparator");
  auto mm = KE::minmax_element(ex, KE::cbegin(dx), KE::cend(dx));
  auto hmm = std::minmax_element(x.begin(), x.end());
  report(mm.first - KE::cbegin(dx) == hmm.first - x.begin() && mm.second - KE::cbegin(dx) == hmm.second - x.begin(),
         "std_minmax_element_first_min_last_max");
  auto mmc = KE::minmax_element(ex, KE::cbegin(df), KE::cend(df), absless);
  auto hmmc = std::minmax_element(f.begin(), f.end(), habsless);
  report(mmc.first - KE::cbegin(df) == hmmc.first - f.begin() && mmc.second - KE::cbegin(df) == hmmc.second - f.begin(),
         "std_minmax_element_comparator");
  // transform_reduce: sum of squares (unary), dot product (binary default), max of products (custom)
  std::vector<int64_t> y(n);
  for (auto& v : y) v = (int64_t)(r.next() % 64) - 32;
  auto dy = to_device(y);
  auto plus = KOKKOS_LAMBDA(int64_t a, int64_t b) { return a + b; };
  auto sq = KOKKOS_LAMBDA(int32_t a) { return (int64_t)a * a; };
  int64_t hsq = 11, hdot = -5, hmx = std::numeric_limits<int64_t>::min();
  for (int64_t i = 0; i < n; ++i) {
    hsq += (int64_t)x[i] * x[i];
    hdot += (int64_t)x[i] * y[i];
    hmx = std::max(hmx, (int64_t)x[i] * y[i]);
  }
  report(KE::transform_reduce(ex, KE::cbegin(dx), KE::cend(dx), (int64_t)11, plus, sq) == hsq,
         "std_transform_reduce_unary");
  report(KE::transform_reduce(ex, KE::cbegin(dx), KE::cend(dx), KE::cbegin(dy), (int64_t)-5) == hdot,
         "std_transform_reduce_dot");
  auto mx = KOKKOS_LAMBDA(int64_t a, int64_t b) { return a > b ? a : b; };
  auto mul = KOKKOS_LAMBDA(int32_t a, int64_t b) { return (int64_t)a * b; };
  report(KE::transform_reduce(ex, KE::cbegin(dx), KE::cend(dx), KE::cbegin(dy), std::numeric_limits<int64_t>::min(),
                              mx, mul) == hmx,
         "std_transform_reduce_binary_custom");
  report(KE::reduce(ex, KE::cbegin(dy), KE::cend(dy), (int64_t)-1000, mx) ==
             *std::max_element(y.begin(), y.end()),
         "std_reduce_custom_joiner");
  // scans with a binary op: transform_exclusive_scan (plus, x*2, init 5), transform_inclusive_scan
  // with init, inclusive_scan with max (running maximum)
  Kokkos::View<int64_t*> o1("o1", n), o2("o2", n), o3("o3", n);
  auto dbl = KOKKOS_LAMBDA(int32_t a) { return (int64_t)2 * a; };
  KE::transform_exclusive_scan(ex, KE::cbegin(dx), KE::cend(dx), KE::begin(o1), (int64_t)5, plus, dbl);
  KE::transform_inclusive_scan(ex, KE::cbegin(dx), KE::cend(dx), KE::begin(o2), plus, dbl, (int64_t)-7);
  KE::inclusive_scan(ex, KE::cbegin(dy), KE::cend(dy), KE::begin(o3), mx);
  auto h1 = to_host(o1), h2 = to_host(o2), h3 = to_host(o3);
  bool ok1 = h1[0] == 5, ok2 = true, ok3 = true;
  int64_t ex1 = 0, in2 = 0, rm = std::numeric_limits<int64_t>::min();
  for (int64_t i = 0; i < n; ++i) {
    if (i > 0) ok1 = ok1 && h1[i] == ex1 + 5;
    ex1 += 2 * (int64_t)x[i];
    in2 += 2 * (int64_t)x[i];
    ok2 = ok2 && h2[i] == in2 - 7;
    rm = std::max(rm, y[i]);
    ok3 = ok3 && h3[i] == rm;
  }
  report(ok1, "std_transform_exclusive_scan");
  report(ok2, "std_transform_inclusive_scan_init");
  report(ok3, "std_inclusive_scan_custom_op");
}

static void test_unordered_map() {
  // TestUnorderedMap.hpp / TestBitset.hpp style: inserts with duplicates
  // (success vs existing counts), find / exists / key_at / value_at,
  // AtomicAdd accumulation, a full table then rehash, erase, Bitset.
  const int64_t n = 1 << 20;
  const uint64_t nkeys = 1 << 18;  // every residue of i * odd mod 2^18 appears 4 times
  Kokkos::UnorderedMap<uint64_t, int64_t> map((uint32_t)nkeys);
  Kokkos::View<int64_t*> cnt("cnt", 3);
  Kokkos::parallel_for(n, KOKKOS_LAMBDA(int64_t i) {
    const uint64_t r = ((uint64_t)i * 2654435761ull) % nkeys;
    const auto res = map.insert(r * 7919ull + 13ull, (int64_t)i);
    Kokkos::atomic_add(&cnt(res.success() ? 0 : res.existing() ? 1 : 2), (int64_t)1);
  });
  auto hc = to_host(cnt);
  report(hc[0] == (int64_t)nkeys && hc[1] == n - (int64_t)nkeys && hc[2] == 0 && map.size() == nkeys &&
             !map.failed_insert() && map.capacity() >= nkeys,
         "unordered_map_insert_success_existing");
  int64_t bad = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, (int64_t)nkeys), KOKKOS_LAMBDA(int64_t r, int64_t& u) {
    const uint64_t k = (uint64_t)r * 7919ull + 13ull;
    const uint32_t idx = map.find(k);
    const bool ok = map.valid_at(idx) && map.key_at(idx) == k &&
                    ((uint64_t)map.value_at(idx) * 2654435761ull) % nkeys == (uint64_t)r &&
                    !map.exists(k + 1);
    u += ok ? 0 : 1;
  }, bad);
  report(bad == 0, "unordered_map_find_exists_values");
  // AtomicAdd: a histogram of i % 3001 in a map
  Kokkos::UnorderedMap<int32_t, int64_t> hist(4096);
  using AddOp = Kokkos::UnorderedMapInsertOpTypes<Kokkos::View<int64_t*>, uint32_t>::AtomicAdd;
  Kokkos::parallel_for(n, KOKKOS_LAMBDA(int64_t i) { hist.insert((int32_t)(i % 3001), (int64_t)1, AddOp()); });
  bad = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, 3001), KOKKOS_LAMBDA(int64_t k, int64_t& u) {
    const uint32_t idx = hist.find((int32_t)k);
    const int64_t want = n / 3001 + (k < n % 3001 ? 1 : 0);
    u += (hist.valid_at(idx) && hist.value_at(idx) == want) ? 0 : 1;
  }, bad);
  report(bad == 0 && hist.size() == 3001, "unordered_map_atomic_add");
  // a set that overflows, then rehash and erase
  Kokkos::UnorderedMap<uint32_t, void> set(100);
  const uint32_t cap0 = set.capacity();
  Kokkos::parallel_for(1000, KOKKOS_LAMBDA(int64_t i) { set.insert((uint32_t)(i * 3 + 1)); });
  const bool full = set.failed_insert() && set.size() == cap0;
  const bool grown = set.rehash(2000);
  set.reset_failed_insert_flag();
  Kokkos::parallel_for(1000, KOKKOS_LAMBDA(int64_t i) { set.insert((uint32_t)(i * 3 + 1)); });
  report(full && grown && !set.failed_insert() && set.size() == 1000 && set.capacity() >= 2000,
         "unordered_set_full_then_rehash");
  set.begin_erase();
  Kokkos::parallel_for(1000, KOKKOS_LAMBDA(int64_t i) {
    if (i % 2 == 0) set.erase((uint32_t)(i * 3 + 1));
  });
  set.end_erase();
  bad = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, 1000), KOKKOS_LAMBDA(int64_t i, int64_t& u) {
    u += set.exists((uint32_t)(i * 3 + 1)) == (i % 2 == 1) ? 0 : 1;
  }, bad);
  report(bad == 0 && set.size() == 500, "unordered_set_erase");
  // Bitset
  const unsigned nb = 1000003;
  Kokkos::Bitset<> bs(nb);
  Kokkos::parallel_for((int64_t)nb, KOKKOS_LAMBDA(int64_t i) {
    if (i % 3 == 0) bs.set((unsigned)i);
  });
  const unsigned c3 = bs.count();
  Kokkos::parallel_for((int64_t)nb, KOKKOS_LAMBDA(int64_t i) {
    if (i % 6 == 0) bs.reset((unsigned)i);
  });
  const unsigned c6 = bs.count();
  bad = 0;
  Kokkos::parallel_reduce(Kokkos::RangePolicy<>(0, (int64_t)nb), KOKKOS_LAMBDA(int64_t i, int64_t& u) {
    const bool want = (i % 3 == 0) && (i % 6 != 0);
    u += bs.test((unsigned)i) == want ? 0 : 1;
    if (i % 977 == 0) {
      const auto f = bs.find_any_unset_near((unsigned)i);
      const auto g = bs.find_any_set_near((unsigned)i);
      u += (!f.first || !bs.test(f.second)) ? 0 : 1;
      u += (!g.first || bs.test(g.second)) ? 0 : 1;
    }
  }, bad);
  bs.set();
  const unsigned call = bs.count();
  bs.reset();
  report(c3 == (nb + 2) / 3 && c6 == (nb + 2) / 3 - (nb + 5) / 6 && bad == 0 && call == nb && bs.count() == 0,
         "bitset_set_reset_count_find");
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
    test_team_collectives();
    test_std_more();
    test_unordered_map();
    test_graph();
    test_errors();
  }
  Kokkos::finalize();
  std::printf("%s (%d failures)\n", g_fail ? "SOME FAILED" : "ALL PASS", g_fail);
  return g_fail ? 1 : 0;
}
