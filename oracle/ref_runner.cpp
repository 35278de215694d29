// ORACLE — test infrastructure only.
//
// Drives the reference Kokkos OpenMP backend (built from its own sources by
// oracle/ref.mk) through its public API on inputs read from a file and
// writes the results, so that golden vectors come from the reference itself.
// Used by tests/golden/make_golden.py in a container that holds the
// reference sources; never shipped or called by the product.
//
//   ref_runner <nthreads> <command> <in.bin> <out.bin> [args...]
//
// commands:
//   reduce <op> <dtype> <n>                 parallel_reduce + built-in reducer
//   stdreduce_f64 <n>                       Experimental::reduce(ex, first, last, 0.0)
//   exscan_i32_i64 <n> <init>               Experimental::exclusive_scan (i32 -> i64)
//   inscan <dtype> <n>                      Experimental::inclusive_scan (same type)
//   scan_total_i64 <n>                      parallel_scan with total (i64)
//   mdrange <op> <dtype> <n0> <n1> <n2> [reps]  MDRangePolicy<Rank<3>> over LayoutLeft View<T***>
//                                           (run reps times: the same result each time)
//   hist <n> <nbins>                        ScatterView histogram into int64 bins
//   sort_u64 <n>                            Kokkos::sort
//   sort_pairs_stable <n>                   Kokkos::sort of (key, index) pairs with a comparator
//   sort_by_key <n>                         Experimental::sort_by_key (u64 keys, i32 values)
//   binsort <n> <nbins> <kmin> <kmax>       BinSort + BinOp1D: counts, offsets, permutation
//   team_reduce_sum_f64 <nseg>              TeamPolicy league reduce: per-segment sums (offsets input)
//   algos_i64 <n>                           std transform_reduce (unary, binary), min/max/minmax_element,
//                                           transform_exclusive_scan, transform_inclusive_scan
//   team_scan_i32 <nseg>                    TeamThreadRange parallel_scan per league rank (offsets input)
//   umap_count <n> <capacity>               UnorderedMap<int32,int64> insert with AtomicAdd: key counts
#include <Kokkos_Core.hpp>
#include <Kokkos_ScatterView.hpp>
#include <Kokkos_Sort.hpp>
#include <Kokkos_StdAlgorithms.hpp>
#include <Kokkos_UnorderedMap.hpp>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace KE = Kokkos::Experimental;
using Exec = Kokkos::OpenMP;
using HostMem = Kokkos::HostSpace;

static std::vector<unsigned char> read_all(const char* path) {
  std::vector<unsigned char> b;
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  b.resize((size_t)sz);
  if (sz && std::fread(b.data(), 1, (size_t)sz, f) != (size_t)sz) { std::exit(2); }
  std::fclose(f);
  return b;
}

static void write_all(const char* path, const void* p, size_t n) {
  FILE* f = std::fopen(path, "wb");
  if (!f) { std::perror(path); std::exit(2); }
  if (n && std::fwrite(p, 1, n, f) != n) std::exit(2);
  std::fclose(f);
}

template <class T>
Kokkos::View<T*, HostMem> to_view(const std::vector<unsigned char>& b, int64_t n) {
  Kokkos::View<T*, HostMem> v("in", n);
  std::memcpy(v.data(), b.data(), sizeof(T) * (size_t)n);
  return v;
}

// ---- reduce ----------------------------------------------------------------
template <class T>
void run_reduce(int op, int64_t n, const std::vector<unsigned char>& in, const char* outp) {
  auto x = to_view<T>(in, n);
  Kokkos::RangePolicy<Exec> pol(0, n);
  switch (op) {
    case 0: { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { u += x(i); }, Kokkos::Sum<T>(r)); write_all(outp, &r, sizeof r); break; }
    case 1: { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { u *= x(i); }, Kokkos::Prod<T>(r)); write_all(outp, &r, sizeof r); break; }
    case 2: { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { if (x(i) < u) u = x(i); }, Kokkos::Min<T>(r)); write_all(outp, &r, sizeof r); break; }
    case 3: { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { if (x(i) > u) u = x(i); }, Kokkos::Max<T>(r)); write_all(outp, &r, sizeof r); break; }
    case 4: if constexpr (std::is_integral_v<T>) { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { u = u && x(i); }, Kokkos::LAnd<T>(r)); write_all(outp, &r, sizeof r); } break;
    case 5: if constexpr (std::is_integral_v<T>) { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { u = u || x(i); }, Kokkos::LOr<T>(r)); write_all(outp, &r, sizeof r); } break;
    case 6: if constexpr (std::is_integral_v<T>) { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { u = u & x(i); }, Kokkos::BAnd<T>(r)); write_all(outp, &r, sizeof r); } break;
    case 7: if constexpr (std::is_integral_v<T>) { T r; Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, T& u) { u = u | x(i); }, Kokkos::BOr<T>(r)); write_all(outp, &r, sizeof r); } break;
    case 8: {
      using V = typename Kokkos::MinLoc<T, int64_t>::value_type; V r;
      Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, V& u) { if (x(i) < u.val) { u.val = x(i); u.loc = i; } }, Kokkos::MinLoc<T, int64_t>(r));
      write_all(outp, &r, sizeof r); break; }
    case 9: {
      using V = typename Kokkos::MaxLoc<T, int64_t>::value_type; V r;
      Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, V& u) { if (x(i) > u.val) { u.val = x(i); u.loc = i; } }, Kokkos::MaxLoc<T, int64_t>(r));
      write_all(outp, &r, sizeof r); break; }
    case 10: {
      using V = typename Kokkos::MinMax<T>::value_type; V r;
      Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, V& u) { if (x(i) < u.min_val) u.min_val = x(i); if (x(i) > u.max_val) u.max_val = x(i); }, Kokkos::MinMax<T>(r));
      write_all(outp, &r, sizeof r); break; }
    case 11: {
      using V = typename Kokkos::MinMaxLoc<T, int64_t>::value_type; V r;
      Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, V& u) {
        if (x(i) < u.min_val) { u.min_val = x(i); u.min_loc = i; }
        if (x(i) > u.max_val) { u.max_val = x(i); u.max_loc = i; } }, Kokkos::MinMaxLoc<T, int64_t>(r));
      write_all(outp, &r, sizeof r); break; }
    default: std::exit(3);
  }
}

// ---- MDRange over LayoutLeft View<T***>; loc = i + n0*(j + n1*k) --------------
template <class T>
void run_mdrange(int op, int64_t n0, int64_t n1, int64_t n2, const std::vector<unsigned char>& in, const char* outp,
                 int reps) {
  for (int rep = 1; rep < reps; ++rep) run_mdrange<T>(op, n0, n1, n2, in, outp, 1);
  Kokkos::View<T***, Kokkos::LayoutLeft, HostMem> x("x", n0, n1, n2);
  std::memcpy(x.data(), in.data(), sizeof(T) * (size_t)(n0 * n1 * n2));
  Kokkos::MDRangePolicy<Exec, Kokkos::Rank<3>> pol({0, 0, 0}, {n0, n1, n2});
  if (op == 0) {
    T r;
    Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, T& u) { u += x(i, j, k); }, Kokkos::Sum<T>(r));
    write_all(outp, &r, sizeof r);
  } else if (op == 8) {
    using V = typename Kokkos::MinLoc<T, int64_t>::value_type; V r;
    Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, V& u) {
      if (x(i, j, k) < u.val) { u.val = x(i, j, k); u.loc = i + n0 * (j + n1 * k); } }, Kokkos::MinLoc<T, int64_t>(r));
    write_all(outp, &r, sizeof r);
  } else if (op == 9) {
    using V = typename Kokkos::MaxLoc<T, int64_t>::value_type; V r;
    Kokkos::parallel_reduce(pol, KOKKOS_LAMBDA(int64_t i, int64_t j, int64_t k, V& u) {
      if (x(i, j, k) > u.val) { u.val = x(i, j, k); u.loc = i + n0 * (j + n1 * k); } }, Kokkos::MaxLoc<T, int64_t>(r));
    write_all(outp, &r, sizeof r);
  } else {
    std::exit(3);
  }
}

struct KeyIdx { uint64_t key; int64_t idx; };

int main(int argc, char** argv) {
  if (argc < 5) { std::fprintf(stderr, "usage: ref_runner <nthreads> <cmd> <in> <out> ...\n"); return 1; }
  const int nthreads = std::atoi(argv[1]);
  const std::string cmd = argv[2];
  const char* inp = argv[3];
  const char* outp = argv[4];
  auto a = [&](int i) { return std::atoll(argv[5 + i]); };
  Kokkos::initialize(Kokkos::InitializationSettings().set_num_threads(nthreads));
  {
    const std::vector<unsigned char> in = read_all(inp);
    if (cmd == "reduce") {
      const int op = (int)a(0), dt = (int)a(1);
      const int64_t n = a(2);
      switch (dt) {
        case 0: run_reduce<int32_t>(op, n, in, outp); break;
        case 1: run_reduce<int64_t>(op, n, in, outp); break;
        case 2: run_reduce<uint32_t>(op, n, in, outp); break;
        case 3: run_reduce<uint64_t>(op, n, in, outp); break;
        case 4: run_reduce<float>(op, n, in, outp); break;
        case 5: run_reduce<double>(op, n, in, outp); break;
      }
    } else if (cmd == "stdreduce_f64") {
      const int64_t n = a(0);
      auto x = to_view<double>(in, n);
      double r = KE::reduce(Exec(), KE::cbegin(x), KE::cend(x), 0.0);
      write_all(outp, &r, sizeof r);
    } else if (cmd == "exscan_i32_i64") {
      const int64_t n = a(0);
      const int64_t init = a(1);
      auto x = to_view<int32_t>(in, n);
      Kokkos::View<int64_t*, HostMem> y("y", n);
      KE::exclusive_scan(Exec(), KE::cbegin(x), KE::cend(x), KE::begin(y), init);
      write_all(outp, y.data(), sizeof(int64_t) * (size_t)n);
    } else if (cmd == "inscan") {
      const int dt = (int)a(0);
      const int64_t n = a(1);
      if (dt == 0) {
        auto x = to_view<int32_t>(in, n);
        Kokkos::View<int32_t*, HostMem> y("y", n);
        KE::inclusive_scan(Exec(), KE::cbegin(x), KE::cend(x), KE::begin(y));
        write_all(outp, y.data(), sizeof(int32_t) * (size_t)n);
      } else if (dt == 5) {
        auto x = to_view<double>(in, n);
        Kokkos::View<double*, HostMem> y("y", n);
        KE::inclusive_scan(Exec(), KE::cbegin(x), KE::cend(x), KE::begin(y));
        write_all(outp, y.data(), sizeof(double) * (size_t)n);
      } else std::exit(3);
    } else if (cmd == "scan_total_i64") {
      const int64_t n = a(0);
      auto x = to_view<int64_t>(in, n);
      Kokkos::View<int64_t*, HostMem> y("y", n + 1);
      int64_t total = 0;
      Kokkos::parallel_scan(Kokkos::RangePolicy<Exec>(0, n),
                            KOKKOS_LAMBDA(int64_t i, int64_t& u, bool fin) { if (fin) y(i) = u; u += x(i); }, total);
      y(n) = total;
      write_all(outp, y.data(), sizeof(int64_t) * (size_t)(n + 1));
    } else if (cmd == "mdrange") {
      const int op = (int)a(0), dt = (int)a(1);
      const int reps = argc > 10 ? (int)a(5) : 1;
      if (dt == 4) run_mdrange<float>(op, a(2), a(3), a(4), in, outp, reps);
      else if (dt == 5) run_mdrange<double>(op, a(2), a(3), a(4), in, outp, reps);
      else std::exit(3);
    } else if (cmd == "hist") {
      const int64_t n = a(0), nb = a(1);
      auto keys = to_view<int32_t>(in, n);
      Kokkos::View<int64_t*, HostMem> bins("bins", nb);
      auto sv = Kokkos::Experimental::create_scatter_view(bins);
      Kokkos::parallel_for(Kokkos::RangePolicy<Exec>(0, n), KOKKOS_LAMBDA(int64_t i) {
        auto acc = sv.access();
        acc(keys(i)) += 1;
      });
      Kokkos::Experimental::contribute(bins, sv);
      write_all(outp, bins.data(), sizeof(int64_t) * (size_t)nb);
    } else if (cmd == "sort_u64") {
      const int64_t n = a(0);
      auto k = to_view<uint64_t>(in, n);
      Kokkos::sort(Exec(), k);
      write_all(outp, k.data(), sizeof(uint64_t) * (size_t)n);
    } else if (cmd == "sort_pairs_stable") {
      const int64_t n = a(0);
      Kokkos::View<KeyIdx*, HostMem> p("p", n);
      const uint64_t* src = (const uint64_t*)in.data();
      for (int64_t i = 0; i < n; ++i) p(i) = KeyIdx{src[i], i};
      struct Cmp {
        KOKKOS_FUNCTION bool operator()(const KeyIdx& x, const KeyIdx& y) const {
          return x.key < y.key || (x.key == y.key && x.idx < y.idx);
        }
      };
      Kokkos::sort(Exec(), p, Cmp{});
      std::vector<int32_t> perm((size_t)n);
      for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)p(i).idx;
      write_all(outp, perm.data(), sizeof(int32_t) * (size_t)n);
    } else if (cmd == "sort_by_key") {
      const int64_t n = a(0);
      auto k = to_view<uint64_t>(in, n);
      Kokkos::View<int32_t*, HostMem> v("v", n);
      for (int64_t i = 0; i < n; ++i) v(i) = (int32_t)i;
      KE::sort_by_key(Exec(), k, v);
      std::vector<unsigned char> o(sizeof(uint64_t) * n + sizeof(int32_t) * n);
      std::memcpy(o.data(), k.data(), sizeof(uint64_t) * (size_t)n);
      std::memcpy(o.data() + sizeof(uint64_t) * n, v.data(), sizeof(int32_t) * (size_t)n);
      write_all(outp, o.data(), o.size());
    } else if (cmd == "binsort") {
      const int64_t n = a(0);
      const int nb = (int)a(1);
      const uint64_t kmin = (uint64_t)a(2), kmax = (uint64_t)a(3);
      auto k = to_view<uint64_t>(in, n);
      using Op = Kokkos::BinOp1D<decltype(k)>;
      Op op(nb, kmin, kmax);
      Kokkos::BinSort<decltype(k), Op> bs(k, op, false);
      bs.create_permute_vector(Exec());
      auto cnt = bs.get_bin_count();
      auto off = bs.get_bin_offsets();
      auto perm = bs.get_permute_vector();
      const int64_t nbb = op.max_bins();
      std::vector<int64_t> o;
      o.push_back(nbb);
      double mul = op.mul_;
      int64_t mbits;
      std::memcpy(&mbits, &mul, 8);
      o.push_back(mbits);
      for (int64_t b = 0; b < nbb; ++b) o.push_back(cnt(b));
      for (int64_t b = 0; b < nbb; ++b) o.push_back((int64_t)off(b));
      for (int64_t i = 0; i < n; ++i) o.push_back((int64_t)perm(i));
      write_all(outp, o.data(), sizeof(int64_t) * o.size());
    } else if (cmd == "team_reduce_sum_f64") {
      // input: nseg+1 int64 offsets followed by the doubles
      const int64_t nseg = a(0);
      const int64_t* offs = (const int64_t*)in.data();
      const int64_t n = offs[nseg];
      Kokkos::View<int64_t*, HostMem> o("o", nseg + 1);
      std::memcpy(o.data(), offs, sizeof(int64_t) * (size_t)(nseg + 1));
      Kokkos::View<double*, HostMem> x("x", n);
      std::memcpy(x.data(), in.data() + sizeof(int64_t) * (nseg + 1), sizeof(double) * (size_t)n);
      Kokkos::View<double*, HostMem> r("r", nseg);
      using TP = Kokkos::TeamPolicy<Exec>;
      Kokkos::parallel_for(TP(nseg, Kokkos::AUTO), KOKKOS_LAMBDA(const TP::member_type& t) {
        const int64_t s = t.league_rank();
        double v = 0;
        Kokkos::parallel_reduce(Kokkos::TeamThreadRange(t, o(s), o(s + 1)), [&](int64_t i, double& u) { u += x(i); }, v);
        Kokkos::single(Kokkos::PerTeam(t), [&]() { r(s) = v; });
      });
      write_all(outp, r.data(), sizeof(double) * (size_t)nseg);
    } else if (cmd == "algos_i64") {
      // out: [transform_reduce(x, 3, +, v*v%1009), min_element, max_element,
      //       minmax_element first, second, transform_reduce(x, x, 11) (dot),
      //       transform_exclusive_scan(x, 5, +, 2v+1)[n], transform_inclusive_scan(x, +, v%7)[n]]
      const int64_t n = a(0);
      auto x = to_view<int64_t>(in, n);
      Kokkos::View<int64_t*, HostMem> ex("ex", n), inc("inc", n);
      std::vector<int64_t> o;
      o.push_back(KE::transform_reduce(Exec(), KE::cbegin(x), KE::cend(x), int64_t{3},
                                       KOKKOS_LAMBDA(int64_t p, int64_t q) { return p + q; },
                                       KOKKOS_LAMBDA(int64_t v) { return v * v % 1009; }));
      o.push_back(KE::min_element(Exec(), x) - KE::begin(x));
      o.push_back(KE::max_element(Exec(), x) - KE::begin(x));
      auto mm = KE::minmax_element(Exec(), x);
      o.push_back(mm.first - KE::begin(x));
      o.push_back(mm.second - KE::begin(x));
      o.push_back(KE::transform_reduce(Exec(), KE::cbegin(x), KE::cend(x), KE::cbegin(x), int64_t{11}));
      KE::transform_exclusive_scan(Exec(), KE::cbegin(x), KE::cend(x), KE::begin(ex), int64_t{5},
                                   KOKKOS_LAMBDA(int64_t p, int64_t q) { return p + q; },
                                   KOKKOS_LAMBDA(int64_t v) { return 2 * v + 1; });
      KE::transform_inclusive_scan(Exec(), KE::cbegin(x), KE::cend(x), KE::begin(inc),
                                   KOKKOS_LAMBDA(int64_t p, int64_t q) { return p + q; },
                                   KOKKOS_LAMBDA(int64_t v) { return v % 7; });
      for (int64_t i = 0; i < n; ++i) o.push_back(ex(i));
      for (int64_t i = 0; i < n; ++i) o.push_back(inc(i));
      write_all(outp, o.data(), sizeof(int64_t) * o.size());
    } else if (cmd == "team_scan_i32") {
      // input: nseg+1 int64 offsets followed by the int32 values; out: per
      // segment exclusive scan (TeamThreadRange parallel_scan) into int32
      const int64_t nseg = a(0);
      const int64_t* offs = (const int64_t*)in.data();
      const int64_t n = offs[nseg];
      Kokkos::View<int64_t*, HostMem> o("o", nseg + 1);
      std::memcpy(o.data(), offs, sizeof(int64_t) * (size_t)(nseg + 1));
      Kokkos::View<int32_t*, HostMem> x("x", n), y("y", n);
      std::memcpy(x.data(), in.data() + sizeof(int64_t) * (nseg + 1), sizeof(int32_t) * (size_t)n);
      using TP = Kokkos::TeamPolicy<Exec>;
      Kokkos::parallel_for(TP(nseg, Kokkos::AUTO), KOKKOS_LAMBDA(const TP::member_type& t) {
        const int64_t s = t.league_rank();
        Kokkos::parallel_scan(Kokkos::TeamThreadRange(t, o(s), o(s + 1)), [&](int64_t i, int32_t& u, bool fin) {
          if (fin) y(i) = u;
          u += x(i);
        });
      });
      write_all(outp, y.data(), sizeof(int32_t) * (size_t)n);
    } else if (cmd == "umap_count") {
      // out: [size, failed_insert, (key, count) pairs sorted by key]
      const int64_t n = a(0), cap = a(1);
      auto k = to_view<int32_t>(in, n);
      using Map = Kokkos::UnorderedMap<int32_t, int64_t, HostMem>;
      Map m(cap);
      using Op = Kokkos::UnorderedMapInsertOpTypes<Kokkos::View<int64_t*, HostMem>, int32_t>::AtomicAdd;
      Op op;
      Kokkos::parallel_for(Kokkos::RangePolicy<Exec>(0, n), KOKKOS_LAMBDA(int64_t i) { m.insert(k(i), int64_t{1}, op); });
      std::vector<std::pair<int32_t, int64_t>> kv;
      for (uint32_t i = 0; i < m.capacity(); ++i)
        if (m.valid_at(i)) kv.push_back({m.key_at(i), m.value_at(i)});
      std::sort(kv.begin(), kv.end());
      std::vector<int64_t> o;
      o.push_back((int64_t)m.size());
      o.push_back(m.failed_insert() ? 1 : 0);
      for (auto& e : kv) {
        o.push_back(e.first);
        o.push_back(e.second);
      }
      write_all(outp, o.data(), sizeof(int64_t) * o.size());
    } else {
      std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
      Kokkos::finalize();
      return 3;
    }
  }
  Kokkos::finalize();
  return 0;
}
