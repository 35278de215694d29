// The header-template path (include/Kokkos_GB300.hpp) on inputs for which the
// reference produced golden outputs (tests/golden/make_golden.py with
// oracle/ref_runner.cpp): the same calls as the reference runner's commands,
// on the GPU, with the results written in the same layout for
// tests/test_api_golden.py to compare bit for bit.
//
//   test_api_golden algos_i64 <in> <out> <n>
//   test_api_golden team_scan_i32 <in> <out> <nseg>
//   test_api_golden umap_count <in> <out> <n> <capacity>
#include <Kokkos_GB300.hpp>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace KE = Kokkos::Experimental;

static std::vector<unsigned char> read_all(const char* path) {
  std::vector<unsigned char> b;
  FILE* f = std::fopen(path, "rb");
  if (!f) std::exit(2);
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  b.resize((size_t)sz);
  if (sz && std::fread(b.data(), 1, (size_t)sz, f) != (size_t)sz) std::exit(2);
  std::fclose(f);
  return b;
}
static void write_all(const char* path, const void* p, size_t n) {
  FILE* f = std::fopen(path, "wb");
  if (!f) std::exit(2);
  if (n && std::fwrite(p, 1, n, f) != n) std::exit(2);
  std::fclose(f);
}
template <class T>
static Kokkos::View<T*> to_device(const T* h, int64_t n) {
  Kokkos::View<T*> d("d", n);
  Kokkos::View<T*, Kokkos::HostSpace> m(const_cast<T*>(h), n);
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

int main(int argc, char** argv) {
  if (argc < 5) return 1;
  const std::string cmd = argv[1];
  const char* inp = argv[2];
  const char* outp = argv[3];
  auto a = [&](int i) { return std::atoll(argv[4 + i]); };
  Kokkos::initialize(argc, argv);
  int rc = 0;
  {
    KE::GB300 ex;
    const std::vector<unsigned char> in = read_all(inp);
    if (cmd == "algos_i64") {
      const int64_t n = a(0);
      auto x = to_device((const int64_t*)in.data(), n);
      Kokkos::View<int64_t*> e("e", n), c("c", n);
      std::vector<int64_t> o;
      auto plus = KOKKOS_LAMBDA(int64_t p, int64_t q) { return p + q; };
      o.push_back(KE::transform_reduce(ex, KE::cbegin(x), KE::cend(x), int64_t{3}, plus,
                                       KOKKOS_LAMBDA(int64_t v) { return v * v % 1009; }));
      o.push_back(KE::min_element(ex, KE::cbegin(x), KE::cend(x)) - KE::cbegin(x));
      o.push_back(KE::max_element(ex, KE::cbegin(x), KE::cend(x)) - KE::cbegin(x));
      auto mm = KE::minmax_element(ex, KE::cbegin(x), KE::cend(x));
      o.push_back(mm.first - KE::cbegin(x));
      o.push_back(mm.second - KE::cbegin(x));
      o.push_back(KE::transform_reduce(ex, KE::cbegin(x), KE::cend(x), KE::cbegin(x), int64_t{11}));
      KE::transform_exclusive_scan(ex, KE::cbegin(x), KE::cend(x), KE::begin(e), int64_t{5}, plus,
                                   KOKKOS_LAMBDA(int64_t v) { return 2 * v + 1; });
      KE::transform_inclusive_scan(ex, KE::cbegin(x), KE::cend(x), KE::begin(c), plus,
                                   KOKKOS_LAMBDA(int64_t v) { return v % 7; });
      auto he = to_host(e), hc = to_host(c);
      o.insert(o.end(), he.begin(), he.end());
      o.insert(o.end(), hc.begin(), hc.end());
      write_all(outp, o.data(), o.size() * sizeof(int64_t));
    } else if (cmd == "team_scan_i32") {
      const int64_t nseg = a(0);
      const int64_t* offs = (const int64_t*)in.data();
      const int64_t n = offs[nseg];
      auto o = to_device(offs, nseg + 1);
      auto x = to_device((const int32_t*)(in.data() + sizeof(int64_t) * (nseg + 1)), n);
      Kokkos::View<int32_t*> y("y", n);
      using TP = Kokkos::TeamPolicy<>;
      Kokkos::parallel_for(TP((int)nseg, Kokkos::AUTO), KOKKOS_LAMBDA(const TP::member_type& t) {
        const int64_t s = t.league_rank();
        Kokkos::parallel_scan(Kokkos::TeamThreadRange(t, o(s), o(s + 1)), [&](int64_t i, int32_t& u, bool fin) {
          if (fin) y(i) = u;
          u += x(i);
        });
      });
      auto hy = to_host(y);
      write_all(outp, hy.data(), hy.size() * sizeof(int32_t));
    } else if (cmd == "umap_count") {
      const int64_t n = a(0), cap = a(1);
      auto k = to_device((const int32_t*)in.data(), n);
      Kokkos::UnorderedMap<int32_t, int64_t> m((uint32_t)cap);
      using Op = Kokkos::UnorderedMapInsertOpTypes<Kokkos::View<int64_t*>, uint32_t>::AtomicAdd;
      Op op;
      Kokkos::parallel_for(Kokkos::RangePolicy<>(0, n), KOKKOS_LAMBDA(int64_t i) { m.insert(k(i), int64_t{1}, op); });
      ex.fence();
      // (key, value) of every valid slot, read back and sorted by key
      const uint32_t capn = m.capacity();
      Kokkos::View<int32_t*> kk("kk", capn);
      Kokkos::View<int64_t*> vv("vv", capn);
      Kokkos::View<int32_t*> ok("ok", capn);
      Kokkos::parallel_for(Kokkos::RangePolicy<>(0, capn), KOKKOS_LAMBDA(int64_t i) {
        const bool v = m.valid_at((uint32_t)i);
        ok(i) = v ? 1 : 0;
        kk(i) = v ? m.key_at((uint32_t)i) : 0;
        vv(i) = v ? m.value_at((uint32_t)i) : 0;
      });
      auto hk = to_host(kk);
      auto hv = to_host(vv);
      auto hok = to_host(ok);
      std::vector<std::pair<int32_t, int64_t>> kv;
      for (uint32_t i = 0; i < capn; ++i)
        if (hok[i]) kv.push_back({hk[i], hv[i]});
      std::sort(kv.begin(), kv.end());
      std::vector<int64_t> out;
      out.push_back((int64_t)m.size());
      out.push_back(m.failed_insert() ? 1 : 0);
      for (auto& e : kv) {
        out.push_back(e.first);
        out.push_back(e.second);
      }
      write_all(outp, out.data(), out.size() * sizeof(int64_t));
    } else {
      rc = 3;
    }
    ex.fence();
  }
  Kokkos::finalize();
  return rc;
}
