// A minimal Kokkos Tools profiling library for the tests: counts the
// begin / end callbacks of parallel_for / parallel_reduce / parallel_scan
// (the C interface of core/src/impl/Kokkos_Profiling_C_Interface.h),
// checks that every end matches an open begin, records whether the label
// "sum" was seen and the device type of the device ids, and prints one
// summary line when the library is finalised.
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>

namespace {
std::mutex mu;
std::set<uint64_t> open_ids;
uint64_t next_id = 1, begins[3] = {0, 0, 0}, ends[3] = {0, 0, 0}, unmatched = 0;
uint32_t devtype = 999;
int saw_sum = 0, init_version_ok = 0;

void begin(int k, const char* name, uint32_t devid, uint64_t* id) {
  std::lock_guard<std::mutex> lk(mu);
  *id = next_id++;
  open_ids.insert(*id);
  ++begins[k];
  devtype = devid >> 24;
  if (name && std::strcmp(name, "sum") == 0) saw_sum = 1;
}
void end(int k, uint64_t id) {
  std::lock_guard<std::mutex> lk(mu);
  if (open_ids.erase(id) != 1) ++unmatched;
  ++ends[k];
}
}  // namespace

struct KokkosPDeviceInfo;

extern "C" {
void kokkosp_init_library(const int, const uint64_t version, const uint32_t, KokkosPDeviceInfo*) {
  init_version_ok = version >= 20211015;
}
void kokkosp_finalize_library() {
  std::printf("KOKKOS_TOOL for=%llu/%llu reduce=%llu/%llu scan=%llu/%llu unmatched=%llu open=%zu devtype=%u saw_sum=%d "
              "version_ok=%d\n",
              (unsigned long long)begins[0], (unsigned long long)ends[0], (unsigned long long)begins[1],
              (unsigned long long)ends[1], (unsigned long long)begins[2], (unsigned long long)ends[2],
              (unsigned long long)unmatched, open_ids.size(), devtype, saw_sum, init_version_ok);
  std::fflush(stdout);
}
void kokkosp_begin_parallel_for(const char* n, const uint32_t d, uint64_t* id) { begin(0, n, d, id); }
void kokkosp_end_parallel_for(const uint64_t id) { end(0, id); }
void kokkosp_begin_parallel_reduce(const char* n, const uint32_t d, uint64_t* id) { begin(1, n, d, id); }
void kokkosp_end_parallel_reduce(const uint64_t id) { end(1, id); }
void kokkosp_begin_parallel_scan(const char* n, const uint32_t d, uint64_t* id) { begin(2, n, d, id); }
void kokkosp_end_parallel_scan(const uint64_t id) { end(2, id); }
}
