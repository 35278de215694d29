// Tuning: the in-process tuning table consulted by the entry points, and the
// Kokkos Tools tuning-tool callbacks (see include/gbk_tools.h).
//
// The tool keeps, per tuning context key (the context variables' names and
// values plus the requested output variables), the Cartesian product of the
// output variables' candidate sets.  The first visits of a key try each
// combination in turn, timed with a steady host clock from begin_context to
// end_context (the caller fences before ending the context, as Kokkos'
// tuned dispatch does); afterwards the fastest combination is answered.  A
// context that names gbk.kind / gbk.op / gbk.dtype / gbk.log2n / gbk.extra
// and matches a tuning-table entry is answered from the table at once.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <cstdlib>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gbk_tools.h"
#include "gbk_internal.cuh"

namespace gbk {
namespace {

struct Key {
  int kind, op, dtype, log2n, extra;
  bool operator<(const Key& o) const {
    return std::tie(kind, op, dtype, extra, log2n) < std::tie(o.kind, o.op, o.dtype, o.extra, o.log2n);
  }
};

std::mutex g_tmu;
std::map<Key, gbk_tuning_t> g_table;
bool g_enabled = false;

int ceil_log2(int64_t n) {
  int l = 0;
  while (((int64_t)1 << l) < n && l < 62) ++l;
  return l;
}

bool table_find(int kind, int op, int dtype, int64_t n, int extra, gbk_tuning_t* out) {
  const int l2 = ceil_log2(n < 1 ? 1 : n);
  // nearest log2n among entries of the same (kind, op, dtype, extra)
  auto lo = g_table.lower_bound(Key{kind, op, dtype, -1, extra});
  const gbk_tuning_t* best = nullptr;
  int bestd = 1 << 30;
  for (auto it = lo; it != g_table.end(); ++it) {
    const Key& k = it->first;
    if (k.kind != kind || k.op != op || k.dtype != dtype || k.extra != extra) break;
    const int d = std::abs(k.log2n - l2);
    if (d < bestd) {
      bestd = d;
      best = &it->second;
    }
  }
  if (!best) return false;
  *out = *best;
  return true;
}

// ---- Kokkos Tools tool state ---------------------------------------------------
struct OutVar {
  std::string name;
  int type = kokkos_value_int64;
  std::vector<int64_t> ivals;
  std::vector<double> dvals;
  size_t count() const { return type == kokkos_value_double ? dvals.size() : ivals.size(); }
};
struct KeyState {
  std::vector<size_t> ids;                // output variable ids, in request order
  std::vector<std::vector<size_t>> comb;  // candidate index per id
  std::vector<double> best_time;          // per combination (inf = untried)
  size_t next = 0;
};
struct Active {
  std::string key;
  size_t combo = 0;
  bool timed = false;
  std::chrono::steady_clock::time_point t0;
};
std::map<size_t, std::string> g_in_names;
std::map<size_t, OutVar> g_out;
std::map<std::string, KeyState> g_states;
std::map<size_t, Active> g_active;
std::map<size_t, int> g_goal;  // context id -> Kokkos_Tools_OptimizationType
int64_t g_requests = 0, g_contexts = 0;
uint64_t g_interface_version = 0;

std::string value_text(const Kokkos_Tools_VariableValue& v) {
  char buf[96];
  const Kokkos_Tools_VariableInfo* m = v.metadata;
  const int t = m ? m->type : kokkos_value_int64;
  if (t == kokkos_value_double) std::snprintf(buf, sizeof buf, "%.17g", v.value.double_value);
  else if (t == kokkos_value_string) std::snprintf(buf, sizeof buf, "%.63s", v.value.string_value);
  else std::snprintf(buf, sizeof buf, "%lld", (long long)v.value.int_value);
  return buf;
}

void set_value(Kokkos_Tools_VariableValue& v, const OutVar& o, size_t idx) {
  if (o.type == kokkos_value_double) v.value.double_value = o.dvals[idx];
  else v.value.int_value = o.ivals[idx];
}

}  // namespace

// Entry-point hook: the table's configuration for a call with tune == NULL.
const gbk_tuning_t* tuned_config(int kind, int op, int dtype, int64_t n, int extra, gbk_tuning_t* storage) {
  std::lock_guard<std::mutex> lk(g_tmu);
  if (!g_enabled || g_table.empty()) return nullptr;
  return table_find(kind, op, dtype, n, extra, storage) ? storage : nullptr;
}

}  // namespace gbk

using namespace gbk;

extern "C" {

int gbk_tuner_clear(void) {
  std::lock_guard<std::mutex> lk(g_tmu);
  g_table.clear();
  return GBK_OK;
}

int gbk_tuner_set(int kind, int op, int dtype, int log2n, int extra, const gbk_tuning_t* cfg) {
  if (!cfg) return GBK_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_tmu);
  g_table[Key{kind, op, dtype, log2n, extra}] = *cfg;
  return GBK_OK;
}

int gbk_tuner_lookup(int kind, int op, int dtype, int64_t n, int extra, gbk_tuning_t* cfg) {
  if (!cfg) return GBK_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_tmu);
  return table_find(kind, op, dtype, n, extra, cfg) ? GBK_OK : GBK_ERR_UNSUPPORTED;
}

int gbk_tuner_load(const char* path) {
  if (!path) return GBK_ERR_INVALID_ARGUMENT;
  FILE* f = std::fopen(path, "r");
  if (!f) return GBK_ERR_INVALID_ARGUMENT;
  std::map<Key, gbk_tuning_t> t;
  char line[256];
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    Key k;
    gbk_tuning_t c;
    if (std::sscanf(line, "%d %d %d %d %d %d %d %d %d", &k.kind, &k.op, &k.dtype, &k.log2n, &k.extra, &c.block,
                    &c.items_per_thread, &c.ctas_per_sm, &c.variant) == 9)
      t[k] = c;
  }
  std::fclose(f);
  std::lock_guard<std::mutex> lk(g_tmu);
  g_table.swap(t);
  return GBK_OK;
}

int gbk_tuner_save(const char* path) {
  if (!path) return GBK_ERR_INVALID_ARGUMENT;
  FILE* f = std::fopen(path, "w");
  if (!f) return GBK_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_tmu);
  std::fprintf(f, "# kind op dtype log2n extra block items_per_thread ctas_per_sm variant\n");
  for (auto& kv : g_table)
    std::fprintf(f, "%d %d %d %d %d %d %d %d %d\n", kv.first.kind, kv.first.op, kv.first.dtype, kv.first.log2n,
                 kv.first.extra, kv.second.block, kv.second.items_per_thread, kv.second.ctas_per_sm, kv.second.variant);
  std::fclose(f);
  return GBK_OK;
}

int gbk_tuner_enable(int on) {
  std::lock_guard<std::mutex> lk(g_tmu);
  g_enabled = on != 0;
  return GBK_OK;
}

int64_t gbk_tuner_size(void) {
  std::lock_guard<std::mutex> lk(g_tmu);
  return (int64_t)g_table.size();
}

// ---- Kokkos Tools tuning callbacks -------------------------------------------------
void kokkosp_init_library(const int load_seq, const uint64_t interface_version, const uint32_t device_info_count,
                          Kokkos_Profiling_KokkosPDeviceInfo* device_info) {
  (void)load_seq;
  (void)device_info_count;
  (void)device_info;
  std::lock_guard<std::mutex> lk(g_tmu);
  g_interface_version = interface_version;
}

void kokkosp_finalize_library(void) {
  const char* path = std::getenv("GBK_TOOL_REPORT");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "w");
  if (!f) return;
  std::lock_guard<std::mutex> lk(g_tmu);
  std::fprintf(f, "interface_version %llu\n", (unsigned long long)g_interface_version);
  for (auto& kv : g_in_names) std::fprintf(f, "input %zu %s\n", kv.first, kv.second.c_str());
  for (auto& kv : g_out)
    std::fprintf(f, "output %zu %s type %d candidates %zu\n", kv.first, kv.second.name.c_str(), kv.second.type,
                 kv.second.count());
  std::fprintf(f, "requests %lld contexts %lld keys %zu\n", (long long)g_requests, (long long)g_contexts,
               g_states.size());
  for (auto& kv : g_states) {
    const KeyState& st = kv.second;
    if (st.best_time.empty()) continue;
    const size_t b = (size_t)(std::min_element(st.best_time.begin(), st.best_time.end()) - st.best_time.begin());
    std::fprintf(f, "best %s ->", kv.first.c_str());
    for (size_t i = 0; i < st.ids.size() && i < st.comb[b].size(); ++i) {
      auto it = g_out.find(st.ids[i]);
      if (it == g_out.end() || it->second.count() == 0) continue;
      if (it->second.type == kokkos_value_double) std::fprintf(f, " %s=%g", it->second.name.c_str(), it->second.dvals[st.comb[b][i]]);
      else std::fprintf(f, " %s=%lld", it->second.name.c_str(), (long long)it->second.ivals[st.comb[b][i]]);
    }
    std::fprintf(f, " tried %zu of %zu\n", std::min(st.next, st.comb.size()), st.comb.size());
  }
  std::fclose(f);
}

void kokkosp_declare_input_type(const char* name, const size_t id, Kokkos_Tools_VariableInfo* info) {
  (void)info;
  std::lock_guard<std::mutex> lk(g_tmu);
  g_in_names[id] = name ? name : "";
}

void kokkosp_declare_output_type(const char* name, const size_t id, Kokkos_Tools_VariableInfo* info) {
  OutVar o;
  o.name = name ? name : "";
  if (info) {
    o.type = info->type;
    if (info->valueQuantity == kokkos_value_set) {
      const size_t n = info->candidates.set.size;
      for (size_t i = 0; i < n; ++i) {
        if (info->type == kokkos_value_double) o.dvals.push_back(info->candidates.set.values.double_value[i]);
        else if (info->type == kokkos_value_int64) o.ivals.push_back(info->candidates.set.values.int_value[i]);
      }
    } else if (info->valueQuantity == kokkos_value_range && info->type == kokkos_value_int64) {
      const auto& r = info->candidates.range;
      const int64_t step = r.step.int_value > 0 ? r.step.int_value : 1;
      const int64_t lo = r.lower.int_value + (r.openLower ? step : 0);
      for (int64_t v = lo; (r.openUpper ? v < r.upper.int_value : v <= r.upper.int_value) && o.ivals.size() < 64;
           v += step)
        o.ivals.push_back(v);
    } else if (info->valueQuantity == kokkos_value_range && info->type == kokkos_value_double) {
      // e.g. the coordinates Kokkos' MDRange and team-size tuners declare
      // (core/src/Kokkos_Tuners.hpp:334-348): at most 16 evenly spread points
      const auto& r = info->candidates.range;
      const double lo = r.lower.double_value, hi = r.upper.double_value;
      double step = r.step.double_value > 0 ? r.step.double_value : (hi - lo) / 16;
      const double span = hi - lo;
      if (span > 0 && span / step > 16) step = span / 16;
      for (double v = lo + (r.openLower ? step : 0.0); (r.openUpper ? v < hi : v <= hi) && o.dvals.size() < 16;
           v += step)
        o.dvals.push_back(v);
    }
  }
  std::lock_guard<std::mutex> lk(g_tmu);
  g_out[id] = o;
}

void kokkosp_declare_optimization_goal(const size_t context_id, const Kokkos_Tools_OptimizationGoal goal) {
  std::lock_guard<std::mutex> lk(g_tmu);
  g_goal[context_id] = goal.goal;
}

void kokkosp_begin_context(const size_t context_id) {
  std::lock_guard<std::mutex> lk(g_tmu);
  ++g_contexts;
  Active& a = g_active[context_id];
  a.t0 = std::chrono::steady_clock::now();
  a.timed = false;
}

void kokkosp_request_values(const size_t context_id, const size_t nctx, const Kokkos_Tools_VariableValue* cvals,
                            const size_t ntune, Kokkos_Tools_VariableValue* tvals) {
  std::lock_guard<std::mutex> lk(g_tmu);
  ++g_requests;
  // Context key and the gbk.* context variables.
  std::vector<std::pair<std::string, std::string>> kv;
  int gk[5] = {-1, -1, -1, -1, 0};
  const char* gnames[5] = {"gbk.kind", "gbk.op", "gbk.dtype", "gbk.log2n", "gbk.extra"};
  for (size_t i = 0; i < nctx; ++i) {
    auto it = g_in_names.find(cvals[i].type_id);
    const std::string nm = it != g_in_names.end() ? it->second : std::to_string(cvals[i].type_id);
    kv.emplace_back(nm, value_text(cvals[i]));
    for (int j = 0; j < 5; ++j)
      if (nm == gnames[j]) gk[j] = (int)cvals[i].value.int_value;
  }
  std::sort(kv.begin(), kv.end());
  std::string key;
  for (auto& p : kv) key += p.first + "=" + p.second + ";";
  key += "|";
  for (size_t i = 0; i < ntune; ++i) key += std::to_string(tvals[i].type_id) + ",";
  Active& a = g_active[context_id];
  a.key = key;
  // 1. tuning table
  if (g_enabled && gk[0] >= 0 && gk[1] >= 0 && gk[2] >= 0 && gk[3] >= 0) {
    gbk_tuning_t c;
    if (table_find(gk[0], gk[1], gk[2], (int64_t)1 << gk[3], gk[4], &c)) {
      for (size_t i = 0; i < ntune; ++i) {
        auto it = g_out.find(tvals[i].type_id);
        if (it == g_out.end()) continue;
        const std::string& nm = it->second.name;
        const int64_t v = nm == "gbk.block" ? c.block
                          : nm == "gbk.items_per_thread" ? c.items_per_thread
                          : nm == "gbk.ctas_per_sm" ? c.ctas_per_sm
                          : nm == "gbk.variant" ? c.variant : INT64_MIN;
        if (v != INT64_MIN) tvals[i].value.int_value = v;
      }
      a.timed = false;
      a.combo = (size_t)-1;
      return;
    }
  }
  // 2. online exhaustive search over the candidate sets
  KeyState& s = g_states[key];
  if (s.comb.empty()) {
    s.ids.clear();
    size_t total = 1;
    for (size_t i = 0; i < ntune; ++i) {
      s.ids.push_back(tvals[i].type_id);
      auto it = g_out.find(tvals[i].type_id);
      const size_t c = it != g_out.end() ? it->second.count() : 0;
      total *= c ? c : 1;
    }
    total = std::min<size_t>(total, 4096);
    for (size_t k = 0; k < total; ++k) {
      std::vector<size_t> idx(ntune, 0);
      size_t r = k;
      for (size_t i = 0; i < ntune; ++i) {
        auto it = g_out.find(tvals[i].type_id);
        const size_t c = it != g_out.end() ? std::max<size_t>(it->second.count(), 1) : 1;
        idx[i] = r % c;
        r /= c;
      }
      s.comb.push_back(idx);
    }
    s.best_time.assign(s.comb.size(), INFINITY);
  }
  size_t pick;
  if (s.next < s.comb.size()) {
    pick = s.next++;
  } else {
    pick = (size_t)(std::min_element(s.best_time.begin(), s.best_time.end()) - s.best_time.begin());
  }
  for (size_t i = 0; i < ntune && i < s.comb[pick].size(); ++i) {
    auto it = g_out.find(tvals[i].type_id);
    if (it == g_out.end() || it->second.count() == 0) continue;
    set_value(tvals[i], it->second, s.comb[pick][i]);
  }
  a.combo = pick;
  a.timed = true;
}

void kokkosp_end_context(const size_t context_id, Kokkos_Tools_VariableValue objective) {
  (void)objective;
  const auto t1 = std::chrono::steady_clock::now();
  std::lock_guard<std::mutex> lk(g_tmu);
  auto it = g_active.find(context_id);
  if (it == g_active.end()) return;
  Active a = it->second;
  g_active.erase(it);
  if (!a.timed) return;
  auto st = g_states.find(a.key);
  if (st == g_states.end() || a.combo >= st->second.best_time.size()) return;
  // The tool's objective is the context's elapsed time, always minimised
  // (a declared goal refers to the caller's own objective value).
  const double dt = std::chrono::duration<double>(t1 - a.t0).count();
  double& b = st->second.best_time[a.combo];
  if (dt < b) b = dt;
}

}  // extern "C"
