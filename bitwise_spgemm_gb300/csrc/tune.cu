// tune.cu — the autotuner's cache: measured SpMM schedules per shape bucket.
//
// A schedule says which engine runs the SpMM (tensor cores or CUDA cores —
// the tensor-core density threshold of the bucket), on the tensor cores
// which tile form (K tiles per stage, B by TMA boxes or pre-tiled, split-K
// or not), and on the CUDA cores which prototype-row kernel (register
// gathers or TMA-staged slices) and which of its shapes.  bsp_tune (capi.cu) times the
// candidates on the caller's data and stores the fastest here under a bucket
// key (log2 sizes, density in half octaves, dtype, plan mode); bsp_spmm then
// looks the bucket up before its cost model.  The cache lives in the process
// and, when BSP_TUNE_CACHE names a file, is loaded from it at first use and
// written back after every new entry: to a temporary file in the same
// directory, then renamed over the old one, so a reader never sees half a
// file.  A file that does not parse is ignored as a whole.
//
// File format (JSON, one entry per line):
//   {"bsp_tune_cache": 2, "entries": [
//    {"key": "M13K13N9d9t0p2", "engine": 2, "proto_path": 0, "proto_variant": 4, "tc_tps": 0,
//     "tc_tiled": -1, "tc_split": -1, "ms": 0.0328},
//    ...
//   ]}
// (one entry per line; a version-1 file, without the tile form, does not parse)
#include <unistd.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "bsp_internal.cuh"
#include "plan.cuh"
#include "tune.h"

namespace bsp {
namespace {

std::mutex g_mu;
std::map<std::string, TuneSched> g_cache;
std::atomic<int> g_entries{0};
std::atomic<bool> g_env_loaded{false};

int bits_of(int64_t x) {  // ceil(log2(x)) for x >= 1
  int b = 0;
  while (((int64_t)1 << b) < x && b < 62) b++;
  return b;
}

// Parses the whole file into `out`; false if any line of it is malformed.
bool parse_file(const char* path, std::map<std::string, TuneSched>& out) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool header = false, closed = false, ok = true;
  while (fgets(line, sizeof line, f)) {
    if (strstr(line, "\"bsp_tune_cache\": 2")) {
      header = true;
      continue;
    }
    if (strstr(line, "\"key\"")) {
      char key[96];
      TuneSched t;
      double ms = 0;
      if (sscanf(line,
                 " {\"key\": \"%95[^\"]\", \"engine\": %d, \"proto_path\": %d, \"proto_variant\": %d, "
                 "\"tc_tps\": %d, \"tc_tiled\": %d, \"tc_split\": %d, \"ms\": %lf",
                 key, &t.engine, &t.proto_path, &t.proto_variant, &t.tc_tps, &t.tc_tiled, &t.tc_split, &ms) != 8 ||
          (t.engine != 1 && t.engine != 2) || t.proto_path < 0 || t.proto_path > 1 || t.proto_variant < 0 ||
          t.proto_variant > 8 || (t.tc_tps != 0 && t.tc_tps != 2 && t.tc_tps != 3) || t.tc_tiled < -1 ||
          t.tc_tiled > 1 || t.tc_split < -1 || t.tc_split > 0) {
        ok = false;
        break;
      }
      t.ms = ms;
      out[key] = t;
      continue;
    }
    if (strstr(line, "]}")) {
      closed = true;
      continue;
    }
    for (const char* c = line; *c; c++)
      if (*c != ' ' && *c != '\n' && *c != '\r' && *c != '\t') {
        ok = false;
        break;
      }
    if (!ok) break;
  }
  fclose(f);
  return ok && header && closed;
}

bool write_file(const char* path, const std::map<std::string, TuneSched>& m) {
  std::string tmp = std::string(path) + ".tmp" + std::to_string((long)getpid());
  FILE* f = fopen(tmp.c_str(), "w");
  if (!f) return false;
  bool ok = fprintf(f, "{\"bsp_tune_cache\": 2, \"entries\": [\n") > 0;
  size_t i = 0;
  for (const auto& kv : m) {
    ok = ok && fprintf(f,
                       " {\"key\": \"%s\", \"engine\": %d, \"proto_path\": %d, \"proto_variant\": %d, "
                       "\"tc_tps\": %d, \"tc_tiled\": %d, \"tc_split\": %d, \"ms\": %.6f}%s\n",
                       kv.first.c_str(), kv.second.engine, kv.second.proto_path, kv.second.proto_variant,
                       kv.second.tc_tps, kv.second.tc_tiled, kv.second.tc_split, kv.second.ms,
                       ++i < m.size() ? "," : "") > 0;
  }
  ok = ok && fprintf(f, "]}\n") > 0;
  ok = (fclose(f) == 0) && ok;
  if (!ok || rename(tmp.c_str(), path) != 0) {
    remove(tmp.c_str());
    return false;
  }
  return true;
}

void load_env_locked() {  // caller holds g_mu; the flag is raised after the entries are in
  if (g_env_loaded.load()) return;
  const char* p = getenv("BSP_TUNE_CACHE");
  std::map<std::string, TuneSched> m;
  if (p && *p && parse_file(p, m)) {
    for (const auto& kv : m) g_cache[kv.first] = kv.second;
    g_entries.store((int)g_cache.size());
  }
  g_env_loaded.store(true);
}

}  // namespace

std::string tune_key(const bsp_plan* plan, int64_t N, int dtype) {
  const double dens = plan->M > 0 && plan->K > 0 ? (double)plan->nnz / ((double)plan->M * (double)plan->K) : 0.0;
  const int db = dens > 0 ? (int)std::floor(-2.0 * std::log2(dens)) : 99;
  char k[96];
  snprintf(k, sizeof k, "M%dK%dN%dd%dt%dp%d", bits_of(plan->M), bits_of(plan->K), bits_of(N), db, dtype, plan->mode);
  return k;
}

bool tune_lookup(const bsp_plan* plan, int64_t N, int dtype, TuneSched* out) {
  if (g_entries.load(std::memory_order_acquire) == 0 && g_env_loaded.load(std::memory_order_acquire)) return false;
  std::lock_guard<std::mutex> lk(g_mu);
  load_env_locked();
  auto it = g_cache.find(tune_key(plan, N, dtype));
  if (it == g_cache.end()) return false;
  *out = it->second;
  return true;
}

void tune_store(const std::string& key, const TuneSched& t) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_env_locked();
  g_cache[key] = t;
  g_entries.store((int)g_cache.size());
  const char* p = getenv("BSP_TUNE_CACHE");
  if (p && *p) write_file(p, g_cache);
}

int tune_cache_load(const char* path, int* entries) {
  std::map<std::string, TuneSched> m;
  if (!parse_file(path, m)) return BSP_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  g_env_loaded = true;
  g_cache = m;
  g_entries.store((int)g_cache.size());
  if (entries) *entries = (int)g_cache.size();
  return BSP_OK;
}

int tune_cache_save(const char* path) {
  std::lock_guard<std::mutex> lk(g_mu);
  return write_file(path, g_cache) ? BSP_OK : BSP_ERR_INVALID_ARG;
}

void tune_cache_clear() {
  std::lock_guard<std::mutex> lk(g_mu);
  g_env_loaded = true;
  g_cache.clear();
  g_entries.store(0);
}

int tune_cache_size() {
  std::lock_guard<std::mutex> lk(g_mu);
  load_env_locked();
  return (int)g_cache.size();
}

}  // namespace bsp
