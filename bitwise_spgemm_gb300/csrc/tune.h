// tune.h — the autotuner's cache of measured SpMM schedules (tune.cu).
#pragma once
#include <stdint.h>

#include <string>

struct bsp_plan;

namespace bsp {

struct TuneSched {
  int engine = 2;         // 1 = tensor cores, 2 = CUDA cores
  int proto_path = 0;     // CUDA cores, prototype rows: 0 = register gathers, 1 = TMA-staged slices
  int proto_variant = 4;  // kernel shape of that path
  double ms = 0.0;        // measured time of the schedule
  // tensor cores: the tile form (0 / -1 = the launcher's own rule)
  int tc_tps = 0;         // K tiles per pipeline stage: 2 (three stages) or 3 (two stages)
  int tc_tiled = -1;      // B by TMA boxes (0) or copied into tile order first (1)
  int tc_split = -1;      // split-K over the reduction when the output grid is small: 0 = never
};

std::string tune_key(const bsp_plan* plan, int64_t N, int dtype);
bool tune_lookup(const bsp_plan* plan, int64_t N, int dtype, TuneSched* out);
void tune_store(const std::string& key, const TuneSched& t);
int tune_cache_load(const char* path, int* entries);
int tune_cache_save(const char* path);
void tune_cache_clear();
int tune_cache_size();

}  // namespace bsp
