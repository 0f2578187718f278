// plan.cuh — the plan object behind the opaque bsp_plan handle.
#pragma once
#include "bsp_internal.cuh"

struct bsp_plan {
  int64_t M = 0, K = 0, Kw = 0;
  int mode = BSP_PLAN_DIRECT;
  int device = 0;
  int64_t nnz = 0, n_proto = 0, proto_nnz = 0, delta_nnz = 0, direct_rows = 0, direct_nnz = 0;
  int64_t proto_max_nnz = 0;  // set bits of the densest prototype (compensated sums above 4096)
  // device storage (owned)
  void* arena = nullptr;        // row_cluster, delta_ptr, cons
  void* delta_arena = nullptr;  // delta_idx
  void* tc_arena = nullptr;     // occ, occT, wordsT
  bool arena_pooled = false, delta_pooled = false, tc_pooled = false;  // from the stream-ordered pool
  int32_t* row_cluster = nullptr;
  int32_t* delta_ptr = nullptr;
  uint32_t* delta_idx = nullptr;
  uint32_t* cons = nullptr;
  uint32_t* delta_pad = nullptr;   // [n_slot][32] row slots by descending delta count (or null)
  int64_t n_slot = 0;              // clustered rows with a slot
  int32_t* cons_ptr = nullptr;     // [n_proto + 1]: each prototype's columns in cons_idx
  uint32_t* cons_idx = nullptr;    // prototype columns, ascending per prototype (proto plans)
  int32_t* direct_list = nullptr;  // rows without a cluster (ascending), direct_rows entries
  uint32_t* occ = nullptr;         // occupied 32-column K tiles per 128-row block (tensor-core path)
  int64_t occ_tiles = 0;           // number of occupied (128-row, 32-column) tiles
  uint32_t* occT = nullptr;        // occupied 32-row tiles per 128-column block (transposed product)
  uint32_t* wordsT = nullptr;      // A's words column by column, [Kw][M] (tensor-core word loads), or null
  int64_t occT_tiles = 0;
};

namespace bsp {
int plan_build(const uint32_t* words, int64_t M, int64_t K, const bsp_plan_params* prm,
               bsp_plan* plan, cudaStream_t s);
void plan_free(bsp_plan* plan);
// Returns pooled blocks in stream order on s (other blocks with cudaFree).
int plan_free_async(bsp_plan* plan, cudaStream_t s);
}  // namespace bsp
