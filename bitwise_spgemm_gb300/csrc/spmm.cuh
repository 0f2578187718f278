// spmm.cuh — argument block and launchers of the CUDA-core SpMM kernels.
#pragma once
#include <cuda.h>

#include "bsp_internal.cuh"

namespace bsp {

// One problem of the batched form on the tensor cores: B's tensor map (64x32
// boxes, 128-byte swizzle; first, so the record keeps the map's alignment), A
// and C.
struct BatchProblemTc {
  CUtensorMap map;   // forward: B [K][N]; Aᵀ·G: G [M][N] (64x32 boxes); SDDMM: G [M][N] (64x256 boxes)
  CUtensorMap map2;  // SDDMM: X [K][N] (64x256 boxes); otherwise unused
  CUtensorMap map3;  // SDDMM: G [M][N] in 64x128 boxes (the persistent batched SDDMM); otherwise unused
  const uint32_t* A;
  int64_t M, K, Kw;
  float* C;          // forward: C [M][N]; Aᵀ·G: dX [K][N]; SDDMM: dA [M][K]
  int64_t ldc;
};
// Tensor map of a batch problem's B [K][N] (row stride ldb elements), or of
// G [M][N] for the batched Aᵀ·G: 64-column x 32-row boxes.
int make_batch_map(CUtensorMap* m, const void* B, int bdt, int64_t K, int64_t N, int64_t ldb);
// Tensor map of G [M][N] or X [K][N] for the batched SDDMM: 64-column x
// 256-row boxes.
int make_batch_map_sddmm(CUtensorMap* m, const void* T, int bdt, int64_t rows, int64_t N, int64_t ld,
                         int box_rows = 256);
// Work item b = {problem, 256-row block, 256-column block, reduction tiles}:
// one CTA each.  kind 0 = forward C = A·B, 1 = dX = Aᵀ·G (rows: K),
// 2 = dA = (G·Xᵀ) ⊙ A (columns: K).
int launch_batched_tc(const BatchProblemTc* probs, const int4* items, int n_items, int64_t N, int bdt,
                      cudaStream_t s, int kind = 0);

struct SpmmArgs {
  const uint32_t* A;  // packed rows [M][Kw], LSB-first
  int64_t M, K, Kw;
  const void* B;      // [K][ldb] of bdt
  int bdt;
  int64_t ldb, N;
  float* C;           // [M][ldc]
  int64_t ldc;
  // prototype mode (plan)
  const int32_t* row_cluster;  // [M], -1 = walk A's row
  const int32_t* delta_ptr;    // [M+1]
  const uint32_t* delta_idx;   // column | 0x80000000 for "subtract"
  int64_t n_delta;             // entries in delta_idx
  const uint32_t* cons;        // [n_proto][Kw] prototype masks
  int64_t n_proto;
  int64_t proto_max_nnz;       // set bits of the densest prototype (TwoSum above 4096)
  const uint32_t* delta_pad;   // [n_slot][32] row slots (row, cluster, count, start, 28 entries), or null
  int64_t n_slot;              // clustered rows, in slot order
  const int32_t* cons_ptr;     // [n_proto + 1] prototype column lists, or null
  const uint32_t* cons_idx;
  float* P;                    // [n_proto][ldp] prototype sums (workspace)
  int64_t ldp;
  // optional row subset for the walking kernel (rows of A without a cluster)
  const int32_t* row_list;     // [n_list] or nullptr = rows 0..M-1
  int64_t n_list;
};

// vec = B/C layouts allow 16-byte vector access (else lane-per-column path)
int launch_spmm_rows(const SpmmArgs& a, bool proto, bool vec, cudaStream_t s);
int launch_proto_sums(const SpmmArgs& a, cudaStream_t s);
// Clustered rows through registers, launched as a programmatic dependent of
// the prototype-sum kernel; rows without a cluster are left to the walker.
int launch_spmm_proto_regs(const SpmmArgs& a, int variant, cudaStream_t s);

// Prototype rows through TMA bulk copies staged in shared memory
// (spmm_bulk.cu).  Needs the vector layout; rows without a cluster are
// skipped (walk them with launch_spmm_rows over the plan's direct-row list).
int launch_spmm_proto_bulk(const SpmmArgs& a, int variant, cudaStream_t s);
// Device-side error word of the bulk kernels (0 = none); clear resets it.
int bulk_device_error(int* out, bool clear);
// Prototype sums from the column lists with B slices staged by bulk copies
// (B 16-byte aligned, ldb·esize and N·esize multiples of 16).
int launch_proto_sums_bulk(const SpmmArgs& a, int variant, cudaStream_t s);

// Tensor-core path (spmm_tc.cu) for 16-bit B: occupancy bitmap of 32-column
// K tiles per 128-row block ([ceil(M/128)][tc_occupancy_words(K)]), then the
// tcgen05 kernel over the occupied tiles.
int tc_occupancy_words(int64_t K);
// Longest reduction (K forward, M transposed) the tensor-core kernels take:
// a CTA lists its occupied 32-column tiles in shared memory.
int64_t tc_max_reduction();
int tc_occupancy_t_words(int64_t M);
int launch_occupancy(const uint32_t* A, int64_t M, int64_t K, uint32_t* occ, uint32_t* occT,
                     unsigned long long* count, unsigned long long* countT, cudaStream_t s);
// ws (optional): room for split-K partials (used when the output grid is
// small and ws_bytes ≥ tc_split_bytes(...)) and, after them, for B in tile
// order (used when the rest holds tc_tiled_b_bytes(...)); else ignored.
// At (optional): A's words column by column ([Kw][M], launch_transpose_words)
// for coalesced word loads; null = loads from the rows.
// form: the tile form a tuned schedule fixes (0 / -1 fields = the rule):
// K tiles per stage (2 or 3), B pre-tiled (1) or by TMA boxes (0), split-K
// allowed (-1) or not (0).
struct TcForm {
  int tps = 0, tiled = -1, split = -1;
};
int launch_spmm_tc(const SpmmArgs& a, const uint32_t* occ, const uint32_t* At, cudaStream_t s, void* ws = nullptr,
                   size_t ws_bytes = 0, TcForm form = TcForm{});
int launch_transpose_words(const uint32_t* words, int64_t M, int64_t Kw, uint32_t* At, cudaStream_t s);
int tc_split_count(int64_t out_rows, int64_t out_cols, int64_t red_tiles);
size_t tc_split_bytes(int64_t out_rows, int64_t out_cols, int64_t red_tiles);
// B (fwd) / G (trans) copied into tile order for one bulk copy per tile: the
// workspace it takes, and the workspace with which the tensor-core launch
// both splits the reduction (when it would) and tiles B.
size_t tc_tiled_b_bytes(int64_t red_rows, int64_t cols);
size_t tc_preferred_bytes(int64_t out_rows, int64_t out_cols, int64_t red_rows);
// dX[K][N] = Aᵀ·G on the tensor cores, Aᵀ read from A's row words
int launch_spmm_t_tc(const uint32_t* A, int64_t M, int64_t K, const void* G, int gdt, int64_t ldg, int64_t N,
                     float* dX, int64_t lddx, const uint32_t* occT, const uint32_t* At, cudaStream_t s, void* ws = nullptr, size_t ws_bytes = 0);
// dA[M][K] = (G·Xᵀ) at A's set bits, 0 elsewhere, on the tensor cores
int launch_sddmm_tc(const uint32_t* A, int64_t M, int64_t K, const void* G, int64_t ldg, const void* X,
                    int64_t ldx, int dt, int64_t N, float* dA, int64_t ldda, cudaStream_t s);
// same on CUDA cores (any dtype / layout): warp per row, one dot product per set bit
int launch_sddmm_rows(const uint32_t* A, int64_t M, int64_t K, const void* G, int64_t ldg, const void* X,
                      int64_t ldx, int dt, int64_t N, float* dA, int64_t ldda, cudaStream_t s);
int tc_device_error(int* out, bool clear);
int batched_device_error(int* out, bool clear);



}  // namespace bsp
