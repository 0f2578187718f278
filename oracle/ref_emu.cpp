/*
 * ref_emu.cpp — runs reference kernels on the CPU (see ref_shim.h) and
 * exports them with a C ABI for the oracle-pinning tests.  TEST
 * INFRASTRUCTURE ONLY.
 *
 * The kernel bodies are not in this repository: build_ref.py extracts them
 * at build time from the reference checkout into oracle/_ref/*.inc
 * (generate_groups_large  source/src/main.cu:50-247,
 *  dense2bitmask          source/src/main.cu:591-628,
 *  group2dense            source/src/main.cu:829-850,
 *  layout_trans, uint8_layout_trans  backup/layout_trans.cu:75-97,
 *  uint8_spmm_2d_1d       backup/layout_trans.cu:158-171)
 * and compiles this file with oracle/_ref on the include path.
 *
 * The compile-time configuration the kernels expect (source/src/common.h:
 * 20-28) is supplied here; SIZE_N, which the reference fixes at 8192, is a
 * runtime value so that small cases can run.
 */
#include "ref_shim.h"

#include <vector>

emu_state g_emu;

static int g_size_n = 0;
#define TILE_WIDTH 32
#define MAX_GROUP_NUM 2
#define OUTPUT_MAX_GROUP_NUM 2
#define SPLIT_K 2048
#define SIZE_N g_size_n

#include "ref_generate_groups_large.inc"
#include "ref_dense2bitmask.inc"
#include "ref_group2dense.inc"
#include "ref_layout_trans.inc"
#include "ref_uint8_spmm.inc"

static const size_t kStack = 64 * 1024;
static emu_body_fn s_body;
static void* s_arg;

static void fiber_entry() {
  s_body(s_arg);
  g_emu.cur->done = 1;
}

int emu_launch(dim3 grid, dim3 block, emu_body_fn body, void* arg) {
  int nt = (int)block.x;
  if (nt <= 0 || nt > 4096) return -1;
  std::vector<emu_fiber> f(nt);
  std::vector<char> stacks((size_t)nt * kStack);
  s_body = body;
  s_arg = arg;
  g_emu.gdim = grid;
  g_emu.bdim = block;
  for (unsigned by = 0; by < grid.y; by++)
    for (unsigned bx = 0; bx < grid.x; bx++) {
      g_emu.bidx = dim3(bx, by, 0);
      for (int t = 0; t < nt; t++) {
        getcontext(&f[t].ctx);
        f[t].ctx.uc_stack.ss_sp = &stacks[(size_t)t * kStack];
        f[t].ctx.uc_stack.ss_size = kStack;
        f[t].ctx.uc_link = &g_emu.sched;
        makecontext(&f[t].ctx, fiber_entry, 0);
        f[t].tid = dim3((unsigned)t, 0, 0);
        f[t].done = 0;
      }
      int remaining = nt;
      while (remaining > 0) {
        for (int t = 0; t < nt; t++) {
          if (f[t].done) continue;
          g_emu.cur = &f[t];
          swapcontext(&g_emu.sched, &f[t].ctx);
          if (f[t].done) remaining--;
        }
      }
    }
  return 0;
}

/* ---- kernel bodies ------------------------------------------------------ */

struct d2b_args { float* dense; int* bits; };
static void d2b_body(void* p) {
  d2b_args* a = (d2b_args*)p;
  dense2bitmask<int, float>(a->dense, a->bits);
}

struct ggl_args {
  int* bits; int* gmask; signed char* gval; float* dense; int* gid;
  int* scnt; int* snnz; int* ht; int* htr; int* nnz;
};
static void ggl_body(void* p) {
  ggl_args* a = (ggl_args*)p;
  generate_groups_large<int, float, signed char>(a->bits, a->gmask, a->gval, a->dense, a->gid,
                                                 a->scnt, a->snnz, a->ht, a->htr, a->nnz);
}

struct g2d_args { float* gv; float* dense; int* gid; int* bits; };
static void g2d_body(void* p) {
  g2d_args* a = (g2d_args*)p;
  group2dense<float, int>(a->gv, a->dense, a->gid, a->bits);
}

struct lt_args { uint8_t* src8; float* srcf; int* dst; size_t row, col; int bw; };
static void lt8_body(void* p) {
  lt_args* a = (lt_args*)p;
  uint8_layout_trans(a->src8, a->dst, a->row, a->col);
}
static void ltf_body(void* p) {
  lt_args* a = (lt_args*)p;
  layout_trans(a->srcf, a->dst, a->row, a->col, a->bw);
}

struct us_args { int* mask; float* B; float* C; };
static void us_body(void* p) {
  us_args* a = (us_args*)p;
  uint8_spmm_2d_1d(a->mask, a->B, a->C);
}

/* ---- C ABI -------------------------------------------------------------- */
extern "C" {

/* dense2bitmask<int,float> on an M×K float matrix, launched like
 * source/src/main.cu:2036-2038 with the block size replaced by tile_rows
 * (the reference's SPLIT_K=2048 exceeds the 1024-thread limit).  The output
 * is zeroed first: the reference never clears dB_bitmask before its
 * atomicOr accumulation (main.cu:1950).  MSB-first words [M][K/32].        */
int ref_dense2bitmask(const float* dense, int M, int K, int tile_rows, int* words) {
  if (K % 32 || M % tile_rows) return -1;
  memset(words, 0, sizeof(int) * (size_t)M * (K / 32));
  d2b_args a = {const_cast<float*>(dense), words};
  return emu_launch(dim3(K / 32, M / tile_rows), dim3(tile_rows), d2b_body, &a);
}

/* generate_groups_large<int,float,signed char>, launched like
 * source/src/main.cu:2045-2059 with tile_rows threads per block.
 * words: MSB-first masks [M][K/32]; dense: the M×K matrix they came from.
 * Outputs: group_id [M][K/32], group_mask [T][2], group_val [T][2][32]
 * (int8, zero-initialised), spill_cnt/spill_nnz [T] (zeroed), hash tables
 * [T][2048], nnz [1] (zeroed).  T = (M/tile_rows)*(K/32).                 */
int ref_generate_groups_large(const int* words, const float* dense, int M, int K,
                              int tile_rows, int* group_id, int* group_mask,
                              signed char* group_val, int* spill_cnt, int* spill_nnz,
                              int* hash_table, int* hash_table_rev, int* nnz) {
  if (K % 32 || M % tile_rows || tile_rows > SPLIT_K) return -1;
  int T = (M / tile_rows) * (K / 32);
  memset(group_val, 0, (size_t)T * MAX_GROUP_NUM * TILE_WIDTH);
  memset(spill_cnt, 0, sizeof(int) * T);
  memset(spill_nnz, 0, sizeof(int) * T);
  *nnz = 0;
  ggl_args a = {const_cast<int*>(words), group_mask, group_val, const_cast<float*>(dense),
                group_id, spill_cnt, spill_nnz, hash_table, hash_table_rev, nnz};
  return emu_launch(dim3(K / 32, M / tile_rows), dim3(tile_rows), ggl_body, &a);
}

/* group2dense<float,int>: grid (N/32, M/tile_rows), block tile_rows, as the
 * commented call at source/src/main.cu:2250.  bitmask and group_idx are in
 * the reference's tile-major order: index (bid*tile_rows + row_in_tile)
 * with bid = row_block*(N/32) + word.                                      */
int ref_group2dense(const float* group_values, float* dense, const int* group_idx,
                    const int* bitmask_tile_major, int M, int N, int tile_rows) {
  if (N % 32 || M % tile_rows) return -1;
  g_size_n = N;
  g2d_args a = {const_cast<float*>(group_values), dense, const_cast<int*>(group_idx),
                const_cast<int*>(bitmask_tile_major)};
  return emu_launch(dim3(N / 32, M / tile_rows), dim3(tile_rows), g2d_body, &a);
}

/* uint8_layout_trans<<<m, k>>> (backup/layout_trans.cu:388): dst holds
 * 8 planes of one int per element. */
int ref_uint8_layout_trans(const uint8_t* src, int m, int k, int* dst) {
  lt_args a = {const_cast<uint8_t*>(src), nullptr, dst, (size_t)m, (size_t)k, 8};
  return emu_launch(dim3(m), dim3(k), lt8_body, &a);
}

/* layout_trans<<<m, k>>> over the float bit patterns (layout_trans.cu:75-85). */
int ref_layout_trans(const float* src, int m, int k, int bit_width, int* dst) {
  lt_args a = {nullptr, const_cast<float*>(src), dst, (size_t)m, (size_t)k, bit_width};
  return emu_launch(dim3(m), dim3(k), ltf_body, &a);
}

/* uint8_spmm_2d_1d over 8 mask planes [8][m][k] (one int per bit), B k×n,
 * C m×n zeroed first as main() does (layout_trans.cu:395).  Launched as the
 * kernel's own comment describes (gridDim.x = k, gridDim.y = m,
 * blockDim.x = n; layout_trans.cu:159-161): main() passes dim3(m, k)
 * (:398), which only agrees when m == k.                                   */
int ref_uint8_spmm(const int* mask, const float* B, float* C, int m, int k, int n) {
  memset(C, 0, sizeof(float) * (size_t)m * n);
  us_args a = {const_cast<int*>(mask), const_cast<float*>(B), C};
  return emu_launch(dim3(k, m), dim3(n), us_body, &a);
}

}  // extern "C"
