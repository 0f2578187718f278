/*
 * ref_emu_out.cpp — runs the reference's tiled-CSR conversion and symbolic
 * output pass on the CPU (fiber model of ref_shim.h) and exports them with
 * a C ABI for the oracle-pinning tests.  TEST INFRASTRUCTURE ONLY.
 *
 * The kernel bodies are not in this repository: build_ref.py extracts them
 * from the reference checkout into oracle/_ref/*.inc
 *   csr2tiledcsr   source/src/main.cu:499-588      (a <<<1,1>>> kernel)
 *   pre_spgemm     source/src/transform.cuh:984-1157
 * and this file includes each one inside a namespace per tile shape, so
 * the compile-time constants the reference takes from source/src/common.h
 * (TILE_HEIGHT, SPLIT_K, MAX_TILEA_NNZ) can differ between instantiations.
 * SIZE_M, SIZE_K and SIZE_N, fixed at 8192 there, are runtime values here.
 *
 * Conditions under which the extracted kernels compute what they mean to:
 *  - pre_spgemm loads B's row masks with blockDim.x = TILE_HEIGHT threads
 *    (transform.cuh:1044-1047) but indexes them with columns < SPLIT_K, so
 *    it is only defined for TILE_HEIGHT == SPLIT_K; the shapes below keep
 *    them equal.
 *  - pre_spgemm has no barrier at the end of its K-tile loop
 *    (transform.cuh:1050-1056): the next tile's loads may overwrite shared
 *    memory another warp still reads.  The serialised fibers take the worst
 *    order, so the pinning cases use one K tile (SIZE_K == SPLIT_K).
 *  - pre_spgemm reads MAX_TILEA_NNZ column entries past each tile's start
 *    (:1040-1043), past the end of the array for the last tiles; the
 *    wrapper pads the column array by MAX_TILEA_NNZ zeros.
 *  - a row that spills on the first pass makes one atomicCAS on
 *    output_row_group[-1] (:1075-1077 with output_group_idx = -1).  The
 *    shim's shared arrays are 4 KiB aligned and zero-initialised; the CAS
 *    compares that word with a nonzero group mask and so never writes.
 *  - the kernels' diagnostic printf lines (main.cu:579-585) are compiled
 *    out; they read tiled_csr_value[nnz-1] even when nnz == 0.
 */
#include "ref_shim.h"

#include <vector>

static int g_out_m = 0, g_out_k = 0, g_out_n = 0;

#define TILE_WIDTH 32
#define OUTPUT_MAX_GROUP_NUM 2
#define SIZE_M g_out_m
#define SIZE_K g_out_k
#define SIZE_N g_out_n
#define printf(...) ((void)0)

/* ---- tile shape 64 x 64 ------------------------------------------------- */
#define TILE_HEIGHT 64
#define SPLIT_K 64
#define MAX_TILEA_NNZ (64 * 64)
namespace shape64 {
#include "ref_csr2tiledcsr.inc"
#include "ref_pre_spgemm.inc"
}  // namespace shape64
#undef TILE_HEIGHT
#undef SPLIT_K
#undef MAX_TILEA_NNZ

/* ---- tile shape 256 x 256 ----------------------------------------------- */
#define TILE_HEIGHT 256
#define SPLIT_K 256
#define MAX_TILEA_NNZ (256 * 256)
namespace shape256 {
#include "ref_csr2tiledcsr.inc"
#include "ref_pre_spgemm.inc"
}  // namespace shape256
#undef TILE_HEIGHT
#undef SPLIT_K
#undef MAX_TILEA_NNZ

/* ---- tile shape 32 x 128 (csr2tiledcsr only: tiles need not be square) -- */
#define TILE_HEIGHT 32
#define SPLIT_K 128
namespace shape32x128 {
#include "ref_csr2tiledcsr.inc"
}  // namespace shape32x128
#undef TILE_HEIGHT
#undef SPLIT_K

#undef printf

/* ---- kernel bodies ------------------------------------------------------ */

struct c2t_args {
  int tiles; int64_t nnz; int* off; int* col; float* val;
  int* toff; int* tcol; float* tval; int* acc; int* tnnz; int* trow;
};

template <int H, int W>
static void c2t_body(void* p) {
  c2t_args* a = (c2t_args*)p;
  if (H == 64 && W == 64)
    shape64::csr2tiledcsr<float, float>(a->tiles, a->nnz, a->off, a->col, a->val, a->toff,
                                        a->tcol, a->tval, a->acc, a->tnnz, a->trow);
  else if (H == 256 && W == 256)
    shape256::csr2tiledcsr<float, float>(a->tiles, a->nnz, a->off, a->col, a->val, a->toff,
                                         a->tcol, a->tval, a->acc, a->tnnz, a->trow);
  else
    shape32x128::csr2tiledcsr<float, float>(a->tiles, a->nnz, a->off, a->col, a->val, a->toff,
                                            a->tcol, a->tval, a->acc, a->tnnz, a->trow);
}

struct pre_args {
  int* bbits; int* scnt; int* snnz; int* toff; int* tcol; int* acc; int* gidx;
  int* cbits; int* gmask; int* rrow; int* rtile; int* rcnt_off; int* nnz_off;
  int* rbuf; int* nbuf; int* nnz;
};

template <int H>
static void pre_body(void* p) {
  pre_args* a = (pre_args*)p;
  if (H == 64)
    shape64::pre_spgemm<int>(a->bbits, a->scnt, a->snnz, a->toff, a->tcol, a->acc, a->gidx,
                             a->cbits, a->gmask, a->rrow, a->rtile, a->rcnt_off, a->nnz_off,
                             a->rbuf, a->nbuf, a->nnz);
  else
    shape256::pre_spgemm<int>(a->bbits, a->scnt, a->snnz, a->toff, a->tcol, a->acc, a->gidx,
                              a->cbits, a->gmask, a->rrow, a->rtile, a->rcnt_off, a->nnz_off,
                              a->rbuf, a->nbuf, a->nnz);
}

/* ---- C ABI -------------------------------------------------------------- */
extern "C" {

/* csr2tiledcsr<float,float><<<1,1>>> as source/src/main.cu:2016-2027
 * launches it, tiles of tile_h rows x tile_w columns (64x64, 256x256 or
 * 32x128).  M % tile_h == 0 and K % tile_w == 0 (the reference's shapes).
 * Outputs, zeroed here as the caller's cudaMalloc'd buffers would need:
 * tile_nnz_acc [T+1], tile_nnz [T], tile_row_nnz [M][K/tile_w],
 * tiled_offset [T][tile_h+1], tiled_col [nnz], tiled_val [nnz].            */
int ref_csr2tiledcsr(const int* row_ptr, const int* col, const float* val, int M, int K,
                     int tile_h, int tile_w, int* tile_nnz_acc, int* tile_nnz,
                     int* tile_row_nnz, int* tiled_offset, int* tiled_col, float* tiled_val) {
  if (!((tile_h == 64 && tile_w == 64) || (tile_h == 256 && tile_w == 256) ||
        (tile_h == 32 && tile_w == 128)))
    return -1;
  if (M % tile_h || K % tile_w) return -1;
  int T = (M / tile_h) * (K / tile_w);
  int64_t nnz = row_ptr[M];
  memset(tile_nnz_acc, 0, sizeof(int) * (T + 1));
  memset(tile_nnz, 0, sizeof(int) * T);
  memset(tile_row_nnz, 0, sizeof(int) * (size_t)M * (K / tile_w));
  memset(tiled_offset, 0, sizeof(int) * (size_t)T * (tile_h + 1));
  g_out_m = M;
  g_out_k = K;
  c2t_args a = {T, nnz, const_cast<int*>(row_ptr), const_cast<int*>(col),
                const_cast<float*>(val), tiled_offset, tiled_col, tiled_val,
                tile_nnz_acc, tile_nnz, tile_row_nnz};
  emu_body_fn body = tile_h == 64 ? c2t_body<64, 64>
                   : tile_h == 256 ? c2t_body<256, 256> : c2t_body<32, 128>;
  return emu_launch(dim3(1), dim3(1), body, &a);
}

/* pre_spgemm<int> launched as source/src/main.cu:2153-2172: grid (N/32,
 * M/tile), block tile, with tile = TILE_HEIGHT = SPLIT_K in {64, 256} and
 * K == tile (one K tile; see the header).  Inputs: B's row masks [K][N/32]
 * (any bit order; the pass only ORs them) and A's tiled CSR from
 * ref_csr2tiledcsr with the same tile.  Outputs in the kernel's tile-major
 * order, index (rb*(N/32) + w)*tile + r: output masks c_bits and output
 * group ids group_idx; group masks [T][2]; spill counters [T] (zeroed);
 * nnz [1] = Σ popcount(group masks) (zeroed).                              */
int ref_pre_spgemm(const int* b_bits, const int* tiled_offset, const int* tiled_col,
                   const int* tile_nnz_acc, int M, int K, int N, int tile, int* c_bits,
                   int* group_idx, int* group_mask, int* spill_cnt, int* spill_nnz, int* nnz) {
  if (tile != 64 && tile != 256) return -1;
  if (K != tile || M % tile || N % 32) return -1;
  int T = (M / tile) * (N / 32);
  int tilesA = M / tile;
  int64_t nnzA = tile_nnz_acc[tilesA];
  int pad = tile * tile;
  std::vector<int> col((size_t)nnzA + pad, 0);
  memcpy(col.data(), tiled_col, sizeof(int) * (size_t)nnzA);
  std::vector<int> rrow(1), rtile(1), rcnt_off(T + 1), nnz_off(T + 1), rbuf(1), nbuf(1);
  memset(spill_cnt, 0, sizeof(int) * T);
  memset(spill_nnz, 0, sizeof(int) * T);
  *nnz = 0;
  g_out_m = M;
  g_out_k = K;
  g_out_n = N;
  pre_args a = {const_cast<int*>(b_bits), spill_cnt, spill_nnz,
                const_cast<int*>(tiled_offset), col.data(), const_cast<int*>(tile_nnz_acc),
                group_idx, c_bits, group_mask, rrow.data(), rtile.data(), rcnt_off.data(),
                nnz_off.data(), rbuf.data(), nbuf.data(), nnz};
  return emu_launch(dim3(N / 32, M / tile), dim3(tile), tile == 64 ? pre_body<64> : pre_body<256>,
                    &a);
}

}  // extern "C"
