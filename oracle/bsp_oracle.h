/*
 * bsp_oracle.h — CPU restatement of the reference's bitmap-SpMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  These functions are the checker for the CUDA
 * library: only the tests, the smoke check and the benchmark's CPU-baseline
 * leg may call them.  The library never calls, links or falls back to them.
 *
 * Every function names the reference file:line whose behaviour it restates
 * (paths relative to the ZSL98/bitwise_spgemm project root).
 */
#ifndef BSP_ORACLE_H_
#define BSP_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* dtype codes match enum bsp_dtype in include/bsp.h */
enum { ORC_F32 = 0, ORC_F16 = 1, ORC_BF16 = 2, ORC_I8 = 3, ORC_U8 = 4 };

int orc_pack_rows(const void* dense, int dtype, int64_t M, int64_t K,
                  int64_t ld, uint32_t* words, int msb_first);
int orc_pack_cols(const void* dense, int dtype, int64_t M, int64_t K,
                  int64_t ld, uint32_t* words_t, int msb_first);
void orc_transpose_bits(const uint32_t* words, int64_t M, int64_t K,
                        uint32_t* words_t);
void orc_unpack_rows_f32(const uint32_t* words, int64_t M, int64_t K,
                         float* dense, int64_t ld, int msb_first);
int orc_bitplanes(const uint8_t* v, int64_t M, int64_t K, int64_t ld,
                  int planes, uint32_t* words, int msb_first);

int orc_group_rows(const uint32_t* words, int64_t M, int64_t Kw,
                   int tile_rows, int max_groups, int32_t* group_id,
                   uint32_t* group_mask, int32_t* group_row,
                   int32_t* spill_cnt, int32_t* spill_nnz,
                   int32_t* spill_rows, int64_t* grouped_nnz);
void orc_group_to_dense(const float* group_values, const int32_t* group_id,
                        const uint32_t* words, int64_t M, int64_t K,
                        int tile_rows, int max_groups, float* dense,
                        int64_t ldd);

void orc_spmm_f64(const uint32_t* words, int64_t M, int64_t K, const float* B,
                  int64_t ldb, int64_t N, double* C, int64_t ldc);
void orc_spmm_abs_f64(const uint32_t* words, int64_t M, int64_t K,
                      const float* B, int64_t ldb, int64_t N, double* C,
                      int64_t ldc);
void orc_spmm_f32(const uint32_t* words, int64_t M, int64_t K, const float* B,
                  int64_t ldb, int64_t N, float* C, int64_t ldc);
void orc_spmm_f32_mt(const uint32_t* words, int64_t M, int64_t K,
                     const float* B, int64_t ldb, int64_t N, float* C,
                     int64_t ldc, int threads);
void orc_spmm_t_f64(const uint32_t* words, int64_t M, int64_t K,
                    const float* G, int64_t ldg, int64_t N, double* dB,
                    int64_t lddb);
void orc_sddmm_f64(const uint32_t* words, int64_t M, int64_t K,
                   const float* G, int64_t ldg, const float* X, int64_t ldx,
                   int64_t N, double* vals);

void orc_dense_check_sum(const float* A, const float* B, float* C, int m,
                         int n, int k);
int64_t orc_check(const float* A, const float* B, const float* C, int m,
                  int n, int k);
void orc_dense_check_sum_mt(const float* A, const float* B, float* C, int m,
                            int n, int k, int row0, int row1, int threads);

void orc_symbolic_rows(const uint32_t* a_words, int64_t M, int64_t K,
                       const uint32_t* b_words, int64_t N, uint32_t* c_words);
void orc_bitplane_spmm_f64(const int8_t* A, int64_t M, int64_t K,
                           int64_t lda, const float* B, int64_t ldb,
                           int64_t N, double* C, int64_t ldc);

/* 8x8 bitmap tiles of packed LSB-first rows (tSparse format,
 * coo2bmp_noTuple_d, source/src/main.cu:692-779, find_tile_index,
 * source/src/mm.h:83-104): returns the number n of nonzero tiles, written in
 * ascending tile_row*ceil(K/8)+tile_col order with bit (r%8)*8 + c%8, and
 * offset[0..n] = exclusive scan of their popcounts.                        */
int64_t orc_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K,
                           uint64_t* bmp, int32_t* tile_row, int32_t* tile_col,
                           int32_t* offset);
void orc_tiles8_to_rows(const uint64_t* bmp, const int32_t* tile_row,
                        const int32_t* tile_col, int64_t n, int64_t M,
                        int64_t K, uint32_t* words);
/* CSR -> tiled CSR of csr2tiledcsr, source/src/main.cu:499-588, with the
 * tile shape as parameters (TILE_HEIGHT x SPLIT_K there).                  */
void orc_csr_to_tiled(const int32_t* row_ptr, const int32_t* col,
                      const float* val, int64_t M, int64_t K, int tile_rows,
                      int tile_cols, int32_t* tile_nnz_acc,
                      int32_t* tiled_offset, int32_t* tiled_col,
                      float* tiled_val);

#ifdef __cplusplus
}
#endif
#endif
