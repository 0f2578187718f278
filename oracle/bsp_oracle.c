/*
 * bsp_oracle.c — CPU restatement of the reference's bitmap-SpMM path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only the
 * tests, the smoke check and the benchmark's CPU-baseline leg may load this
 * code; the library never links it and has no CPU fallback.
 *
 * Reference = ZSL98/bitwise_spgemm; paths below are relative to its root.
 * Plain C99 + pthreads, no intrinsics, identical results on x86-64 and Arm.
 */
#include "bsp_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static int64_t ceil32(int64_t k) { return (k + 31) / 32; }

static int popc32(uint32_t x) {
  int c = 0;
  while (x) { x &= x - 1; c++; }
  return c;
}

static uint32_t brev32(uint32_t x) {
  uint32_t r = 0;
  for (int i = 0; i < 32; i++) r |= ((x >> i) & 1u) << (31 - i);
  return r;
}

/* Nonzero test of one element.  dense2bitmask (source/src/main.cu:617) tests
 * `MatB_dense[...] != 0`: for floats -0.0 is zero and NaN is nonzero; for
 * half/bfloat16 the same holds for the bit pattern with the sign cleared.   */
static int nonzero_at(const void* p, int dtype, int64_t idx) {
  switch (dtype) {
    case ORC_F32: return ((const float*)p)[idx] != 0.0f;
    case ORC_F16:
    case ORC_BF16: return (((const uint16_t*)p)[idx] & 0x7FFFu) != 0;
    case ORC_I8: return ((const int8_t*)p)[idx] != 0;
    case ORC_U8: return ((const uint8_t*)p)[idx] != 0;
    default: return -1;
  }
}

/* Restates dense2bitmask, source/src/main.cu:591-628: one word per (row,
 * 32-column tile), word index row*(cols/32)+tile (:597-598), column i of the
 * tile at bit 31-i (:619) in MSB mode, at bit i in LSB mode.  Ragged K: the
 * bits past column K-1 stay zero.                                            */
int orc_pack_rows(const void* dense, int dtype, int64_t M, int64_t K,
                  int64_t ld, uint32_t* words, int msb_first) {
  if (dtype < ORC_F32 || dtype > ORC_U8) return -1;
  int64_t Kw = ceil32(K);
  for (int64_t r = 0; r < M; r++) {
    for (int64_t w = 0; w < Kw; w++) {
      uint32_t word = 0;
      for (int i = 0; i < 32; i++) {
        int64_t c = w * 32 + i;
        if (c < K && nonzero_at(dense, dtype, r * ld + c)) word |= 1u << i;
      }
      words[r * Kw + w] = msb_first ? brev32(word) : word;
    }
  }
  return 0;
}

/* Column-packed form of the same test: words_t[k][w] bit i = A[32w+i][k]. */
int orc_pack_cols(const void* dense, int dtype, int64_t M, int64_t K,
                  int64_t ld, uint32_t* words_t, int msb_first) {
  if (dtype < ORC_F32 || dtype > ORC_U8) return -1;
  int64_t Mw = ceil32(M);
  for (int64_t k = 0; k < K; k++) {
    for (int64_t w = 0; w < Mw; w++) {
      uint32_t word = 0;
      for (int i = 0; i < 32; i++) {
        int64_t r = w * 32 + i;
        if (r < M && nonzero_at(dense, dtype, r * ld + k)) word |= 1u << i;
      }
      words_t[k * Mw + w] = msb_first ? brev32(word) : word;
    }
  }
  return 0;
}

void orc_transpose_bits(const uint32_t* words, int64_t M, int64_t K,
                        uint32_t* words_t) {
  int64_t Kw = ceil32(K), Mw = ceil32(M);
  memset(words_t, 0, (size_t)(K * Mw) * sizeof(uint32_t));
  for (int64_t r = 0; r < M; r++)
    for (int64_t k = 0; k < K; k++)
      if ((words[r * Kw + k / 32] >> (k % 32)) & 1u)
        words_t[k * Mw + r / 32] |= 1u << (r % 32);
}

void orc_unpack_rows_f32(const uint32_t* words, int64_t M, int64_t K,
                         float* dense, int64_t ld, int msb_first) {
  int64_t Kw = ceil32(K);
  for (int64_t r = 0; r < M; r++)
    for (int64_t c = 0; c < K; c++) {
      uint32_t w = words[r * Kw + c / 32];
      int bit = msb_first ? 31 - (int)(c % 32) : (int)(c % 32);
      dense[r * ld + c] = (float)((w >> bit) & 1u);
    }
}

/* Restates uint8_layout_trans, backup/layout_trans.cu:87-97: plane b holds
 * ((uint8)v >> b) & 1 (:95), planes stored one after another (b*M*K, :95);
 * here each plane is packed 32 columns per word instead of one int per bit. */
int orc_bitplanes(const uint8_t* v, int64_t M, int64_t K, int64_t ld,
                  int planes, uint32_t* words, int msb_first) {
  if (planes < 1 || planes > 8) return -1;
  int64_t Kw = ceil32(K);
  for (int b = 0; b < planes; b++)
    for (int64_t r = 0; r < M; r++)
      for (int64_t w = 0; w < Kw; w++) {
        uint32_t word = 0;
        for (int i = 0; i < 32; i++) {
          int64_t c = w * 32 + i;
          if (c < K && ((v[r * ld + c] >> b) & 1u)) word |= 1u << i;
        }
        words[((int64_t)b * M + r) * Kw + w] = msb_first ? brev32(word) : word;
      }
  return 0;
}

/* Restates generate_groups_large, source/src/main.cu:50-247, with its
 * shared-memory atomicCAS race serialised in ascending row order:
 *  - tile = (row block of tile_rows rows, one word column w); tiles numbered
 *    rb*Kw + w like bid = blockIdx.y*gridDim.x + blockIdx.x (:64);
 *  - a zero word goes to group 0 and leaves the masks alone (:105-108);
 *  - otherwise the first group whose mask does not intersect the word takes
 *    it (:112-127, :164-180) and ORs it in (:131-133);
 *  - no group fits: the row spills, group_id = -1 (:124, :156), spilled row
 *    count and popcount grow (:157-166), the row is appended to the tile's
 *    spill list (spilled_row_hash_table, :158);
 *  - group_row[g][i] = local row owning bit i of group g (:186-190);
 *  - grouped_nnz = Σ popcount(group masks) (:199-204).
 * Deviation (reference bug): the reference overwrites the -1 with the group
 * counter (= max_groups) at :184; here spilled rows keep -1.                 */
int orc_group_rows(const uint32_t* words, int64_t M, int64_t Kw,
                   int tile_rows, int max_groups, int32_t* group_id,
                   uint32_t* group_mask, int32_t* group_row,
                   int32_t* spill_cnt, int32_t* spill_nnz,
                   int32_t* spill_rows, int64_t* grouped_nnz) {
  if (tile_rows < 1 || max_groups < 1 || max_groups > 32) return -1;
  int64_t n_rb = (M + tile_rows - 1) / tile_rows;
  int64_t total = 0;
  uint32_t gm[32];
  for (int64_t rb = 0; rb < n_rb; rb++) {
    for (int64_t w = 0; w < Kw; w++) {
      int64_t t = rb * Kw + w;
      int32_t nsp = 0, nspnnz = 0;
      for (int g = 0; g < max_groups; g++) gm[g] = 0;
      if (group_row)
        for (int64_t i = 0; i < (int64_t)max_groups * 32; i++)
          group_row[t * max_groups * 32 + i] = -1;
      if (spill_rows)
        for (int64_t i = 0; i < tile_rows; i++) spill_rows[t * tile_rows + i] = -1;
      for (int64_t lr = 0; lr < tile_rows; lr++) {
        int64_t r = rb * tile_rows + lr;
        if (r >= M) break;
        uint32_t m = words[r * Kw + w];
        int g = 0;
        if (m != 0) {
          while (g < max_groups && (gm[g] & m) != 0) g++;
          if (g == max_groups) {
            g = -1;
            if (spill_rows) spill_rows[t * tile_rows + nsp] = (int32_t)lr;
            nsp++;
            nspnnz += popc32(m);
          } else {
            gm[g] |= m;
            if (group_row)
              for (int i = 0; i < 32; i++)
                if ((m >> i) & 1u) group_row[(t * max_groups + g) * 32 + i] = (int32_t)lr;
          }
        }
        group_id[r * Kw + w] = g;
      }
      for (int g = 0; g < max_groups; g++) {
        group_mask[t * max_groups + g] = gm[g];
        total += popc32(gm[g]);
      }
      if (spill_cnt) spill_cnt[t] = nsp;
      if (spill_nnz) spill_nnz[t] = nspnnz;
    }
  }
  if (grouped_nnz) *grouped_nnz = total;
  return 0;
}

/* Restates group2dense, source/src/main.cu:829-850: rows with a group
 * (:836) copy, for each set bit i of their word (:840), the group's value at
 * position i (:842-844) to the dense output.  LSB-first bits, row-major words
 * and runtime sizes instead of the reference's MSB-first, tile-major arrays
 * and SIZE_N.                                                               */
void orc_group_to_dense(const float* group_values, const int32_t* group_id,
                        const uint32_t* words, int64_t M, int64_t K,
                        int tile_rows, int max_groups, float* dense,
                        int64_t ldd) {
  int64_t Kw = ceil32(K);
  for (int64_t r = 0; r < M; r++) {
    int64_t rb = r / tile_rows;
    for (int64_t w = 0; w < Kw; w++) {
      int32_t g = group_id[r * Kw + w];
      if (g < 0) continue;
      uint32_t m = words[r * Kw + w];
      int64_t t = rb * Kw + w;
      for (int i = 0; i < 32; i++)
        if (((m >> i) & 1u) && w * 32 + i < K)
          dense[r * ldd + w * 32 + i] = group_values[(t * max_groups + g) * 32 + i];
    }
  }
}

/* C = A·B with A given by packed LSB-first row words: the 0/1-mask SpMM of
 * backup/layout_trans.cu:158-171 (add row k of B for every set bit k of row
 * i) accumulated in double, k ascending.                                    */
void orc_spmm_f64(const uint32_t* words, int64_t M, int64_t K, const float* B,
                  int64_t ldb, int64_t N, double* C, int64_t ldc) {
  int64_t Kw = ceil32(K);
  for (int64_t i = 0; i < M; i++) {
    double* c = C + i * ldc;
    for (int64_t j = 0; j < N; j++) c[j] = 0.0;
    for (int64_t w = 0; w < Kw; w++) {
      uint32_t m = words[i * Kw + w];
      while (m) {
        int b = 0;
        while (!((m >> b) & 1u)) b++;
        m &= m - 1;
        const float* brow = B + (w * 32 + b) * ldb;
        for (int64_t j = 0; j < N; j++) c[j] += (double)brow[j];
      }
    }
  }
}

/* Σ_k A_ik |B_kj| in double: the scale of the FP32 summation error bound,
 * used to normalise componentwise errors.                                   */
void orc_spmm_abs_f64(const uint32_t* words, int64_t M, int64_t K,
                      const float* B, int64_t ldb, int64_t N, double* C,
                      int64_t ldc) {
  int64_t Kw = ceil32(K);
  for (int64_t i = 0; i < M; i++) {
    double* c = C + i * ldc;
    for (int64_t j = 0; j < N; j++) c[j] = 0.0;
    for (int64_t w = 0; w < Kw; w++) {
      uint32_t m = words[i * Kw + w];
      while (m) {
        int b = 0;
        while (!((m >> b) & 1u)) b++;
        m &= m - 1;
        const float* brow = B + (w * 32 + b) * ldb;
        for (int64_t j = 0; j < N; j++) c[j] += fabs((double)brow[j]);
      }
    }
  }
}

/* FP32 sum in the order of the reference's CPU check(),
 * backup/bit_wise_gemm.cu:18-22 (p ascending, `sum += A*B` in float).  For a
 * 0/1 A the skipped terms are exact zeros, so this equals check()'s sum up
 * to the sign of a zero result.                                            */
void orc_spmm_f32(const uint32_t* words, int64_t M, int64_t K, const float* B,
                  int64_t ldb, int64_t N, float* C, int64_t ldc) {
  int64_t Kw = ceil32(K);
  for (int64_t i = 0; i < M; i++) {
    float* c = C + i * ldc;
    for (int64_t j = 0; j < N; j++) c[j] = 0.0f;
    for (int64_t w = 0; w < Kw; w++) {
      uint32_t m = words[i * Kw + w];
      while (m) {
        int b = 0;
        while (!((m >> b) & 1u)) b++;
        m &= m - 1;
        const float* brow = B + (w * 32 + b) * ldb;
        for (int64_t j = 0; j < N; j++) c[j] += brow[j];
      }
    }
  }
}

typedef struct {
  const uint32_t* words; int64_t M, K; const float* B; int64_t ldb, N;
  float* C; int64_t ldc; int64_t r0, r1;
} spmm_job;

static void* spmm_worker(void* p) {
  spmm_job* j = (spmm_job*)p;
  int64_t Kw = ceil32(j->K);
  orc_spmm_f32(j->words + j->r0 * Kw, j->r1 - j->r0, j->K, j->B, j->ldb, j->N,
               j->C + j->r0 * j->ldc, j->ldc);
  return NULL;
}

/* orc_spmm_f32 with rows split over `threads` pthreads (same per-row order). */
void orc_spmm_f32_mt(const uint32_t* words, int64_t M, int64_t K,
                     const float* B, int64_t ldb, int64_t N, float* C,
                     int64_t ldc, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t th[256];
  spmm_job jobs[256];
  for (int t = 0; t < threads; t++) {
    spmm_job jb = {words, M, K, B, ldb, N, C, ldc, M * t / threads,
                   M * (t + 1) / threads};
    jobs[t] = jb;
    pthread_create(&th[t], NULL, spmm_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
}

/* dB = Aᵀ·G: dB[k][j] = Σ_i A_ik G[i][j], double accumulation, i ascending. */
void orc_spmm_t_f64(const uint32_t* words, int64_t M, int64_t K,
                    const float* G, int64_t ldg, int64_t N, double* dB,
                    int64_t lddb) {
  int64_t Kw = ceil32(K);
  for (int64_t k = 0; k < K; k++)
    for (int64_t j = 0; j < N; j++) dB[k * lddb + j] = 0.0;
  for (int64_t i = 0; i < M; i++)
    for (int64_t w = 0; w < Kw; w++) {
      uint32_t m = words[i * Kw + w];
      while (m) {
        int b = 0;
        while (!((m >> b) & 1u)) b++;
        m &= m - 1;
        int64_t k = w * 32 + b;
        for (int64_t j = 0; j < N; j++) dB[k * lddb + j] += (double)G[i * ldg + j];
      }
    }
}

/* Straight-through mask gradient sampled at the set bits of A:
 * vals[e] = Σ_j G[i][j]·X[k][j] for the e-th set bit (i,k) in row-major,
 * k-ascending order (dL/dA for loss = Σ (A·X) ⊙ G).                       */
void orc_sddmm_f64(const uint32_t* words, int64_t M, int64_t K,
                   const float* G, int64_t ldg, const float* X, int64_t ldx,
                   int64_t N, double* vals) {
  int64_t Kw = ceil32(K), e = 0;
  for (int64_t i = 0; i < M; i++)
    for (int64_t w = 0; w < Kw; w++) {
      uint32_t m = words[i * Kw + w];
      while (m) {
        int b = 0;
        while (!((m >> b) & 1u)) b++;
        m &= m - 1;
        int64_t k = w * 32 + b;
        double s = 0.0;
        for (int64_t j = 0; j < N; j++) s += (double)G[i * ldg + j] * (double)X[k * ldx + j];
        vals[e++] = s;
      }
    }
}

/* The reference's CPU path, check() of backup/bit_wise_gemm.cu:13-32:
 * dense row-major A (m×k) times row-major B (k×n), FP32 `sum += A*B` with
 * p ascending (:18-22).  orc_dense_check_sum stores the sums;
 * orc_check returns -1 when every |sum - C| / |sum| <= 1e-5 (:24), else the
 * flat index of the first failing element, like check()'s early return.    */
void orc_dense_check_sum(const float* A, const float* B, float* C, int m,
                         int n, int k) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      float sum = 0.f;
      for (int p = 0; p < k; ++p) sum += A[i * k + p] * B[j + p * n];
      C[i * n + j] = sum;
    }
}

int64_t orc_check(const float* A, const float* B, const float* C, int m,
                  int n, int k) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      float sum = 0.f;
      for (int p = 0; p < k; ++p) sum += A[i * k + p] * B[j + p * n];
      if (fabsf(sum - C[i * n + j]) / fabsf(sum) > 1e-5f) return (int64_t)i * n + j;
    }
  return -1;
}

typedef struct {
  const float *A, *B; float* C; int m, n, k, r0, r1;
} dense_job;

static void* dense_worker(void* p) {
  dense_job* j = (dense_job*)p;
  for (int i = j->r0; i < j->r1; ++i)
    for (int jj = 0; jj < j->n; ++jj) {
      float sum = 0.f;
      for (int q = 0; q < j->k; ++q) sum += j->A[(int64_t)i * j->k + q] * j->B[jj + (int64_t)q * j->n];
      j->C[(int64_t)i * j->n + jj] = sum;
    }
  return NULL;
}

/* check()'s triple loop over rows [row0, row1) split across pthreads; every
 * element is summed exactly as in orc_dense_check_sum.                     */
void orc_dense_check_sum_mt(const float* A, const float* B, float* C, int m,
                            int n, int k, int row0, int row1, int threads) {
  (void)m;
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t th[256];
  dense_job jobs[256];
  int rows = row1 - row0;
  for (int t = 0; t < threads; t++) {
    dense_job jb = {A, B, C, m, n, k, row0 + rows * t / threads,
                    row0 + rows * (t + 1) / threads};
    jobs[t] = jb;
    pthread_create(&th[t], NULL, dense_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
}

/* Symbolic output mask of pre_spgemm, source/src/transform.cuh:1028-1057:
 * the mask of C's row i in word column w is the OR of B's row masks
 * b_words[k][w] over the set bits k of A's row i.                          */
void orc_symbolic_rows(const uint32_t* a_words, int64_t M, int64_t K,
                       const uint32_t* b_words, int64_t N, uint32_t* c_words) {
  int64_t Kw = ceil32(K), Nw = ceil32(N);
  for (int64_t i = 0; i < M; i++) {
    uint32_t* c = c_words + i * Nw;
    for (int64_t w = 0; w < Nw; w++) c[w] = 0;
    for (int64_t kw = 0; kw < Kw; kw++) {
      uint32_t m = a_words[i * Kw + kw];
      while (m) {
        int b = 0;
        while (!((m >> b) & 1u)) b++;
        m &= m - 1;
        const uint32_t* br = b_words + (kw * 32 + b) * Nw;
        for (int64_t w = 0; w < Nw; w++) c[w] |= br[w];
      }
    }
  }
}

/* Bit-serial int8 × dense product of spgemm_compute_1dthread_tcore_v3
 * (source/src/transform.cuh:2199-2246) with the plane weights 1,2,...,64,-128
 * of initialize_multiplicand (source/src/main.cu:895-910): for two's
 * complement int8 A this is exactly A·B; computed plane by plane in double. */
void orc_bitplane_spmm_f64(const int8_t* A, int64_t M, int64_t K,
                           int64_t lda, const float* B, int64_t ldb,
                           int64_t N, double* C, int64_t ldc) {
  static const double wts[8] = {1, 2, 4, 8, 16, 32, 64, -128};
  for (int64_t i = 0; i < M; i++) {
    double* c = C + i * ldc;
    for (int64_t j = 0; j < N; j++) c[j] = 0.0;
    for (int b = 0; b < 8; b++)
      for (int64_t k = 0; k < K; k++)
        if ((((uint8_t)A[i * lda + k]) >> b) & 1u) {
          const float* brow = B + k * ldb;
          for (int64_t j = 0; j < N; j++) c[j] += wts[b] * (double)brow[j];
        }
  }
}

/* 8x8 bitmap tiles, source/src/main.cu:692-779 (tile index = row/8 *
 * ncols8 + col/8, position bit = (row%8)*8 + col%8, tiles reduced by OR in
 * ascending tile index, offsets = exclusive scan of the popcounts).        */
int64_t orc_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K,
                           uint64_t* bmp, int32_t* tile_row, int32_t* tile_col,
                           int32_t* offset) {
  int64_t Kw = ceil32(K), Mt = (M + 7) / 8, Kt = (K + 7) / 8, n = 0, run = 0;
  for (int64_t ty = 0; ty < Mt; ty++)
    for (int64_t tx = 0; tx < Kt; tx++) {
      uint64_t m = 0;
      for (int64_t r = 0; r < 8; r++) {
        int64_t row = ty * 8 + r;
        if (row >= M) break;
        for (int64_t c = 0; c < 8; c++) {
          int64_t col = tx * 8 + c;
          if (col >= K) break;
          if ((words[row * Kw + col / 32] >> (col % 32)) & 1u) m |= 1ull << (r * 8 + c);
        }
      }
      if (!m) continue;
      bmp[n] = m;
      tile_row[n] = (int32_t)ty;
      tile_col[n] = (int32_t)tx;
      offset[n] = (int32_t)run;
      for (int b = 0; b < 64; b++) run += (m >> b) & 1u;
      n++;
    }
  offset[n] = (int32_t)run;
  return n;
}

void orc_tiles8_to_rows(const uint64_t* bmp, const int32_t* tile_row,
                        const int32_t* tile_col, int64_t n, int64_t M,
                        int64_t K, uint32_t* words) {
  int64_t Kw = ceil32(K);
  for (int64_t i = 0; i < M * Kw; i++) words[i] = 0;
  for (int64_t t = 0; t < n; t++)
    for (int b = 0; b < 64; b++) {
      if (!((bmp[t] >> b) & 1u)) continue;
      int64_t row = (int64_t)tile_row[t] * 8 + b / 8, col = (int64_t)tile_col[t] * 8 + b % 8;
      if (row < M && col < K) words[row * Kw + col / 32] |= 1u << (col % 32);
    }
}

/* csr2tiledcsr, source/src/main.cu:499-588: tile (ty, tx) of tile_rows x
 * tile_cols, id ty*ceil(K/tile_cols)+tx; its entries in row order, each row's
 * in CSR order; local column col % tile_cols; tile_nnz_acc = exclusive scan
 * of the tiles' entry counts (T+1 values); tiled_offset[(tile_rows+1)*t + j]
 * = entries of the tile in its local rows before j.                        */
void orc_csr_to_tiled(const int32_t* row_ptr, const int32_t* col,
                      const float* val, int64_t M, int64_t K, int tile_rows,
                      int tile_cols, int32_t* tile_nnz_acc,
                      int32_t* tiled_offset, int32_t* tiled_col,
                      float* tiled_val) {
  int64_t Mt = (M + tile_rows - 1) / tile_rows, Kt = (K + tile_cols - 1) / tile_cols, T = Mt * Kt;
  int32_t* cnt = (int32_t*)calloc((size_t)T, sizeof(int32_t));
  int32_t* fill = (int32_t*)calloc((size_t)T, sizeof(int32_t));
  for (int64_t i = 0; i < M; i++)
    for (int32_t j = row_ptr[i]; j < row_ptr[i + 1]; j++) cnt[(i / tile_rows) * Kt + col[j] / tile_cols]++;
  int32_t run = 0;
  for (int64_t t = 0; t < T; t++) {
    tile_nnz_acc[t] = run;
    run += cnt[t];
  }
  tile_nnz_acc[T] = run;
  for (int64_t t = 0; t < T; t++) {
    int64_t ty = t / Kt, tx = t % Kt;
    int32_t r = 0;
    for (int j = 0; j < tile_rows; j++) {
      tiled_offset[(tile_rows + 1) * t + j] = r;
      int64_t row = ty * tile_rows + j;
      if (row < M)
        for (int32_t e = row_ptr[row]; e < row_ptr[row + 1]; e++) r += (col[e] / tile_cols == tx);
    }
    tiled_offset[(tile_rows + 1) * t + tile_rows] = r;
  }
  for (int64_t i = 0; i < M; i++)
    for (int32_t j = row_ptr[i]; j < row_ptr[i + 1]; j++) {
      int64_t t = (i / tile_rows) * Kt + col[j] / tile_cols;
      int32_t e = tile_nnz_acc[t] + fill[t]++;
      tiled_col[e] = col[j] % tile_cols;
      if (val && tiled_val) tiled_val[e] = val[j];
    }
  free(cnt);
  free(fill);
}
