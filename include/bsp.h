/*
 * bsp.h — C ABI of the GB300 (sm_103a) bitmap SpMM library.
 *
 * The operation is C = A·B where A is an M×K 0/1 matrix stored as packed
 * 32-bit row bitmasks and B is a dense K×N matrix.  Every entry point takes
 * caller-owned device buffers, an explicit CUDA stream and returns an int
 * status (0 = BSP_OK, negative = error).  No entry point aborts the process.
 *
 * The reference (ZSL98/bitwise_spgemm) has no library API: its kernels are
 * raw __global__ functions launched from main() on the default stream, with
 * caller-cudaMalloc'ed buffers and shapes fixed by #defines
 * (source/src/common.h:15-35).  Each declaration below names the reference
 * kernel or host function it replaces; shapes and layouts that were
 * compile-time constants there are runtime parameters here.
 *
 * Packed-word layout (shared by every entry point): row r of an M×K bit
 * matrix occupies Kw = ceil(K/32) consecutive uint32 words; word w holds
 * columns 32w..32w+31.  With BSP_LSB_FIRST column 32w+i is bit i (the layout
 * of the benchmark configurations); with BSP_MSB_FIRST it is bit 31-i (the
 * layout of dense2bitmask, source/src/main.cu:611-621).  Bits past column
 * K-1 in the last word are zero.  Compute entry points read LSB-first words.
 */
#ifndef BSP_H_
#define BSP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* bsp_stream_t;

/* ---- status codes ------------------------------------------------------ */
enum bsp_status {
  BSP_OK = 0,
  BSP_ERR_INVALID_ARG = -1,   /* null pointer, negative/zero size, bad enum  */
  BSP_ERR_ALIGNMENT = -2,     /* pointer or leading dimension misaligned     */
  BSP_ERR_WORKSPACE = -3,     /* workspace missing or smaller than required  */
  BSP_ERR_UNSUPPORTED = -4,   /* valid but not implemented combination       */
  BSP_ERR_CUDA = -5,          /* a CUDA runtime call or launch failed        */
  BSP_ERR_DEVICE_TIMEOUT = -6,/* a bounded device-side wait gave up          */
  BSP_ERR_ALLOC = -7,         /* device/host allocation failed               */
  BSP_ERR_CAPACITY = -8,      /* input exceeds a documented size limit       */
  BSP_ERR_QUEUE = -9,         /* batched work-queue descriptor is corrupt    */
  BSP_ERR_INTERNAL = -10
};

/* ---- element types ----------------------------------------------------- */
enum bsp_dtype {
  BSP_F32 = 0,
  BSP_F16 = 1,
  BSP_BF16 = 2,
  BSP_I8 = 3,
  BSP_U8 = 4
};

enum bsp_bit_order { BSP_LSB_FIRST = 0, BSP_MSB_FIRST = 1 };

/* Human-readable name of a status code (static string). */
const char* bsp_status_string(int status);
/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int bsp_version(void);
/* The cudaError_t of the most recent BSP_ERR_CUDA on this host thread. */
int bsp_last_cuda_error(void);

/* ======================================================================== */
/* Packing / format conversion                                              */
/* ======================================================================== */

/* Dense M×K matrix (row stride ld elements) → packed row masks words[M][Kw].
 * A bit is set iff the element is nonzero (x != 0: -0.0 counts as zero, NaN
 * as nonzero).  Replaces dense2bitmask, source/src/main.cu:591-628 (MSB-first,
 * 32-column tiles, atomicOr per nonzero) — here one warp ballot per word.    */
int bsp_pack_rows(const void* dense, int dtype, int64_t M, int64_t K,
                  int64_t ld, uint32_t* words, int bit_order,
                  bsp_stream_t stream);

/* Dense M×K → column-packed masks words_t[K][ceil(M/32)] (the packed rows of
 * Aᵀ).  The transposed form of dense2bitmask (source/src/main.cu:591-628),
 * used by the backward pass.                                                */
int bsp_pack_cols(const void* dense, int dtype, int64_t M, int64_t K,
                  int64_t ld, uint32_t* words_t, int bit_order,
                  bsp_stream_t stream);

/* Packed rows of an M×K bit matrix (LSB-first) → packed rows of its K×M
 * transpose.  No reference counterpart; the bit-matrix form of the
 * row→column re-tiling done by csr2tiledcsr, source/src/main.cu:499-588.   */
int bsp_transpose_bits(const uint32_t* words, int64_t M, int64_t K,
                       uint32_t* words_t, bsp_stream_t stream);

/* Packed masks → dense 0/1 matrix of dtype (row stride ld).  The scatter of
 * group2dense, source/src/main.cu:829-850, for a full mask.                  */
int bsp_unpack_rows(const uint32_t* words, int64_t M, int64_t K, void* dense,
                    int dtype, int64_t ld, int bit_order, bsp_stream_t stream);

/* Bit-plane split of an 8-bit matrix: plane b (0 ≤ b < planes ≤ 8) gets bit
 * ((uint8)v >> b) & 1 of every element, packed: words[b][M][Kw].  Replaces
 * uint8_layout_trans / layout_trans, backup/layout_trans.cu:75-97, which
 * wrote one int per bit.                                                     */
int bsp_bitplanes(const uint8_t* values, int64_t M, int64_t K, int64_t ld,
                  int planes, uint32_t* words, int bit_order,
                  bsp_stream_t stream);

/* ======================================================================== */
/* Row grouping (reference-compatible first fit)                            */
/* ======================================================================== */

/* Grouping of packed rows, one tile per (block of tile_rows rows, 32-column
 * word).  Tiles are numbered t = rb*Kw + w (rb = row block, w = word), as
 * bid = blockIdx.y*gridDim.x + blockIdx.x in the reference.  Inside a tile the
 * rows are visited in ascending order; a zero word joins group 0 without
 * changing its mask; a nonzero word joins the first group g < max_groups whose
 * mask it does not intersect (the mask gains its bits); otherwise the row
 * spills.  Replaces generate_groups_large, source/src/main.cu:50-247, whose
 * shared-memory atomicCAS race is replaced by this deterministic order.
 *
 * Outputs (all device, any of the optional ones may be NULL):
 *   group_id   [M*Kw]  int32: group of row r in word w, -1 if spilled
 *                      (reference intent main.cu:124/:156; its overwrite of
 *                      the -1 at main.cu:184 is not reproduced).
 *   group_mask [T*max_groups] uint32: OR of the member words.
 *   group_row  [T*max_groups*32] int32 (optional): local row (0..tile_rows-1)
 *                      that owns bit position i of group g, -1 if none; bit
 *                      position i is column 32w+i (LSB-first) — the
 *                      group_ele_row_idx table of main.cu:115-121/:186-190.
 *   spill_cnt  [T]     int32 (optional): spilled rows per tile.
 *   spill_nnz  [T]     int32 (optional): set bits of spilled rows per tile.
 *   spill_rows [T*tile_rows] int32 (optional): ascending local indices of the
 *                      spilled rows, -1 padded (spilled_row_hash_table).
 *   grouped_nnz[1]     int64 (optional): Σ popcount(group_mask) (the nnz
 *                      counter of main.cu:199-204).
 * tile_rows ∈ [1, 4096], max_groups ∈ [1, 32].                              */
int bsp_group_rows(const uint32_t* words, int64_t M, int64_t Kw,
                   int tile_rows, int max_groups, int32_t* group_id,
                   uint32_t* group_mask, int32_t* group_row,
                   int32_t* spill_cnt, int32_t* spill_nnz,
                   int32_t* spill_rows, int64_t* grouped_nnz,
                   bsp_stream_t stream);

/* Scatter of grouped values back to a dense matrix: for tile t=(rb,w) and
 * row r of that tile with group g = group_id[r*Kw+w] ≥ 0, every set bit i of
 * the row's word copies group_values[(t*max_groups+g)*32+i] into
 * dense[r*ldd + 32w+i].  Replaces group2dense, source/src/main.cu:829-850
 * (which used MSB-first bits and fixed SIZE_N / TILE_HEIGHT).               */
int bsp_group_to_dense(const float* group_values, const int32_t* group_id,
                       const uint32_t* words, int64_t M, int64_t K,
                       int tile_rows, int max_groups, float* dense,
                       int64_t ldd, bsp_stream_t stream);

/* ======================================================================== */
/* SpMM plans (similarity row grouping for the SpMM schedule)               */
/* ======================================================================== */

typedef struct bsp_plan bsp_plan;

enum bsp_plan_mode {
  BSP_PLAN_AUTO = 0,     /* choose from the measured cluster structure      */
  BSP_PLAN_DIRECT = 1,   /* every row walks its own set bits                */
  BSP_PLAN_PROTO = 2     /* rows = cluster prototype sum ± delta bits       */
};

typedef struct bsp_plan_params {
  int mode;              /* enum bsp_plan_mode                              */
  int signature_hashes;  /* MinHash functions per row (1..8), 0 = default   */
  int min_cluster_rows;  /* smallest cluster that gets a prototype, 0 = dflt*/
  uint32_t seed;         /* MinHash permutation seed                        */
} bsp_plan_params;

typedef struct bsp_plan_info {
  int64_t M, K;
  int64_t nnz;           /* set bits of A                                   */
  int mode;              /* the mode actually used                          */
  int64_t n_proto;       /* prototypes (clusters with a prototype)          */
  int64_t proto_nnz;     /* set bits over all prototypes                    */
  int64_t delta_nnz;     /* ± delta entries over all prototype rows         */
  int64_t direct_rows;   /* rows without a prototype                        */
  int64_t direct_nnz;    /* set bits of those rows                          */
  int64_t occ_tiles;     /* (128-row, 32-column) bit tiles holding a set bit */
} bsp_plan_info;

/* Build a plan for A (packed LSB-first words[M][ceil(K/32)]).  Runs grouping
 * kernels on `stream` (and, for the tensor-core structures, on a library side
 * stream joined back into it), synchronising it to size the plan's device
 * buffers, which the plan owns, and before returning.  The plan is immutable and may be used from
 * any stream afterwards.  params may be NULL (defaults).  The similarity
 * grouping has no counterpart in the reference; its first-fit grouping of
 * disjoint rows is bsp_group_rows.                                           */
int bsp_plan_create(const uint32_t* words, int64_t M, int64_t K,
                    const bsp_plan_params* params, bsp_plan** plan,
                    bsp_stream_t stream);
int bsp_plan_destroy(bsp_plan* plan);
/* Same, without waiting for the device: the plan's device memory goes back
 * to the library's pool in stream order, after the work already queued on
 * `stream` (e.g. the SpMM that used the plan).  Work using the plan on other
 * streams must be ordered before that point by the caller (an event).  The
 * host object is released at once; the handle is invalid on return.  No
 * counterpart in the reference, whose device buffers are released with
 * cudaFree (e.g. source/src/main.cu:1665). */
int bsp_plan_destroy_async(bsp_plan* plan, bsp_stream_t stream);
int bsp_plan_get_info(const bsp_plan* plan, bsp_plan_info* info);

/* ======================================================================== */
/* SpMM                                                                     */
/* ======================================================================== */

/* Device workspace (bytes) that bsp_spmm needs for this plan and N. */
int bsp_spmm_workspace(const bsp_plan* plan, int64_t N, size_t* bytes);

/* Workspace (bytes, ≥ the above) with which the tensor-core path (16-bit
 * B) also (1) splits the reduction: when the output has fewer 256x256 tiles
 * than half the SMs, up to 8 slices of the occupied K tiles run on separate
 * CTAs and their FP32 partials (kept in the workspace) are added in a fixed
 * order; and (2) copies B into tile order first (ceil(K/32)·ceil(N/256)
 * blocks of 16 KB), so that each tile reaches shared memory as one bulk
 * copy.  A smaller workspace only turns these off (results are identical).
 * bsp_spmm_t uses its own workspace the same way when it is large enough. */
int bsp_spmm_workspace_preferred(const bsp_plan* plan, int64_t N, size_t* bytes);

/* C[M×N] (FP32, row stride ldc) = A·B, A given by its packed words and,
 * optionally, a plan built from the same words (NULL = walk every row's set
 * bits).  B is K×N of b_dtype ∈ {F32, F16, BF16}, row stride ldb elements;
 * accumulation is FP32, rows with more than 4096 set bits use a compensated
 * (two-term) sum.  Replaces the 0/1-mask SpMM of uint8_spmm_2d_1d /
 * indexed_spmm_*, backup/layout_trans.cu:120-171 (one global atomicAdd per
 * set bit and column) and the bit-serial compute kernel
 * spgemm_compute_1dthread_tcore_v3, source/src/transform.cuh:2062-2248.
 * Integer-valued B gives results identical to the reference's sum.        */
int bsp_spmm(const uint32_t* A_words, int64_t M, int64_t K, const void* B,
             int b_dtype, int64_t ldb, int64_t N, float* C, int64_t ldc,
             const bsp_plan* plan, void* workspace, size_t workspace_bytes,
             bsp_stream_t stream);

/* ======================================================================== */
/* Batched SpMM                                                             */
/* ======================================================================== */

/* One problem of a batch: C[M×N] = A·B with A packed (LSB-first) words
 * [M][ceil(K/32)] and B K×N (row stride ldb elements, 16-byte aligned,
 * ldb*2 a multiple of 16), C FP32 (16-byte aligned, ldc a multiple of 4).  */
typedef struct bsp_problem {
  const uint32_t* A_words;
  int64_t M, K;
  const void* B;
  int64_t ldb;
  float* C;
  int64_t ldc;
} bsp_problem;

typedef struct bsp_batch bsp_batch;

/* Prepare a batch of n independent problems sharing N (multiple of 8) and a
 * 16-bit B type: encodes every problem's B tensor map and uploads them with
 * a work list of (problem, 256-row block, 256-column block) items sorted
 * longest reduction first; synchronises the stream once.  The problems'
 * buffers are referenced, not copied — they must outlive the batch.  Limit:
 * K ≤ 131072 per problem (BSP_ERR_CAPACITY).  No reference counterpart (the
 * reference runs one fixed-size problem per launch).                       */
int bsp_batch_create(const bsp_problem* problems, int n, int64_t N,
                     int b_dtype, bsp_batch** batch, bsp_stream_t stream);
int bsp_batch_destroy(bsp_batch* batch);
/* Every problem of the batch in one tensor-core launch, with no host
 * synchronisation and no allocation; it can be captured in a CUDA graph.
 * For N ≤ 128 the launch is persistent: a CTA per SM takes items from a
 * work queue in the batch's device memory, which a memset in the same stream
 * resets first.  For wider N it is one CTA per work item.  Runs of one batch
 * must not overlap on the GPU: they share the queue and the C buffers.     */
int bsp_batched_spmm(const bsp_batch* batch, bsp_stream_t stream);
/* Times the persistent kernel's shapes (pipeline stages, epilogue warps, A
 * words loaded ahead) on this batch — each once to warm up, then three runs
 * — keeps the fastest in the batch for later bsp_batched_spmm calls and
 * returns its index and ms per run.  It runs the batch (writes its C
 * buffers) four times per shape and synchronises the stream.  Batches of
 * N > 128 have
 * one shape (index 0); a gradient batch is refused (BSP_ERR_INVALID_ARG).
 * On an error the batch keeps its previous shape.                         */
int bsp_batch_tune(bsp_batch* batch, bsp_stream_t stream, int* shape, float* ms);

/* One problem of a batched backward pass of Y = A·X (A a 0/1 mask, packed
 * LSB-first words [M][ceil(K/32)]; X [K×N] and the incoming gradient
 * G = dL/dY [M×N] 16-bit, row strides ldx, ldg elements, 16-byte aligned):
 *   dX = Aᵀ·G            [K×N] FP32, row stride lddx (NULL: not computed)
 *   dA = (G·Xᵀ) ⊙ A      [M×K] FP32, row stride ldda, zero off A's bits
 *                         (the straight-through mask gradient; NULL: skip)
 * dX and dA 16-byte aligned with strides a multiple of 4; dA needs
 * K % 8 == 0.  Limit: M ≤ 131072 for dX (BSP_ERR_CAPACITY).               */
typedef struct bsp_problem_grad {
  const uint32_t* A_words;
  int64_t M, K;
  const void* X;
  int64_t ldx;
  const void* G;
  int64_t ldg;
  float* dX;
  int64_t lddx;
  float* dA;
  int64_t ldda;
} bsp_problem_grad;

/* Prepare a gradient batch: n problems sharing N (multiple of 8) and the
 * 16-bit type of X and G.  Encodes the G and X tensor maps, uploads them
 * with the work lists — (problem, 256-row block of dX, 256-column block)
 * and (problem, 128-row block of dA, 256-column block of dA) — sorted
 * longest reduction first; synchronises the stream once.  Buffers are
 * referenced and must outlive the batch; bsp_batch_destroy releases it.
 * No reference counterpart (the reference has no backward pass); the
 * single-problem forms are bsp_spmm_t and bsp_sddmm.                      */
int bsp_batch_grad_create(const bsp_problem_grad* problems, int n, int64_t N,
                          int dtype, bsp_batch** batch, bsp_stream_t stream);
/* Every dX and dA of a gradient batch: two tensor-core launches, no host
 * synchronisation, no allocation.  dX (for N ≤ 128 one persistent launch,
 * else a CTA per work item) sums every 32-row tile of A (a batch has no
 * occupancy plan); dA is one persistent
 * launch (a CTA per SM taking items from a work queue in the batch's
 * device memory, reset by a memset in the same stream) that writes zeros
 * off A's set bits.  Runs of one batch must not overlap on the GPU: they
 * share the queue and write the same dX and dA buffers.                    */
int bsp_batched_spmm_grad(const bsp_batch* batch, bsp_stream_t stream);

/* ======================================================================== */
/* Autotuner                                                                */
/* ======================================================================== */

/* A measured SpMM schedule: engine 1 = tensor cores, 2 = CUDA cores (per
 * shape bucket, this is the tensor-core density threshold); on the tensor
 * cores the tile form (K tiles per stage, B pre-tiled or by TMA boxes,
 * split-K or not); on the CUDA cores with a prototype plan, proto_path 0 =
 * register gathers / 1 = TMA-staged slices and proto_variant = that
 * kernel's shape (columns per warp, gathers in flight, CTAs per SM); ms =
 * its time.                                                                 */
typedef struct bsp_schedule {
  int engine;
  int proto_path;
  int proto_variant;
  float ms;
  int tc_stage_tiles;  /* tensor cores: K tiles per stage (2 or 3; 0 = rule) */
  int tc_tiled_b;      /* tensor cores: B copied into tile order (1), TMA boxes (0), rule (-1) */
  int tc_split;        /* tensor cores: split-K by the rule (-1) or never (0) */
} bsp_schedule;

/* Times every candidate schedule of bsp_spmm for this plan and these
 * operands (the tensor cores in 8 tile forms when allowed; each
 * prototype-kernel shape on both paths; 2 warm-up + 5 timed runs each, CUDA
 * events on `stream`, which it synchronises), leaves C holding the fastest one's result, returns it in
 * *best and caches it for the shape bucket (log2 of M, K, N; density in half
 * octaves; dtype; plan mode).  bsp_spmm uses a cached schedule for its
 * bucket unless BSP_TC, BSP_PROTO_PATH or BSP_PROTO_VARIANT force a choice.
 * With BSP_TUNE_CACHE=<file> the cache is read from that JSON file at first
 * use and rewritten (temporary file, then rename) after each new entry; a
 * file that does not parse is ignored.  The reference fixed its tile shapes
 * at compile time (source/src/common.h:15-35); no counterpart.            */
int bsp_tune(const uint32_t* A_words, int64_t M, int64_t K, const void* B,
             int b_dtype, int64_t ldb, int64_t N, float* C, int64_t ldc,
             const bsp_plan* plan, void* workspace, size_t workspace_bytes,
             bsp_stream_t stream, bsp_schedule* best);
/* Replace the in-process cache by a file's entries (BSP_ERR_INVALID_ARG and
 * no change if it does not parse), write it atomically, clear it, count it. */
int bsp_tune_cache_load(const char* path, int* entries);
int bsp_tune_cache_save(const char* path);
int bsp_tune_cache_clear(void);
int bsp_tune_cache_size(int* entries);

/* ======================================================================== */
/* Backward pass                                                            */
/* ======================================================================== */

/* dX[K×N] (FP32, row stride lddx) = Aᵀ·G for G[M×N] of g_dtype (row stride
 * ldg).  With a plan and 16-bit G the tensor cores read Aᵀ's bit tiles
 * straight from A's row words (no transposed copy is made); otherwise the
 * bits are transposed into the workspace (bsp_spmm_t_workspace bytes) and
 * walked like bsp_spmm.  The backward of the forward SpMM; no reference
 * counterpart (the reference has no backward).                            */
int bsp_spmm_t_workspace(int64_t M, int64_t K, size_t* bytes);
/* ... and with room for the tensor-core reduction split (as for bsp_spmm). */
int bsp_spmm_t_workspace_preferred(int64_t M, int64_t K, int64_t N, size_t* bytes);
int bsp_spmm_t(const uint32_t* A_words, int64_t M, int64_t K, const void* G,
               int g_dtype, int64_t ldg, int64_t N, float* dX, int64_t lddx,
               const bsp_plan* plan, void* workspace, size_t workspace_bytes,
               bsp_stream_t stream);

/* Straight-through mask gradient: dA[M×K] (FP32, row stride ldda) =
 * Σ_j G[i][j]·X[k][j] where A has bit (i,k) set, 0 elsewhere — the SDDMM of
 * G[M×N] and X[K×N] (same dtype).  16-bit operands run on the tensor cores
 * (dense product over N, masked store; blocks of A without bits skipped);
 * FP32 or unaligned operands use one warp dot product per set bit.  The
 * plan (optional) feeds the choice between the two.  No reference
 * counterpart.                                                            */
int bsp_sddmm(const uint32_t* A_words, int64_t M, int64_t K, const void* G,
              int64_t ldg, const void* X, int64_t ldx, int dtype, int64_t N,
              float* dA, int64_t ldda, const bsp_plan* plan,
              bsp_stream_t stream);

/* ======================================================================== */
/* Output side and multi-bit operands                                       */
/* ======================================================================== */

/* Symbolic product of two bit matrices: C_words[M][ceil(N/32)] gets, for
 * row i, the OR of B_words' row masks k over the set bits k of A's row i —
 * the bit pattern of A·B's nonzeros when B (K×N) is itself a bitmap.  The
 * symbolic half of pre_spgemm, source/src/transform.cuh:1028-1057; its
 * first-fit grouping of the output rows (:1058-1157) is bsp_group_rows on
 * C_words.  Both inputs and the output are LSB-first packed rows.          */
int bsp_symbolic_rows(const uint32_t* A_words, int64_t M, int64_t K,
                      const uint32_t* B_words, int64_t N, uint32_t* C_words,
                      bsp_stream_t stream);

/* The same mask through a prototype plan of A (bsp_plan_create).  A row of
 * cluster c counts, per output column, the set bits of its columns' B masks
 * as its cluster's counts (bit-sliced, from the consensus columns) plus its
 * added columns minus its removed ones, and keeps the columns with a
 * nonzero count; rows without a cluster OR their masks.  The result is
 * identical to bsp_symbolic_rows.  Workspace: bsp_symbolic_workspace bytes
 * (the clusters' count planes).  A plan that is not a prototype plan, or
 * K ≥ 65536, runs bsp_symbolic_rows.  Same reference step as
 * bsp_symbolic_rows (transform.cuh:1028-1057); the plan has no counterpart
 * there. */
int bsp_symbolic_workspace(const bsp_plan* plan, int64_t N, size_t* bytes);
int bsp_symbolic_rows_planned(const uint32_t* A_words, int64_t M, int64_t K,
                              const uint32_t* B_words, int64_t N,
                              uint32_t* C_words, const bsp_plan* plan,
                              void* workspace, size_t workspace_bytes,
                              bsp_stream_t stream);

/* Bit-plane product: C[M×N] (FP32, row stride ldc) = Σ_b w_b·(P_b·B) for the
 * planes P_b (0 ≤ b < n_planes ≤ 8) of an M×K 8-bit matrix, packed as
 * bsp_bitplanes writes them (planes[b][M][ceil(K/32)], LSB-first), with
 * w_b = 2^b, except w = −2^(n_planes−1) for the top plane when
 * is_signed != 0 (two's complement).  B is K×N of b_dtype ∈ {F32, F16,
 * BF16}; every plane is summed in FP32 with a compensated (two-term) sum,
 * then scaled by its exact power-of-two weight.  Replaces the bit-serial
 * int8 product of spgemm_compute_1dthread_tcore_v3,
 * source/src/transform.cuh:2199-2246, with the plane weights
 * (1, 2, ..., 64, -128) of initialize_multiplicand, main.cu:895-910.      */
int bsp_bitplane_spmm(const uint32_t* planes, int n_planes, int is_signed,
                      int64_t M, int64_t K, const void* B, int b_dtype,
                      int64_t ldb, int64_t N, float* C, int64_t ldc,
                      bsp_stream_t stream);

/* C = A·B for a dense int8 A (M×K, row stride lda): splits A into its 8
 * bit planes in the workspace (bsp_spmm_i8_workspace bytes) and runs
 * bsp_bitplane_spmm with the signed weights.  The whole path of the
 * reference's multi-bit operand (layout_trans, backup/layout_trans.cu:75-97,
 * then the bit-serial product above).                                     */
/* The same product as one bitmap SpMM with the planes laid along K, for a
 * weight matrix A that is reused (plan it once with bsp_plan_create):
 *   C = [P_0 | P_1 | ... | P_{n-1}] · [w_0·B; w_1·B; ...; w_{n-1}·B]
 * bsp_bitplanes_rows writes A's planes side by side per row,
 * words[M][n_planes*ceil(K/32)] (a bitmap with K' = n_planes*32*ceil(K/32)
 * columns), and bsp_stack_planes_b writes the K'×N matrix of w_b·B blocks
 * (rows K..32*ceil(K/32)-1 of every block are 0; scaling by a power of two
 * is exact in every supported dtype).  bsp_spmm on the two, with a plan of
 * the plane words, then runs on the tensor cores for 16-bit B when its cost
 * model says so.                                                           */
int bsp_bitplanes_rows(const uint8_t* values, int64_t M, int64_t K, int64_t ld,
                       int n_planes, uint32_t* words, bsp_stream_t stream);
int bsp_stack_planes_b(const void* B, int b_dtype, int64_t ldb, int64_t K,
                       int64_t N, int n_planes, int is_signed, void* B_out,
                       int64_t ld_out, bsp_stream_t stream);

int bsp_spmm_i8_workspace(int64_t M, int64_t K, size_t* bytes);
int bsp_spmm_i8(const int8_t* A, int64_t M, int64_t K, int64_t lda,
                const void* B, int b_dtype, int64_t ldb, int64_t N, float* C,
                int64_t ldc, void* workspace, size_t workspace_bytes,
                bsp_stream_t stream);

/* ======================================================================== */
/* Interchange formats                                                      */
/* ======================================================================== */

/* Packed rows -> 8x8 bitmap tiles (the tSparse format of coo2bmp_noTuple_d,
 * source/src/main.cu:692-779, and find_tile_index, source/src/mm.h:83-104):
 * the nonzero tiles in ascending tile_row*ceil(K/8)+tile_col order, each a
 * uint64 with bit (r%8)*8 + c%8 for element (8*tile_row+r, 8*tile_col+c);
 * offset[t] = Σ popcount of the tiles before t (offset[n] = nnz, where the
 * values of tile t start in the reference's elems array).  Output arrays
 * hold T = ceil(M/8)*ceil(K/8) entries (offset T+1); the first *n_tiles
 * (device int64) are valid and offset[t] = nnz for t ≥ n.  Workspace:
 * bsp_tiles8_workspace bytes.  Limit: M·K < 2^31.                         */
int bsp_tiles8_workspace(int64_t M, int64_t K, size_t* bytes);
int bsp_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K,
                       uint64_t* bmp, int32_t* tile_row, int32_t* tile_col,
                       int32_t* offset, int64_t* n_tiles, void* workspace,
                       size_t workspace_bytes, bsp_stream_t stream);

/* 8x8 bitmap tiles (n_tiles of them, any order, host count) -> packed rows
 * (every word of words[M][ceil(K/32)] is written).  Tiles outside the
 * matrix and bits past column K-1 are ignored.                             */
int bsp_tiles8_to_rows(const uint64_t* bmp, const int32_t* tile_row,
                       const int32_t* tile_col, int64_t n_tiles, int64_t M,
                       int64_t K, uint32_t* words, bsp_stream_t stream);

/* CSR (row_ptr[M+1], col_idx[nnz], optional values of value_bytes bytes
 * each) -> tiled CSR of csr2tiledcsr, source/src/main.cu:499-588, with the
 * tile shape tile_rows x tile_cols as parameters (TILE_HEIGHT x SPLIT_K
 * there).  Tile t = ty*ceil(K/tile_cols)+tx holds its entries contiguously
 * from tile_nnz_acc[t] (T+1 values, exclusive scan of the tiles' counts),
 * rows in order and each row's entries in CSR order; tiled_col is the local
 * column (col % tile_cols); tiled_offset[(tile_rows+1)*t + j] counts the
 * tile's entries in its local rows before j.  Values are copied unchanged
 * (the reference also cast them to its value type; cast before or after).
 * Entries whose column is outside [0, K) are dropped.  Workspace:
 * bsp_csr_to_tiled_workspace bytes.  Limits: nnz < 2^31, value_bytes ≤ 8. */
int bsp_csr_to_tiled_workspace(int64_t M, int64_t K, int64_t nnz,
                               int tile_rows, int tile_cols, size_t* bytes);
int bsp_csr_to_tiled(const int32_t* row_ptr, const int32_t* col_idx,
                     const void* values, int value_bytes, int64_t M,
                     int64_t K, int64_t nnz, int tile_rows, int tile_cols,
                     int32_t* tile_nnz_acc, int32_t* tiled_offset,
                     int32_t* tiled_col, void* tiled_values, void* workspace,
                     size_t workspace_bytes, bsp_stream_t stream);

/* bsp_spmm without a workspace argument, for callers that may not allocate
 * device memory when they run the SpMM (plugin callbacks handed only
 * pointers, hot loops that must not call the allocator, processes whose
 * device memory belongs to another allocator).  It runs bsp_spmm with, as
 * workspace, a static device array of 8 MiB inside the library, held on
 * every GPU that loads the library until the process exits: the array holds
 * the prototype sums and, for 16-bit B on the tensor cores, the split-K
 * partials and the tiled copy of B whenever they fit in it (the same route
 * bsp_spmm takes with an 8 MiB workspace, whatever the plan).
 * Limit: bsp_spmm_workspace(plan, N) must be ≤ 8 MiB (≈ n_proto * N * 4
 * bytes), else BSP_ERR_CAPACITY.  The first call on a device looks the
 * array's address up (cudaGetSymbolAddress) and keeps it: make that first
 * call before any stream capture, and do not use the library across a
 * cudaDeviceReset (the kept address would be stale).  All calls share the
 * one array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  The array keeps the
 * last call's contents; nothing in it needs to start at zero.  No
 * counterpart in the reference.                                            */
int bsp_spmm_noalloc(const uint32_t* A_words, int64_t M, int64_t K,
                     const void* B, int b_dtype, int64_t ldb, int64_t N,
                     float* C, int64_t ldc, const bsp_plan* plan,
                     bsp_stream_t stream);

/* Measurement helper (no reference counterpart): the L2 row-gather roof of
 * the clustered-row SpMM.  n_warps warps (a multiple of 8) each read
 * per_warp row indices from row_idx ([n_warps][per_warp], values < rows;
 * larger ones are skipped) and gather one slice of slice_bytes (512, 1024
 * or 2048) bytes from the start of each row of buf ([rows][row_bytes],
 * 16-byte aligned), one slice in flight per warp.  sink receives nothing
 * unless the sum of the gathered values is impossible ([n_warps] floats).
 * Time it with events: bytes = n_warps * per_warp * slice_bytes.          */
int bsp_probe_gather(const void* buf, int64_t rows, int64_t row_bytes,
                     const uint32_t* row_idx, int64_t n_warps, int64_t per_warp,
                     int slice_bytes, float* sink, bsp_stream_t stream);

/* Device-side status of the asynchronous kernels (0 = none; 1 = a bounded
 * mbarrier wait of the TMA-staged SpMM expired and its output is invalid).
 * Synchronises the device; clear != 0 resets the word.  No reference
 * counterpart (the reference has no device-side error reporting).         */
int bsp_device_status(int* status, int clear);

#ifdef __cplusplus
}
#endif
#endif /* BSP_H_ */
