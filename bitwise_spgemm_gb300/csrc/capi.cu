// capi.cu — the extern "C" entry points of include/bsp.h: argument
// validation, layout checks and dispatch to the kernels.  Every entry point
// returns a bsp_status and never aborts (the reference's CHECK_* macros
// printed and returned EXIT_FAILURE, source/src/common.h:37-55).
#include <climits>
#include <cstdlib>
#include <new>

#include "bsp_internal.cuh"
#include "plan.cuh"
#include "tune.h"
#include "spmm.cuh"

namespace bsp {

static thread_local int g_last_cuda_error = 0;

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return BSP_OK;
  g_last_cuda_error = (int)e;
  return BSP_ERR_CUDA;
}

int num_sms() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    cache[dev] = n;
  }
  return cache[dev];
}

}  // namespace bsp

using namespace bsp;

namespace {

constexpr int64_t kMaxCols = (int64_t)INT_MAX - 64;  // column indices are int32 on the device

bool valid_dtype(int dt) { return dt >= BSP_F32 && dt <= BSP_U8; }
bool valid_order(int o) { return o == BSP_LSB_FIRST || o == BSP_MSB_FIRST; }

int check_dims(int64_t M, int64_t K) {
  if (M < 0 || K < 0) return BSP_ERR_INVALID_ARG;
  if (K > kMaxCols || M > kMaxCols) return BSP_ERR_CAPACITY;
  return BSP_OK;
}

int current_device() {
  int d = -1;
  cudaGetDevice(&d);
  return d;
}

}  // namespace

extern "C" {

const char* bsp_status_string(int status) {
  switch (status) {
    case BSP_OK: return "BSP_OK";
    case BSP_ERR_INVALID_ARG: return "BSP_ERR_INVALID_ARG: invalid argument";
    case BSP_ERR_ALIGNMENT: return "BSP_ERR_ALIGNMENT: misaligned pointer or leading dimension";
    case BSP_ERR_WORKSPACE: return "BSP_ERR_WORKSPACE: workspace missing or too small";
    case BSP_ERR_UNSUPPORTED: return "BSP_ERR_UNSUPPORTED: unsupported combination";
    case BSP_ERR_CUDA: return "BSP_ERR_CUDA: CUDA runtime error";
    case BSP_ERR_DEVICE_TIMEOUT: return "BSP_ERR_DEVICE_TIMEOUT: bounded device wait expired";
    case BSP_ERR_ALLOC: return "BSP_ERR_ALLOC: allocation failed";
    case BSP_ERR_CAPACITY: return "BSP_ERR_CAPACITY: size limit exceeded";
    case BSP_ERR_QUEUE: return "BSP_ERR_QUEUE: corrupt work-queue descriptor";
    case BSP_ERR_INTERNAL: return "BSP_ERR_INTERNAL: internal error";
    default: return "unknown bsp status";
  }
}

int bsp_version(void) { return 100; }

int bsp_last_cuda_error(void) { return g_last_cuda_error; }

int bsp_pack_rows(const void* dense, int dtype, int64_t M, int64_t K, int64_t ld, uint32_t* words,
                  int bit_order, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (!valid_dtype(dtype) || !valid_order(bit_order) || ld < K) return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!dense || !words) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(dense, dtype_size(dtype)) || !is_aligned(words, 4)) return BSP_ERR_ALIGNMENT;
  return launch_pack_rows(dense, dtype, M, K, ld, words, bit_order, (cudaStream_t)stream);
}

int bsp_pack_cols(const void* dense, int dtype, int64_t M, int64_t K, int64_t ld, uint32_t* words_t,
                  int bit_order, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (!valid_dtype(dtype) || !valid_order(bit_order) || ld < K) return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!dense || !words_t) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(dense, dtype_size(dtype)) || !is_aligned(words_t, 4)) return BSP_ERR_ALIGNMENT;
  return launch_pack_cols(dense, dtype, M, K, ld, words_t, bit_order, (cudaStream_t)stream);
}

int bsp_transpose_bits(const uint32_t* words, int64_t M, int64_t K, uint32_t* words_t,
                       bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (M == 0 || K == 0) return BSP_OK;
  if (!words || !words_t) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(words, 4) || !is_aligned(words_t, 4)) return BSP_ERR_ALIGNMENT;
  return launch_transpose_bits(words, M, K, words_t, (cudaStream_t)stream);
}

int bsp_unpack_rows(const uint32_t* words, int64_t M, int64_t K, void* dense, int dtype, int64_t ld,
                    int bit_order, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (!valid_dtype(dtype) || !valid_order(bit_order) || ld < K) return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!dense || !words) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(dense, dtype_size(dtype)) || !is_aligned(words, 4)) return BSP_ERR_ALIGNMENT;
  return launch_unpack_rows(words, M, K, dense, dtype, ld, bit_order, (cudaStream_t)stream);
}

int bsp_bitplanes(const uint8_t* values, int64_t M, int64_t K, int64_t ld, int planes,
                  uint32_t* words, int bit_order, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (planes < 1 || planes > 8 || !valid_order(bit_order) || ld < K) return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!values || !words) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(words, 4)) return BSP_ERR_ALIGNMENT;
  return launch_bitplanes(values, M, K, ld, planes, words, bit_order, (cudaStream_t)stream);
}

int bsp_group_rows(const uint32_t* words, int64_t M, int64_t Kw, int tile_rows, int max_groups,
                   int32_t* group_id, uint32_t* group_mask, int32_t* group_row, int32_t* spill_cnt,
                   int32_t* spill_nnz, int32_t* spill_rows, int64_t* grouped_nnz,
                   bsp_stream_t stream) {
  if (M < 0 || Kw < 0) return BSP_ERR_INVALID_ARG;
  if (tile_rows < 1 || tile_rows > 4096 || max_groups < 1 || max_groups > 32) return BSP_ERR_INVALID_ARG;
  if (Kw > kMaxCols / 32 || M > kMaxCols) return BSP_ERR_CAPACITY;
  if (M > 0 && Kw > 0 && (!words || !group_id || !group_mask)) return BSP_ERR_INVALID_ARG;
  if (grouped_nnz && !is_aligned(grouped_nnz, 8)) return BSP_ERR_ALIGNMENT;
  return launch_group_rows(words, M, Kw, tile_rows, max_groups, group_id, group_mask, group_row,
                           spill_cnt, spill_nnz, spill_rows, grouped_nnz, (cudaStream_t)stream);
}

int bsp_group_to_dense(const float* group_values, const int32_t* group_id, const uint32_t* words,
                       int64_t M, int64_t K, int tile_rows, int max_groups, float* dense,
                       int64_t ldd, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (tile_rows < 1 || tile_rows > 4096 || max_groups < 1 || max_groups > 32 || ldd < K)
    return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!group_values || !group_id || !words || !dense) return BSP_ERR_INVALID_ARG;
  return launch_group_to_dense(group_values, group_id, words, M, K, tile_rows, max_groups, dense,
                               ldd, (cudaStream_t)stream);
}

int bsp_plan_create(const uint32_t* words, int64_t M, int64_t K, const bsp_plan_params* params,
                    bsp_plan** plan, bsp_stream_t stream) {
  if (!plan) return BSP_ERR_INVALID_ARG;
  *plan = nullptr;
  BSP_TRY(check_dims(M, K));
  if (M > 0 && K > 0 && !words) return BSP_ERR_INVALID_ARG;
  bsp_plan_params prm = {BSP_PLAN_AUTO, 8, 4, 0x5eed1234u};
  if (params) {
    if (params->mode < BSP_PLAN_AUTO || params->mode > BSP_PLAN_PROTO) return BSP_ERR_INVALID_ARG;
    if (params->signature_hashes < 0 || params->signature_hashes > 8) return BSP_ERR_INVALID_ARG;
    if (params->min_cluster_rows < 0) return BSP_ERR_INVALID_ARG;
    prm.mode = params->mode;
    if (params->signature_hashes) prm.signature_hashes = params->signature_hashes;
    if (params->min_cluster_rows) prm.min_cluster_rows = params->min_cluster_rows;
    prm.seed = params->seed ? params->seed : prm.seed;
  }
  if (prm.min_cluster_rows < 2) prm.min_cluster_rows = 2;
  bsp_plan* p = new (std::nothrow) bsp_plan();
  if (!p) return BSP_ERR_ALLOC;
  p->device = current_device();
  int st = BSP_OK;
  if (M > 0 && K > 0) {
    st = plan_build(words, M, K, &prm, p, (cudaStream_t)stream);
  } else {
    p->M = M;
    p->K = K;
    p->Kw = ceil_div(K, 32);
  }
  if (st != BSP_OK) {
    plan_free(p);
    delete p;
    return st;
  }
  *plan = p;
  return BSP_OK;
}

int bsp_plan_destroy(bsp_plan* plan) {
  if (!plan) return BSP_OK;
  plan_free(plan);
  delete plan;
  return BSP_OK;
}

int bsp_plan_destroy_async(bsp_plan* plan, bsp_stream_t stream) {
  if (!plan) return BSP_OK;
  const int st = plan_free_async(plan, (cudaStream_t)stream);
  delete plan;
  return st;
}

int bsp_plan_get_info(const bsp_plan* plan, bsp_plan_info* info) {
  if (!plan || !info) return BSP_ERR_INVALID_ARG;
  info->M = plan->M;
  info->K = plan->K;
  info->nnz = plan->nnz;
  info->mode = plan->mode;
  info->n_proto = plan->mode == BSP_PLAN_PROTO ? plan->n_proto : 0;
  info->proto_nnz = plan->mode == BSP_PLAN_PROTO ? plan->proto_nnz : 0;
  info->delta_nnz = plan->mode == BSP_PLAN_PROTO ? plan->delta_nnz : 0;
  info->direct_rows = plan->mode == BSP_PLAN_PROTO ? plan->direct_rows : plan->M;
  info->direct_nnz = plan->mode == BSP_PLAN_PROTO ? plan->direct_nnz : plan->nnz;
  info->occ_tiles = plan->occ_tiles;
  return BSP_OK;
}

static int64_t proto_ldp(int64_t N) { return (N + 7) / 8 * 8; }

// Cost model of the tensor-core decision, in seconds: dense BF16 work on the
// occupied (128 x 32) tiles at ~1.2 PFLOP/s against the B-row gathers of the
// CUDA-core schedule at ~8 TB/s (rates measured on GB300).
static bool use_tensor_cores(const bsp_plan* plan, int64_t N, int esize) {
  if (plan->K > tc_max_reduction()) return false;
  const char* e = getenv("BSP_TC");
  if (e) return e[0] == '1';
  const double tc = (double)plan->occ_tiles * 128.0 * 32.0 * (double)N * 2.0 / 1.2e15;
  double gathers = (double)plan->nnz;
  if (plan->mode == BSP_PLAN_PROTO)
    gathers = (double)(plan->proto_nnz + plan->delta_nnz + plan->direct_nnz + plan->M);
  const double cc = gathers * (double)N * (double)esize / 8e12;
  return tc < cc;
}

// Kernel shape of the prototype path: BSP_PROTO_PATH = "bulk" (TMA-staged
// slices) or "regs" (register gathers), BSP_PROTO_VARIANT its shape index.
// Defaults come from measurement on GB300; the variables exist for tuning.
static int env_int(const char* name, int dflt) {
  const char* e = getenv(name);
  return e ? atoi(e) : dflt;
}
static int proto_path() {  // 0 = register gathers (default), 1 = TMA-staged slices
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("BSP_PROTO_PATH");
    v = (e && e[0] == 'b') ? 1 : 0;
  }
  return v;
}
// Register gathers: 512 columns per warp and two gathers in flight (variant
// 0) for every B type — at 8192x8192x512 FP32 22.55 us a step against 22.9
// for a 1 KB half row with one in flight (variant 4), BF16 16.9 against 25.1.
static int proto_variant(int esz) {
  static int v = -1000;
  if (v == -1000) v = env_int("BSP_PROTO_VARIANT", -1);
  (void)esz;
  if (v >= 0) return v;
  return proto_path() == 1 ? 3 : 0;
}

// Default schedule: the cost model for the engine (BSP_TC=0/1 forces it),
// the measured default shape of the prototype kernels (BSP_PROTO_PATH /
// BSP_PROTO_VARIANT override them).
static TuneSched default_schedule(const bsp_plan* plan, int64_t N, int esz, bool tc_ok) {
  TuneSched t;
  t.engine = (tc_ok && use_tensor_cores(plan, N, esz)) ? 1 : 2;
  t.proto_path = proto_path();
  t.proto_variant = proto_variant(esz);
  return t;
}

// Runs the SpMM with a given schedule (arguments already validated).
static int run_spmm(SpmmArgs a, const bsp_plan* plan, bool vec, const TuneSched& sc, void* workspace,
                    size_t workspace_bytes, cudaStream_t s) {
  // Tensor cores for 16-bit B when the occupied bit tiles make a dense
  // contraction cheaper than gathering B rows.
  if (sc.engine == 1)
    return launch_spmm_tc(a, plan->occ, plan->wordsT, s, workspace, workspace_bytes,
                          TcForm{sc.tc_tps, sc.tc_tiled, sc.tc_split});
  const int64_t N = a.N, K = a.K;
  const bool proto = plan && plan->mode == BSP_PLAN_PROTO && vec;
  if (proto) {
    size_t need = 0;
    bsp_spmm_workspace(plan, N, &need);
    if (!workspace || workspace_bytes < need) return BSP_ERR_WORKSPACE;
    a.row_cluster = plan->row_cluster;
    a.delta_ptr = plan->delta_ptr;
    a.delta_idx = plan->delta_idx;
    a.cons = plan->cons;
    a.n_proto = plan->n_proto;
    a.proto_max_nnz = plan->proto_max_nnz;
    a.cons_ptr = plan->cons_ptr;
    a.delta_pad = plan->delta_pad;
    a.n_slot = plan->n_slot;
    a.cons_idx = plan->cons_idx;
    a.P = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    a.ldp = proto_ldp(N);
    a.n_delta = plan->delta_nnz;
    if (K < (int64_t)1 << 30) {
      // prototype sums, then clustered rows (register gathers, or slices
      // staged by TMA bulk copies); rows without a cluster: walk A
      BSP_TRY(launch_proto_sums(a, s));
      if (sc.proto_path == 1) BSP_TRY(launch_spmm_proto_bulk(a, sc.proto_variant, s));
      else BSP_TRY(launch_spmm_proto_regs(a, sc.proto_variant, s));
      if (plan->direct_rows > 0) {
        SpmmArgs d = a;
        d.row_list = plan->direct_list;
        d.n_list = plan->direct_rows;
        BSP_TRY(launch_spmm_rows(d, false, vec, s));
      }
      return BSP_OK;
    }
    BSP_TRY(launch_proto_sums(a, s));
  }
  return launch_spmm_rows(a, proto, vec, s);
}

int bsp_spmm_workspace(const bsp_plan* plan, int64_t N, size_t* bytes) {
  if (!bytes || N < 0) return BSP_ERR_INVALID_ARG;
  *bytes = 0;
  if (plan && plan->mode == BSP_PLAN_PROTO) {
    *bytes = sizeof(float) * (size_t)plan->n_proto * (size_t)proto_ldp(N) + 256;
  }
  return BSP_OK;
}

int bsp_spmm_workspace_preferred(const bsp_plan* plan, int64_t N, size_t* bytes) {
  BSP_TRY(bsp_spmm_workspace(plan, N, bytes));
  if (plan) {
    const size_t tc = tc_preferred_bytes(plan->M, N, plan->K);
    if (tc > *bytes) *bytes = tc;
  }
  return BSP_OK;
}

// Validation and arguments shared by bsp_spmm and bsp_tune; kDone when the
// product is empty (C already written or nothing to write).
constexpr int kDone = 1;
static int prepare_spmm(const uint32_t* A_words, int64_t M, int64_t K, const void* B, int b_dtype, int64_t ldb,
                        int64_t N, float* C, int64_t ldc, const bsp_plan* plan, cudaStream_t s, SpmmArgs* a,
                        bool* vec, bool* tc_ok, int* esz_out) {
  BSP_TRY(check_dims(M, K));
  if (N < 0 || N > kMaxCols) return BSP_ERR_INVALID_ARG;
  if (b_dtype != BSP_F32 && b_dtype != BSP_BF16 && b_dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (ldb < N || ldc < N) return BSP_ERR_INVALID_ARG;
  if (plan && (plan->M != M || plan->K != K)) return BSP_ERR_INVALID_ARG;
  if (plan && plan->device != current_device()) return BSP_ERR_INVALID_ARG;
  if (M == 0 || N == 0) return kDone;
  if (!C || (K > 0 && (!A_words || !B))) return BSP_ERR_INVALID_ARG;
  const int esz = dtype_size(b_dtype);
  if (!is_aligned(B, esz) || !is_aligned(C, 4) || !is_aligned(A_words, 4)) return BSP_ERR_ALIGNMENT;
  if (K == 0) {  // C = 0
    BSP_CUDA(cudaMemset2DAsync(C, sizeof(float) * ldc, 0, sizeof(float) * N, M, s));
    return kDone;
  }
  const int vcols = b_dtype == BSP_F32 ? 4 : 8;
  *vec = is_aligned(B, 16) && ((ldb * esz) % 16 == 0) && (N % vcols == 0) && is_aligned(C, 16) && (ldc % 4 == 0);
  *a = SpmmArgs{};
  a->A = A_words;
  a->M = M;
  a->K = K;
  a->Kw = ceil_div(K, 32);
  a->B = B;
  a->bdt = b_dtype;
  a->ldb = ldb;
  a->N = N;
  a->C = C;
  a->ldc = ldc;
  *tc_ok = plan && *vec && b_dtype != BSP_F32 && N % 8 == 0 && plan->K <= tc_max_reduction();
  *esz_out = esz;
  return BSP_OK;
}

int bsp_spmm(const uint32_t* A_words, int64_t M, int64_t K, const void* B, int b_dtype,
             int64_t ldb, int64_t N, float* C, int64_t ldc, const bsp_plan* plan, void* workspace,
             size_t workspace_bytes, bsp_stream_t stream) {
  const cudaStream_t s = (cudaStream_t)stream;
  SpmmArgs a;
  bool vec = false, tc_ok = false;
  int esz = 4;
  const int rc = prepare_spmm(A_words, M, K, B, b_dtype, ldb, N, C, ldc, plan, s, &a, &vec, &tc_ok, &esz);
  if (rc != BSP_OK) return rc == kDone ? BSP_OK : rc;
  // A measured schedule for this shape bucket (bsp_tune) replaces the cost
  // model, unless the environment forces a choice.
  TuneSched sc = default_schedule(plan, N, esz, tc_ok);
  TuneSched tuned;
  if (plan && !getenv("BSP_TC") && !getenv("BSP_PROTO_PATH") && !getenv("BSP_PROTO_VARIANT") &&
      tune_lookup(plan, N, b_dtype, &tuned) && (tuned.engine == 2 || tc_ok))
    sc = tuned;
  return run_spmm(a, plan, vec, sc, workspace, workspace_bytes, s);
}

int bsp_tune(const uint32_t* A_words, int64_t M, int64_t K, const void* B, int b_dtype, int64_t ldb, int64_t N,
             float* C, int64_t ldc, const bsp_plan* plan, void* workspace, size_t workspace_bytes,
             bsp_stream_t stream, bsp_schedule* best) {
  if (!plan || !best) return BSP_ERR_INVALID_ARG;
  const cudaStream_t s = (cudaStream_t)stream;
  SpmmArgs a;
  bool vec = false, tc_ok = false;
  int esz = 4;
  const int rc = prepare_spmm(A_words, M, K, B, b_dtype, ldb, N, C, ldc, plan, s, &a, &vec, &tc_ok, &esz);
  if (rc == kDone) return BSP_ERR_INVALID_ARG;  // nothing to time
  BSP_TRY(rc);
  // candidates: the tensor cores in each tile form (2 or 3 K tiles per
  // stage, B by boxes or pre-tiled, split-K by the rule or never); every
  // prototype-kernel shape on both CUDA-core paths; the plain walk when the
  // plan has no prototypes
  TuneSched cand[8 + 9 + 8];
  int nc = 0;
  if (tc_ok)
    for (int tps = 2; tps <= 3; tps++)
      for (int tiled = 0; tiled <= 1; tiled++)
        for (int split = -1; split <= 0; split++) {
          TuneSched t;
          t.engine = 1;
          t.tc_tps = tps;
          t.tc_tiled = tiled;
          t.tc_split = split;
          cand[nc++] = t;
        }
  if (plan->mode == BSP_PLAN_PROTO && vec) {
    for (int v = 0; v <= 8; v++) cand[nc++] = TuneSched{2, 0, v, 0.0};
    for (int v = 0; v <= 7; v++) cand[nc++] = TuneSched{2, 1, v, 0.0};
  } else {
    cand[nc++] = TuneSched{2, 0, proto_variant(esz), 0.0};
  }
  cudaEvent_t e0, e1;
  BSP_CUDA(cudaEventCreate(&e0));
  BSP_CUDA(cudaEventCreate(&e1));
  int bi = -1;
  int last = BSP_OK;
  for (int c = 0; c < nc; c++) {
    bool ok = true;
    for (int r = 0; r < 2 && ok; r++) ok = (last = run_spmm(a, plan, vec, cand[c], workspace, workspace_bytes, s)) == BSP_OK;
    if (!ok) continue;
    const int reps = 5;
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps && ok; r++) ok = (last = run_spmm(a, plan, vec, cand[c], workspace, workspace_bytes, s)) == BSP_OK;
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess || !ok) continue;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cand[c].ms = ms / reps;
    if (bi < 0 || cand[c].ms < cand[bi].ms) bi = c;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (bi < 0) return last != BSP_OK ? last : BSP_ERR_INTERNAL;
  // leave C holding the chosen schedule's result
  BSP_TRY(run_spmm(a, plan, vec, cand[bi], workspace, workspace_bytes, s));
  tune_store(tune_key(plan, N, b_dtype), cand[bi]);
  best->engine = cand[bi].engine;
  best->proto_path = cand[bi].proto_path;
  best->proto_variant = cand[bi].proto_variant;
  best->tc_stage_tiles = cand[bi].tc_tps;
  best->tc_tiled_b = cand[bi].tc_tiled;
  best->tc_split = cand[bi].tc_split;
  best->ms = (float)cand[bi].ms;
  return BSP_OK;
}

int bsp_tune_cache_load(const char* path, int* entries) {
  if (!path) return BSP_ERR_INVALID_ARG;
  return tune_cache_load(path, entries);
}

int bsp_tune_cache_save(const char* path) {
  if (!path) return BSP_ERR_INVALID_ARG;
  return tune_cache_save(path);
}

int bsp_tune_cache_clear(void) {
  tune_cache_clear();
  return BSP_OK;
}

int bsp_tune_cache_size(int* entries) {
  if (!entries) return BSP_ERR_INVALID_ARG;
  *entries = tune_cache_size();
  return BSP_OK;
}

int bsp_symbolic_rows(const uint32_t* A_words, int64_t M, int64_t K, const uint32_t* B_words, int64_t N,
                      uint32_t* C_words, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (N < 0 || N > kMaxCols) return BSP_ERR_INVALID_ARG;
  if (M == 0 || N == 0) return BSP_OK;
  if (!C_words || (K > 0 && (!A_words || !B_words))) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(A_words, 4) || !is_aligned(B_words, 4) || !is_aligned(C_words, 4)) return BSP_ERR_ALIGNMENT;
  const cudaStream_t s = (cudaStream_t)stream;
  if (K == 0) {
    BSP_CUDA(cudaMemsetAsync(C_words, 0, sizeof(uint32_t) * (size_t)M * (size_t)ceil_div(N, 32), s));
    return BSP_OK;
  }
  return launch_symbolic_rows(A_words, M, K, B_words, N, C_words, s);
}

// The planned form needs a prototype plan for this A, counts below 2^16
// (K < 65536) and the workspace for the cluster planes; otherwise the walk.
static bool symbolic_planned_ok(const bsp_plan* plan, int64_t M, int64_t K) {
  return plan && plan->mode == BSP_PLAN_PROTO && plan->n_proto > 0 && plan->M == M && plan->K == K && K < 65536;
}

int bsp_symbolic_workspace(const bsp_plan* plan, int64_t N, size_t* bytes) {
  if (!bytes || N < 0) return BSP_ERR_INVALID_ARG;
  *bytes = 0;
  if (plan && plan->mode == BSP_PLAN_PROTO && plan->n_proto > 0 && plan->K < 65536)
    *bytes = symbolic_planes_bytes(plan->n_proto, N) + 256;
  return BSP_OK;
}

int bsp_symbolic_rows_planned(const uint32_t* A_words, int64_t M, int64_t K, const uint32_t* B_words, int64_t N,
                              uint32_t* C_words, const bsp_plan* plan, void* workspace, size_t workspace_bytes,
                              bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (N < 0 || N > kMaxCols) return BSP_ERR_INVALID_ARG;
  if (plan && (plan->M != M || plan->K != K)) return BSP_ERR_INVALID_ARG;
  if (plan && plan->device != current_device()) return BSP_ERR_INVALID_ARG;
  if (!symbolic_planned_ok(plan, M, K) || M == 0 || N == 0 || K == 0)
    return bsp_symbolic_rows(A_words, M, K, B_words, N, C_words, stream);
  if (!C_words || !A_words || !B_words) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(A_words, 4) || !is_aligned(B_words, 4) || !is_aligned(C_words, 4)) return BSP_ERR_ALIGNMENT;
  const size_t need = symbolic_planes_bytes(plan->n_proto, N) + 256;
  if (!workspace || workspace_bytes < need) return BSP_ERR_WORKSPACE;
  uint32_t* planes = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  return launch_symbolic_planned(A_words, M, K, B_words, N, C_words, plan->row_cluster, plan->delta_ptr,
                                 plan->delta_idx, plan->cons, plan->n_proto, planes, (cudaStream_t)stream);
}

static bool layout16(const void* p, int64_t ld, int esz, int64_t N, int vcols);

int bsp_bitplane_spmm(const uint32_t* planes, int n_planes, int is_signed, int64_t M, int64_t K, const void* B,
                      int b_dtype, int64_t ldb, int64_t N, float* C, int64_t ldc, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (n_planes < 1 || n_planes > 8) return BSP_ERR_INVALID_ARG;
  if (N < 0 || N > kMaxCols || ldb < N || ldc < N) return BSP_ERR_INVALID_ARG;
  if (b_dtype != BSP_F32 && b_dtype != BSP_BF16 && b_dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (M == 0 || N == 0) return BSP_OK;
  if (!C || (K > 0 && (!planes || !B))) return BSP_ERR_INVALID_ARG;
  const int esz = dtype_size(b_dtype);
  if (!is_aligned(B, esz) || !is_aligned(C, 4) || !is_aligned(planes, 4)) return BSP_ERR_ALIGNMENT;
  const cudaStream_t s = (cudaStream_t)stream;
  if (K == 0) {
    BSP_CUDA(cudaMemset2DAsync(C, sizeof(float) * ldc, 0, sizeof(float) * N, M, s));
    return BSP_OK;
  }
  const int vcols = b_dtype == BSP_F32 ? 4 : 8;
  const bool vec = layout16(B, ldb, esz, N, vcols) && layout16(C, ldc, 4, N, 4);
  return launch_bitplane_spmm(planes, n_planes, is_signed != 0, M, K, B, b_dtype, ldb, N, C, ldc, vec, s);
}

int bsp_bitplanes_rows(const uint8_t* values, int64_t M, int64_t K, int64_t ld, int n_planes, uint32_t* words,
                       bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (n_planes < 1 || n_planes > 8 || ld < K) return BSP_ERR_INVALID_ARG;
  if (ceil_div(K, 32) * n_planes > kMaxCols / 32) return BSP_ERR_CAPACITY;
  if (M == 0 || K == 0) return BSP_OK;
  if (!values || !words) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(words, 4)) return BSP_ERR_ALIGNMENT;
  return launch_bitplanes(values, M, K, ld, n_planes, words, BSP_LSB_FIRST, (cudaStream_t)stream, 1);
}

int bsp_stack_planes_b(const void* B, int b_dtype, int64_t ldb, int64_t K, int64_t N, int n_planes, int is_signed,
                       void* B_out, int64_t ld_out, bsp_stream_t stream) {
  BSP_TRY(check_dims(K, N));
  if (n_planes < 1 || n_planes > 8 || ldb < N || ld_out < N) return BSP_ERR_INVALID_ARG;
  if (b_dtype != BSP_F32 && b_dtype != BSP_BF16 && b_dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (K == 0 || N == 0) return BSP_OK;
  if (!B || !B_out) return BSP_ERR_INVALID_ARG;
  const int esz = dtype_size(b_dtype);
  if (!is_aligned(B, esz) || !is_aligned(B_out, esz)) return BSP_ERR_ALIGNMENT;
  return launch_stack_planes_b(B, b_dtype, ldb, K, N, n_planes, is_signed != 0, B_out, ld_out, (cudaStream_t)stream);
}

int bsp_spmm_i8_workspace(int64_t M, int64_t K, size_t* bytes) {
  if (!bytes || M < 0 || K < 0) return BSP_ERR_INVALID_ARG;
  *bytes = sizeof(uint32_t) * 8 * (size_t)M * (size_t)ceil_div(K, 32) + 256;
  return BSP_OK;
}

int bsp_spmm_i8(const int8_t* A, int64_t M, int64_t K, int64_t lda, const void* B, int b_dtype, int64_t ldb,
                int64_t N, float* C, int64_t ldc, void* workspace, size_t workspace_bytes, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (lda < K) return BSP_ERR_INVALID_ARG;
  if (M == 0 || N == 0) return BSP_OK;
  if (K > 0 && !A) return BSP_ERR_INVALID_ARG;
  size_t need = 0;
  BSP_TRY(bsp_spmm_i8_workspace(M, K, &need));
  uint32_t* planes = nullptr;
  if (K > 0) {
    if (!workspace || workspace_bytes < need) return BSP_ERR_WORKSPACE;
    planes = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255);
    BSP_TRY(bsp_bitplanes(reinterpret_cast<const uint8_t*>(A), M, K, lda, 8, planes, BSP_LSB_FIRST, stream));
  }
  return bsp_bitplane_spmm(planes, 8, 1, M, K, B, b_dtype, ldb, N, C, ldc, stream);
}

int bsp_tiles8_workspace(int64_t M, int64_t K, size_t* bytes) {
  if (!bytes || M < 0 || K < 0) return BSP_ERR_INVALID_ARG;
  *bytes = tiles8_workspace_bytes(M, K) + 256;
  return BSP_OK;
}

int bsp_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K, uint64_t* bmp, int32_t* tile_row,
                       int32_t* tile_col, int32_t* offset, int64_t* n_tiles, void* workspace, size_t workspace_bytes,
                       bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (M * K >= ((int64_t)1 << 31)) return BSP_ERR_CAPACITY;
  if (!n_tiles || !offset) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(n_tiles, 8) || !is_aligned(offset, 4)) return BSP_ERR_ALIGNMENT;
  const cudaStream_t s = (cudaStream_t)stream;
  if (M == 0 || K == 0) {
    BSP_CUDA(cudaMemsetAsync(n_tiles, 0, sizeof(int64_t), s));
    BSP_CUDA(cudaMemsetAsync(offset, 0, sizeof(int32_t), s));
    return BSP_OK;
  }
  if (!words || !bmp || !tile_row || !tile_col) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(words, 4) || !is_aligned(bmp, 8) || !is_aligned(tile_row, 4) || !is_aligned(tile_col, 4))
    return BSP_ERR_ALIGNMENT;
  size_t need = 0;
  BSP_TRY(bsp_tiles8_workspace(M, K, &need));
  if (!workspace || workspace_bytes < need) return BSP_ERR_WORKSPACE;
  return launch_rows_to_tiles8(words, M, K, bmp, tile_row, tile_col, offset, n_tiles, workspace, s);
}

int bsp_tiles8_to_rows(const uint64_t* bmp, const int32_t* tile_row, const int32_t* tile_col, int64_t n_tiles,
                       int64_t M, int64_t K, uint32_t* words, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (n_tiles < 0 || n_tiles > ((int64_t)1 << 40)) return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!words || (n_tiles > 0 && (!bmp || !tile_row || !tile_col))) return BSP_ERR_INVALID_ARG;
  if (!is_aligned(words, 4) || !is_aligned(bmp, 8) || !is_aligned(tile_row, 4) || !is_aligned(tile_col, 4))
    return BSP_ERR_ALIGNMENT;
  return launch_tiles8_to_rows(bmp, tile_row, tile_col, n_tiles, M, K, words, (cudaStream_t)stream);
}

int bsp_csr_to_tiled_workspace(int64_t M, int64_t K, int64_t nnz, int tile_rows, int tile_cols, size_t* bytes) {
  if (!bytes || M < 0 || K < 0 || nnz < 0 || tile_rows < 1 || tile_cols < 1) return BSP_ERR_INVALID_ARG;
  *bytes = csr_tiled_workspace_bytes(M, K, nnz, tile_rows, tile_cols) + 256;
  return BSP_OK;
}

int bsp_csr_to_tiled(const int32_t* row_ptr, const int32_t* col_idx, const void* values, int value_bytes, int64_t M,
                     int64_t K, int64_t nnz, int tile_rows, int tile_cols, int32_t* tile_nnz_acc,
                     int32_t* tiled_offset, int32_t* tiled_col, void* tiled_values, void* workspace,
                     size_t workspace_bytes, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (nnz < 0 || tile_rows < 1 || tile_cols < 1 || value_bytes < 0 || value_bytes > 8) return BSP_ERR_INVALID_ARG;
  if (nnz >= ((int64_t)1 << 31)) return BSP_ERR_CAPACITY;
  if (M == 0 || K == 0) return BSP_OK;
  if (!row_ptr || !tile_nnz_acc || !tiled_offset || (nnz > 0 && (!col_idx || !tiled_col))) return BSP_ERR_INVALID_ARG;
  if ((values != nullptr) != (tiled_values != nullptr) || (values && value_bytes == 0)) return BSP_ERR_INVALID_ARG;
  size_t need = 0;
  BSP_TRY(bsp_csr_to_tiled_workspace(M, K, nnz, tile_rows, tile_cols, &need));
  if (!workspace || workspace_bytes < need) return BSP_ERR_WORKSPACE;
  return launch_csr_to_tiled(row_ptr, col_idx, values, value_bytes, M, K, nnz, tile_rows, tile_cols, tile_nnz_acc,
                             tiled_offset, tiled_col, tiled_values, workspace, (cudaStream_t)stream);
}

int bsp_spmm_t_workspace_preferred(int64_t M, int64_t K, int64_t N, size_t* bytes) {
  if (!bytes || M < 0 || K < 0 || N < 0) return BSP_ERR_INVALID_ARG;
  BSP_TRY(bsp_spmm_t_workspace(M, K, bytes));
  const size_t tc = tc_preferred_bytes(K, N, M);
  if (tc > *bytes) *bytes = tc;
  return BSP_OK;
}

int bsp_spmm_t_workspace(int64_t M, int64_t K, size_t* bytes) {
  if (!bytes || M < 0 || K < 0) return BSP_ERR_INVALID_ARG;
  *bytes = sizeof(uint32_t) * (size_t)K * (size_t)ceil_div(M, 32) + 256;
  return BSP_OK;
}

static bool layout16(const void* p, int64_t ld, int esz, int64_t N, int vcols) {
  return is_aligned(p, 16) && ((ld * esz) % 16 == 0) && (N % vcols == 0);
}

int bsp_spmm_t(const uint32_t* A_words, int64_t M, int64_t K, const void* G, int g_dtype, int64_t ldg,
               int64_t N, float* dX, int64_t lddx, const bsp_plan* plan, void* workspace,
               size_t workspace_bytes, bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (N < 0 || N > kMaxCols) return BSP_ERR_INVALID_ARG;
  if (g_dtype != BSP_F32 && g_dtype != BSP_BF16 && g_dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (ldg < N || lddx < N) return BSP_ERR_INVALID_ARG;
  if (plan && (plan->M != M || plan->K != K || plan->device != current_device())) return BSP_ERR_INVALID_ARG;
  if (K == 0 || N == 0) return BSP_OK;
  if (!dX || (M > 0 && (!A_words || !G))) return BSP_ERR_INVALID_ARG;
  const int esz = dtype_size(g_dtype);
  if (!is_aligned(G, esz) || !is_aligned(dX, 4) || !is_aligned(A_words, 4)) return BSP_ERR_ALIGNMENT;
  const cudaStream_t s = (cudaStream_t)stream;
  if (M == 0) {
    BSP_CUDA(cudaMemset2DAsync(dX, sizeof(float) * lddx, 0, sizeof(float) * N, K, s));
    return BSP_OK;
  }
  const int vcols = g_dtype == BSP_F32 ? 4 : 8;
  const bool vec = layout16(G, ldg, esz, N, vcols) && layout16(dX, lddx, 4, N, 4);
  if (plan && vec && g_dtype != BSP_F32 && M <= tc_max_reduction()) {
    const char* e = getenv("BSP_TC");
    const double tc = (double)plan->occT_tiles * 128.0 * 32.0 * (double)N * 2.0 / 1.2e15;
    const double cc = (double)plan->nnz * (double)N * (double)esz / 8e12;
    if (e ? e[0] == '1' : tc < cc)
      return launch_spmm_t_tc(A_words, M, K, G, g_dtype, ldg, N, dX, lddx, plan->occT, plan->wordsT, s, workspace,
                              workspace_bytes);
  }
  // CUDA cores: transpose the bits into the workspace, then walk the rows of Aᵀ
  size_t need = 0;
  bsp_spmm_t_workspace(M, K, &need);
  if (!workspace || workspace_bytes < need) return BSP_ERR_WORKSPACE;
  uint32_t* At = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  BSP_TRY(launch_transpose_bits(A_words, M, K, At, s));
  SpmmArgs a = {};
  a.A = At;
  a.M = K;
  a.K = M;
  a.Kw = ceil_div(M, 32);
  a.B = G;
  a.bdt = g_dtype;
  a.ldb = ldg;
  a.N = N;
  a.C = dX;
  a.ldc = lddx;
  return launch_spmm_rows(a, false, vec, s);
}

int bsp_sddmm(const uint32_t* A_words, int64_t M, int64_t K, const void* G, int64_t ldg, const void* X,
              int64_t ldx, int dtype, int64_t N, float* dA, int64_t ldda, const bsp_plan* plan,
              bsp_stream_t stream) {
  BSP_TRY(check_dims(M, K));
  if (N < 0 || N > kMaxCols) return BSP_ERR_INVALID_ARG;
  if (dtype != BSP_F32 && dtype != BSP_BF16 && dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (ldg < N || ldx < N || ldda < K) return BSP_ERR_INVALID_ARG;
  if (plan && (plan->M != M || plan->K != K || plan->device != current_device())) return BSP_ERR_INVALID_ARG;
  if (M == 0 || K == 0) return BSP_OK;
  if (!dA || !A_words || (N > 0 && (!G || !X))) return BSP_ERR_INVALID_ARG;
  const int esz = dtype_size(dtype);
  if (!is_aligned(G, esz) || !is_aligned(X, esz) || !is_aligned(dA, 4) || !is_aligned(A_words, 4))
    return BSP_ERR_ALIGNMENT;
  const cudaStream_t s = (cudaStream_t)stream;
  const bool tc_ok = dtype != BSP_F32 && N > 0 && layout16(G, ldg, esz, N, 8) && layout16(X, ldx, esz, N, 8) &&
                     layout16(dA, ldda, 4, K, 8);
  bool tc = tc_ok;
  const char* e = getenv("BSP_TC");
  if (tc_ok && e) tc = e[0] == '1';
  else if (tc_ok && plan) {  // dense product on the tensor cores vs one dot product per set bit
    const double dense = (double)M * (double)K * (double)N * 2.0 / 1.2e15;
    const double cores = (double)plan->nnz * (double)N * ((double)esz / 8e12 + 2.0 / 6e13);
    tc = dense < cores;
  }
  if (tc) return launch_sddmm_tc(A_words, M, K, G, ldg, X, ldx, dtype, N, dA, ldda, s);
  return launch_sddmm_rows(A_words, M, K, G, ldg, X, ldx, dtype, N, dA, ldda, s);
}

int bsp_device_status(int* status, int clear) {
  if (!status) return BSP_ERR_INVALID_ARG;
  int a = 0, b = 0, c = 0;
  BSP_TRY(bulk_device_error(&a, clear != 0));
  BSP_TRY(tc_device_error(&b, clear != 0));
  BSP_TRY(batched_device_error(&c, clear != 0));
  *status = a ? a : (b ? b : c);
  return BSP_OK;
}

}  // extern "C"
