// spmm_tc.cu — tensor-core bitmap SpMM for 16-bit B (tcgen05, TMEM).
//
// For matrices whose bits come in dense blocks (or are dense enough that a
// dense contraction beats per-bit adds), C = A·B runs on the 5th-generation
// tensor cores: each 32-column bit tile of A is expanded to 0/1 BF16/FP16
// operands in shared memory (the idea of the reference's tSparse kernel,
// source/src/mm.cu:123-145, which expanded 8x8 bitmap tiles into 0/1 half
// wmma fragments) and multiplied by the matching 32 rows of B.
//
// CTA tile: 128 rows x 256 columns of C, FP32 accumulator in TMEM (256
// columns).  K advances 32 columns (one packed word) per stage, and only over
// the K tiles where some row of the 128-row block has a set bit (the plan's
// occupancy bitmap), so empty bit tiles cost nothing.
//   warps 0-3 (producers): expand the 128 words of the stage into the A
//     operand (K-major core-matrix layout); warp 0 also issues the stage's
//     B tile as four 64x32 TMA boxes in the 128-byte-swizzled MN-major
//     layout; then, after the last stage, read the accumulator back with
//     tcgen05.ld and store C;
//   warp 4: allocates TMEM; its lane 0 issues two tcgen05.mma (K=16) per
//     stage and commits them to the stage's "empty" mbarrier.
// Four stages of 24 KB; every mbarrier wait is bounded (timeout → error 3
// in g_tc_error, the CTA skips to freeing its TMEM).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "ptx.cuh"
#include "spmm_dev.cuh"
#include "tc_common.cuh"

namespace bsp {

__device__ int g_tc_error;

namespace {

constexpr int kTcM = 128;
constexpr int kTcN = 256;
constexpr int kTcK = 32;
constexpr int kLook = 8;  // A words are loaded this many K tiles ahead
constexpr int kAStage = kTcM * kTcK * 2;  // 8 KB
constexpr int kBStage = kTcK * kTcN * 2;  // 16 KB
constexpr int kProducers = 128;
constexpr int kTcThreads = 160;
// kGuard: extra shared memory past the stage buffers and a full 512-column
// TMEM allocation, so that a misread descriptor field cannot reach memory
// the CTA does not own (used for the first bring-up of a descriptor change;
// costs one CTA per SM).
constexpr bool kGuard = false;
constexpr uint32_t kTmemCols = kGuard ? 512 : 256;
using tc::kLbo;
using tc::kSbo;
using tc::expand8;
using tc::kLayoutSw128;
using tc::kLayoutSw64;
constexpr int kFwd = 0, kTrans = 1, kSddmm = 2;
// B (fwd) / G (trans) tile: four TMA boxes of 64 columns x 32 reduction rows,
// 128-byte swizzle, kBox bytes apart (the LBO); 8-row groups 1 KB apart (SBO).
constexpr int kBoxCols = 64;
constexpr uint32_t kBox = kBoxCols * kTcK * 2;  // 4 KB
// SDDMM: G tile 128 rows x 32 (of N) and X tile 256 rows x 32 (of N), one
// box each, K-major with 64-byte swizzle (8-row groups 512 B apart).
constexpr uint32_t kSdSbo = 512;
// Shared memory is requested with this much slack so the stage buffers can
// be aligned to the 1 KB swizzle atom.
constexpr size_t kSmemAlign = 1024;

template <int kStages>
struct __align__(1024) TcSmem {
  uint8_t a[kStages][kAStage];
  uint8_t b[kStages][kBStage];
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t done;
  uint32_t tmem_addr;
  int abort;
  uint8_t guard[kGuard ? 65536 : 16];
};

__host__ __device__ constexpr uint32_t idesc_f16(uint32_t ab_type, uint32_t a_mn, uint32_t b_mn) {
  return tc::idesc_f16(ab_type, a_mn, b_mn, kTcN, kTcM);
}

struct TcArgs {
  const uint32_t* A;  // bit matrix, packed rows [M][Kw]
  int64_t M, K, Kw;
  const void* B;      // fwd: B [K][ldb]; trans: G [M][ldb]; sddmm: X [K][ldb]
  int64_t ldb;
  const void* G;      // sddmm: G [M][ldg]
  int64_t ldg;
  int64_t N;
  float* C;           // fwd: C [M][ldc]; trans: dX [K][ldc]; sddmm: dA [M][ldc]
  int64_t ldc;
  const uint32_t* occ;  // fwd / trans occupancy bitmap (unused by sddmm)
  int occ_words;
  int bdt;
};

struct TileIter {  // set bits of the block's occupancy words, ascending
  const uint32_t* occ;
  int ow, nw;
  uint32_t bits;
  __device__ void init(const uint32_t* o, int n) {
    occ = o;
    nw = n;
    ow = -1;
    bits = 0;
  }
  __device__ __forceinline__ int next() {
    while (bits == 0) {
      if (++ow >= nw) return -1;
      bits = __ldg(occ + ow);
    }
    const int b = __ffs(bits) - 1;
    bits &= bits - 1;
    return ow * 32 + b;
  }
};

// Steps of the reduction: occupied tiles from a bitmap (forward: K tiles of
// the CTA's 128-row block; transposed: row tiles of its 128-column block) or
// every 32-column step of N (SDDMM).
struct StepIter {
  TileIter it;
  int dense_left, dense_i;
  bool dense;
  __device__ void init(const uint32_t* occ, int words, int dense_steps, bool is_dense) {
    dense = is_dense;
    dense_left = dense_steps;
    dense_i = 0;
    if (!dense) it.init(occ, words);
  }
  __device__ __forceinline__ int next() {
    if (dense) return dense_left-- > 0 ? dense_i++ : -1;
    return it.next();
  }
};

// One kernel, three products (MODE):
//   kFwd   C[M,N]  = A · B        A bits K-major from A's words, B MN-major
//   kTrans C[K,N]  = Aᵀ · G       Aᵀ MN-major built from A's row words (no
//                                 transposed copy), G MN-major
//   kSddmm dA[M,K] = (G · Xᵀ) ⊙ A  G and X K-major (TMA, 64-byte swizzle),
//                                 dense over N, masked store
// The bit operands are expanded into core matrices (LBO = 128 B along the
// reduction, SBO = 512 B along M/N); the dense 16-bit operands come by TMA
// in swizzled layouts.  The modes differ only in the producers, the
// descriptors and the epilogue.
template <typename BT, int MODE, int kStages>
__global__ void __launch_bounds__(kTcThreads, 1) k_spmm_tc(TcArgs a, const __grid_constant__ CUtensorMap mapA,
                                                          const __grid_constant__ CUtensorMap mapB) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  TcSmem<kStages>& sm = *reinterpret_cast<TcSmem<kStages>*>(
      smem_raw + ((kSmemAlign - (ptx::smem_addr(smem_raw) & (kSmemAlign - 1))) & (kSmemAlign - 1)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * kTcM;  // output rows: M (fwd, sddmm) or K (trans)
  const int64_t col0 = (int64_t)blockIdx.y * kTcN;  // output columns: N (fwd, trans) or K (sddmm)
  const int64_t out_rows = MODE == kTrans ? a.K : a.M;
  const int64_t out_cols = MODE == kSddmm ? a.K : a.N;
  const uint32_t one = std::is_same<BT, __nv_bfloat16>::value ? 0x3f80u : 0x3c00u;

  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      ptx::mbar_init(&sm.full[s], kProducers + 1);  // producers + the TMA transaction arrival
      ptx::mbar_init(&sm.empty[s], 1);
    }
    ptx::mbar_init(&sm.done, 1);
    sm.abort = 0;
    ptx::fence_mbar_init();
  }
  if (warp == 4) {
    ptx::tmem_alloc(&sm.tmem_addr, kTmemCols);
    ptx::tmem_relinquish();
  }
  // SDDMM: a block of A without set bits needs no product at all
  int any = 1;
  if (MODE == kSddmm) {
    uint32_t acc = 0;
    if (warp < 4 && row0 + tid < a.M) {
      const uint32_t* arow = a.A + (row0 + tid) * a.Kw;
      for (int64_t w = col0 / 32; w < min(a.Kw, (col0 + kTcN) / 32); w++) acc |= __ldg(arow + w);
    }
    any = __syncthreads_or(acc != 0u);
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  ptx::tc_fence_after_sync();
  const uint32_t tmem = sm.tmem_addr;
  const int dense_steps = any ? (int)((a.N + kTcK - 1) / kTcK) : 0;
  const uint32_t* block_occ = a.occ + (int64_t)blockIdx.x * a.occ_words;
  int ntiles = 0;

  if (warp < 4) {
    // ---------------- producers ----------------
    // Operands that are dense 16-bit tiles come by TMA (warp 0 issues the
    // boxes and the stage's transaction count); the bit tiles of A are
    // expanded by all 128 producers from words loaded two tiles ahead.
    StepIter it;
    it.init(block_occ, a.occ_words, dense_steps, MODE == kSddmm);
    auto load_word = [&](int t) -> uint32_t {
      if (t < 0 || MODE == kSddmm) return 0u;
      if (MODE == kFwd) {
        const int64_t arow = row0 + tid;
        return arow < a.M ? __ldg(a.A + arow * a.Kw + t) : 0u;
      }
      const int64_t arow = (int64_t)t * kTcK + (tid & 31);
      const int64_t wcol = row0 / 32 + (tid >> 5);
      return (arow < a.M && wcol < a.Kw) ? __ldg(a.A + arow * a.Kw + wcol) : 0u;
    };
    // tq[0] is the current tile, tq[1..kLook] the next ones; wq[j] holds the
    // A word of tq[j] (loads issued kLook tiles before use)
    int tq[kLook + 1];
    uint32_t wq[kLook];
#pragma unroll
    for (int j = 0; j <= kLook; j++) tq[j] = (j == 0 || tq[j - 1] >= 0) ? it.next() : -1;
#pragma unroll
    for (int j = 0; j < kLook; j++) wq[j] = load_word(tq[j]);
    int i = 0;
    for (; tq[0] >= 0; i++) {
      const int t0 = tq[0];
      const uint32_t w0 = wq[0];
      const uint32_t wnew = load_word(tq[kLook]);
      const int s = i % kStages;
      if (i >= kStages && !ptx::mbar_wait(&sm.empty[s], ((i / kStages) - 1) & 1)) {
        atomicCAS(&g_tc_error, 0, 3);
        sm.abort = 1;
        break;
      }
      if (*(volatile int*)&sm.abort) break;
      if (warp == 0) {
        if (lane == 0) ptx::mbar_arrive_expect_tx(&sm.full[s], MODE == kSddmm ? kAStage + kBStage : kBStage);
        __syncwarp();
        if (MODE == kSddmm) {
          // G rows row0.. and X rows col0.., columns t0*32..: one box each
          if (lane == 0) ptx::tma_load_2d(sm.a[s], &mapA, t0 * kTcK, (int)row0, &sm.full[s]);
          else if (lane == 1) ptx::tma_load_2d(sm.b[s], &mapB, t0 * kTcK, (int)col0, &sm.full[s]);
        } else if (lane < kTcN / kBoxCols) {
          // B (fwd) / G (trans): reduction rows t0*32.., columns col0 + 64*lane
          ptx::tma_load_2d(sm.b[s] + lane * kBox, &mapB, (int)col0 + lane * kBoxCols, t0 * kTcK, &sm.full[s]);
        }
      }
      if (MODE == kFwd) {
        uint8_t* as = sm.a[s] + (tid >> 3) * kSbo + (tid & 7) * 16;
#pragma unroll
        for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(as + c * kLbo) = expand8((w0 >> (8 * c)) & 0xffu, one);
      } else if (MODE == kTrans) {
        const int j = tid & 31, wk = tid >> 5;
        uint8_t* as = sm.a[s] + (j >> 3) * kLbo + (j & 7) * 16;
#pragma unroll
        for (int c = 0; c < 4; c++)
          *reinterpret_cast<uint4*>(as + (wk * 4 + c) * kSbo) = expand8((w0 >> (8 * c)) & 0xffu, one);
      }
      ptx::fence_proxy_async_smem();
      ptx::mbar_arrive(&sm.full[s]);
#pragma unroll
      for (int j = 0; j < kLook - 1; j++) wq[j] = wq[j + 1];
      wq[kLook - 1] = wnew;
#pragma unroll
      for (int j = 0; j < kLook; j++) tq[j] = tq[j + 1];
      tq[kLook] = tq[kLook] >= 0 ? it.next() : -1;
    }
    ntiles = i;
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t ab = std::is_same<BT, __nv_bfloat16>::value ? 1u : 0u;
    const uint32_t idesc = idesc_f16(ab, MODE == kTrans ? 1u : 0u, MODE == kSddmm ? 0u : 1u);
    StepIter it;
    it.init(block_occ, a.occ_words, dense_steps, MODE == kSddmm);
    int i = 0;
    for (int t = it.next(); t >= 0; t = it.next(), i++) {
      const int s = i % kStages;
      if (!ptx::mbar_wait(&sm.full[s], (i / kStages) & 1)) {
        atomicCAS(&g_tc_error, 0, 3);
        sm.abort = 1;
        break;
      }
      if (*(volatile int*)&sm.abort) break;
      ptx::tc_fence_after_sync();
#pragma unroll
      for (int j = 0; j < 2; j++) {
        uint64_t ad, bd;
        if (MODE == kSddmm) {  // both K-major, 64-byte swizzle; K half j starts 32 B in
          ad = ptx::smem_desc_swizzle(sm.a[s] + j * 32, 16, kSdSbo, kLayoutSw64);
          bd = ptx::smem_desc_swizzle(sm.b[s] + j * 32, 16, kSdSbo, kLayoutSw64);
        } else {  // A: core matrices; B: 128-byte swizzle, K half j = two 8-row groups on
          ad = ptx::smem_desc_noswizzle(sm.a[s] + j * 2 * kLbo, kLbo, kSbo);
          bd = ptx::smem_desc_swizzle(sm.b[s] + j * 2 * 1024, kBox, 1024, kLayoutSw128);
        }
        ptx::tc_mma_f16(tmem, ad, bd, idesc, (i > 0) || (j > 0));
      }
      ptx::tc_commit(&sm.empty[s]);
    }
    if (i > 0) ptx::tc_commit(&sm.done);
    else ptx::mbar_arrive(&sm.done);
  }

  // ---------------- epilogue (warps 0-3) ----------------
  if (warp < 4) {
    const bool have = ntiles > 0;
    bool ok = ptx::mbar_wait(&sm.done, 0);
    if (!ok) {
      atomicCAS(&g_tc_error, 0, 3);
      sm.abort = 1;
    }
    ptx::tc_fence_after_sync();
    const int64_t row = row0 + warp * 32 + lane;
    float* crow = a.C + row * a.ldc + col0;
    const bool live = row < out_rows && ok && !*(volatile int*)&sm.abort;
    const uint32_t* arow = a.A + row * a.Kw;
    for (int c8 = 0; c8 < kTcN / 8; c8 += 4) {
      uint32_t r[4][8];
      if (have && ok) {
#pragma unroll
        for (int u = 0; u < 4; u++)
          ptx::tmem_ld_32x32b_x8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((c8 + u) * 8), r[u]);
        ptx::tmem_wait_ld();
      } else {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int q = 0; q < 8; q++) r[u][q] = 0u;
      }
      if (!live) continue;
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int col = (c8 + u) * 8;
        if (col0 + col >= out_cols) continue;
        if (MODE == kSddmm) {  // keep the set bits of A's row only
          const uint32_t bits = (__ldg(arow + (col0 + col) / 32) >> ((col0 + col) & 31)) & 0xffu;
#pragma unroll
          for (int q = 0; q < 8; q++)
            if (!((bits >> q) & 1u)) r[u][q] = 0u;
        }
        *reinterpret_cast<float4*>(crow + col) = make_float4(
            __uint_as_float(r[u][0]), __uint_as_float(r[u][1]), __uint_as_float(r[u][2]), __uint_as_float(r[u][3]));
        *reinterpret_cast<float4*>(crow + col + 4) = make_float4(
            __uint_as_float(r[u][4]), __uint_as_float(r[u][5]), __uint_as_float(r[u][6]), __uint_as_float(r[u][7]));
      }
    }
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  if (warp == 4) {
    ptx::tc_fence_after_sync();
    ptx::tmem_dealloc(tmem, kTmemCols);
  }
}

// Occupancy of Aᵀ's tiles: warp per (128-column block of A, 32 consecutive
// 32-row tiles); lane = row tile, OR of 32 rows x 4 words, one ballot.
__global__ void __launch_bounds__(256) k_tile_occupancy_t(const uint32_t* __restrict__ A, int64_t M, int64_t Kw,
                                                          int occ_words, int64_t nkb, uint32_t* __restrict__ occ,
                                                          unsigned long long* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (warp >= nkb * occ_words) return;
  const int64_t kb = warp / occ_words;
  const int ow = (int)(warp - kb * occ_words);
  const int64_t it = (int64_t)ow * 32 + lane;
  uint32_t acc = 0;
  const int64_t r0 = it * kTcK, r1 = min(M, r0 + kTcK);
  for (int64_t r = r0; r < r1; r++)
    for (int64_t w = kb * 4; w < min(Kw, kb * 4 + 4); w++) acc |= __ldg(A + r * Kw + w);
  const uint32_t m = __ballot_sync(kFull, acc != 0u);
  if (lane == 0) {
    occ[warp] = m;
    if (count && m) atomicAdd(count, (unsigned long long)__popc(m));
  }
}

// Occupancy: warp per (128-row block, 32 consecutive K tiles); lane = K tile,
// OR of the 128 rows' words, one ballot → occupancy word.
__global__ void __launch_bounds__(256) k_tile_occupancy(const uint32_t* __restrict__ A, int64_t M, int64_t Kw,
                                                        int occ_words, uint32_t* __restrict__ occ,
                                                        unsigned long long* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nrb = (M + kTcM - 1) / kTcM;
  if (warp >= nrb * occ_words) return;
  const int64_t rb = warp / occ_words;
  const int ow = (int)(warp - rb * occ_words);
  const int64_t kt = (int64_t)ow * 32 + lane;
  uint32_t acc = 0;
  if (kt < Kw) {
    const int64_t r1 = min(M, (rb + 1) * kTcM);
    for (int64_t r = rb * kTcM; r < r1; r++) acc |= __ldg(A + r * Kw + kt);
  }
  const uint32_t m = __ballot_sync(kFull, acc != 0u);
  if (lane == 0) {
    occ[warp] = m;
    if (count && m) atomicAdd(count, (unsigned long long)__popc(m));
  }
}

}  // namespace

int tc_occupancy_words(int64_t K) { return (int)ceil_div(ceil_div(K, 32), 32); }
int tc_occupancy_t_words(int64_t M) { return (int)ceil_div(ceil_div(M, 32), 32); }

int launch_tile_occupancy(const uint32_t* A, int64_t M, int64_t K, uint32_t* occ,
                          unsigned long long* count, cudaStream_t s) {
  const int ow = tc_occupancy_words(K);
  const int64_t warps = ceil_div(M, kTcM) * ow;
  if (warps == 0) return BSP_OK;
  k_tile_occupancy<<<(unsigned)ceil_div(warps, 8), 256, 0, s>>>(A, M, ceil_div(K, 32), ow, occ, count);
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_tile_occupancy_t(const uint32_t* A, int64_t M, int64_t K, uint32_t* occT,
                            unsigned long long* count, cudaStream_t s) {
  const int ow = tc_occupancy_t_words(M);
  const int64_t nkb = ceil_div(K, kTcM);
  const int64_t warps = nkb * ow;
  if (warps == 0) return BSP_OK;
  k_tile_occupancy_t<<<(unsigned)ceil_div(warps, 8), 256, 0, s>>>(A, M, ceil_div(K, 32), ow, nkb, occT, count);
  BSP_LAUNCHED();
  return BSP_OK;
}

namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link-time dependency on the driver library).
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D map over a row-major [rows][cols] 16-bit matrix (row stride ld
// elements), box = box_cols x box_rows, out-of-range = zero.
int make_map(CUtensorMap* m, const void* base, int dt, int64_t rows, int64_t cols, int64_t ld, uint32_t box_cols,
             uint32_t box_rows, CUtensorMapSwizzle swz) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_tiled();
  if (!enc) return BSP_ERR_UNSUPPORTED;
  const cuuint64_t dims[2] = {(cuuint64_t)(cols > 0 ? cols : 1), (cuuint64_t)(rows > 0 ? rows : 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, dt == BSP_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                         const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? BSP_OK : BSP_ERR_ALIGNMENT;
}

template <typename BT, int MODE, int S>
int launch_stages(const TcArgs& a, const CUtensorMap& ma, const CUtensorMap& mb, dim3 grid, cudaStream_t s) {
  const size_t smem = sizeof(TcSmem<S>) + kSmemAlign;
  static bool configured[64] = {};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(k_spmm_tc<BT, MODE, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured[dev] = true;
  }
  k_spmm_tc<BT, MODE, S><<<grid, kTcThreads, smem, s>>>(a, ma, mb);
  BSP_LAUNCHED();
  return BSP_OK;
}

// Stage ring depth: 4 stages (two CTAs per SM) or 6 / 8 (one CTA per SM);
// BSP_TC_STAGES selects it for tuning.
int tc_stages() {
  static int v = 0;
  if (!v) {
    const char* e = getenv("BSP_TC_STAGES");
    v = e ? atoi(e) : 4;
    if (v != 4 && v != 6 && v != 8) v = 4;
  }
  return v;
}

template <typename BT, int MODE>
int launch_mode(const TcArgs& a, const CUtensorMap& ma, const CUtensorMap& mb, dim3 grid, cudaStream_t s) {
  switch (tc_stages()) {
    case 6: return launch_stages<BT, MODE, 6>(a, ma, mb, grid, s);
    case 8: return launch_stages<BT, MODE, 8>(a, ma, mb, grid, s);
    default: return launch_stages<BT, MODE, 4>(a, ma, mb, grid, s);
  }
}

template <int MODE>
int launch_tc(const TcArgs& a, cudaStream_t s) {
  const int64_t rows = MODE == kTrans ? a.K : a.M;
  const int64_t cols = MODE == kSddmm ? a.K : a.N;
  if (rows == 0 || cols == 0) return BSP_OK;
  const dim3 grid((unsigned)ceil_div(rows, kTcM), (unsigned)ceil_div(cols, kTcN));
  if (ceil_div(cols, kTcN) > 65535 || ceil_div(rows, kTcM) > 0x7fffffff) return BSP_ERR_CAPACITY;
  if (a.N > INT32_MAX || a.M > INT32_MAX || a.K > INT32_MAX) return BSP_ERR_CAPACITY;
  CUtensorMap ma, mb;
  memset(&ma, 0, sizeof(ma));
  if (MODE == kSddmm) {
    BSP_TRY(make_map(&ma, a.G, a.bdt, a.M, a.N, a.ldg, kTcK, kTcM, CU_TENSOR_MAP_SWIZZLE_64B));  // G [M][N]
    BSP_TRY(make_map(&mb, a.B, a.bdt, a.K, a.N, a.ldb, kTcK, kTcN, CU_TENSOR_MAP_SWIZZLE_64B));  // X [K][N]
  } else {
    // B [K][N] (fwd) or G [M][N] (trans), 64 columns x 32 reduction rows per box
    BSP_TRY(make_map(&mb, a.B, a.bdt, MODE == kFwd ? a.K : a.M, a.N, a.ldb, kBoxCols, kTcK,
                     CU_TENSOR_MAP_SWIZZLE_128B));
  }
  if (a.bdt == BSP_BF16) return launch_mode<__nv_bfloat16, MODE>(a, ma, mb, grid, s);
  if (a.bdt == BSP_F16) return launch_mode<__half, MODE>(a, ma, mb, grid, s);
  return BSP_ERR_UNSUPPORTED;
}
}  // namespace

int launch_spmm_tc(const SpmmArgs& sa, const uint32_t* occ, cudaStream_t s) {
  TcArgs a = {};
  a.A = sa.A;
  a.M = sa.M;
  a.K = sa.K;
  a.Kw = sa.Kw;
  a.B = sa.B;
  a.ldb = sa.ldb;
  a.N = sa.N;
  a.C = sa.C;
  a.ldc = sa.ldc;
  a.occ = occ;
  a.occ_words = tc_occupancy_words(sa.K);
  a.bdt = sa.bdt;
  return launch_tc<kFwd>(a, s);
}

int launch_spmm_t_tc(const uint32_t* A, int64_t M, int64_t K, const void* G, int gdt, int64_t ldg, int64_t N,
                     float* dX, int64_t lddx, const uint32_t* occT, cudaStream_t s) {
  TcArgs a = {};
  a.A = A;
  a.M = M;
  a.K = K;
  a.Kw = ceil_div(K, 32);
  a.B = G;
  a.ldb = ldg;
  a.N = N;
  a.C = dX;
  a.ldc = lddx;
  a.occ = occT;
  a.occ_words = tc_occupancy_t_words(M);
  a.bdt = gdt;
  return launch_tc<kTrans>(a, s);
}

int launch_sddmm_tc(const uint32_t* A, int64_t M, int64_t K, const void* G, int64_t ldg, const void* X,
                    int64_t ldx, int dt, int64_t N, float* dA, int64_t ldda, cudaStream_t s) {
  TcArgs a = {};
  a.A = A;
  a.M = M;
  a.K = K;
  a.Kw = ceil_div(K, 32);
  a.B = X;
  a.ldb = ldx;
  a.G = G;
  a.ldg = ldg;
  a.N = N;
  a.C = dA;
  a.ldc = ldda;
  a.bdt = dt;
  return launch_tc<kSddmm>(a, s);
}

int tc_device_error(int* out, bool clear) {
  BSP_CUDA(cudaMemcpyFromSymbol(out, g_tc_error, sizeof(int)));
  if (clear) {
    const int zero = 0;
    BSP_CUDA(cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)));
  }
  return BSP_OK;
}

}  // namespace bsp
