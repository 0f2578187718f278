// spmm_tc.cu — tensor-core bitmap SpMM for 16-bit B (tcgen05, TMEM).
//
// For matrices whose bits come in dense blocks (or are dense enough that a
// dense contraction beats per-bit adds), C = A·B runs on the 5th-generation
// tensor cores: each 32-column bit tile of A is expanded to 0/1 BF16/FP16
// operands in shared memory (the idea of the reference's tSparse kernel,
// source/src/mm.cu:123-145, which expanded 8x8 bitmap tiles into 0/1 half
// wmma fragments) and multiplied by the matching 32 rows of B.
//
// CTA tile: 256 rows x 256 columns of C as two 128-row halves, each with its
// FP32 accumulator in TMEM (2 x 256 columns); both halves multiply the same
// B stage, so every B byte brought into shared memory feeds 256 rows.  K
// advances over the 32-column tiles where either 128-row block has a set bit
// (the plan's occupancy bitmap); a half without bits in a tile skips its
// MMAs.  A stage carries TPS tiles (2 tiles x 3 stages, or 3 x 2 where many
// row blocks share B); per CTA:
//   256·TPS producer threads (one row of one tile each): load the tile's
//     words (column-major copy in the plan: one 128-byte run per warp),
//     expand them into the A operand (K-major core matrices, 2.0 per set
//     bit) and arrive on the stage's "full" mbarrier; after the last stage
//     16 of these warps read the accumulators back (tcgen05.ld), scale by
//     0.5 and store C through a 32x32 staging tile per warp;
//   a TMA warp: B rows of the stage's tiles, either as one bulk copy of 16
//     KB per tile from B already in tile order (k_tile_b) or as four 64x32
//     tensor boxes (128-byte swizzle, MN-major);
//   an MMA warp: allocates TMEM; its lane 0 issues two tcgen05.mma (K=16) per
//     occupied half per tile and commits the stage to its "empty" mbarrier.
// An mbarrier hand-off costs 200-500 cycles on GB300, and the tensor pipe
// queues about one MMA beyond the running one, so the design keeps the
// MMA thread's work between stages minimal and carries several tiles per
// hand-off.  Every mbarrier wait is bounded (timeout -> error 3 in
// g_tc_error, the CTA skips its stores and frees its TMEM).
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

constexpr int kTcM = 128;                 // rows of one MMA and of one occupancy block
constexpr int kHalves = 2;                // a CTA owns two 128-row halves ...
constexpr int kCtaM = kTcM * kHalves;     // ... 256 output rows, sharing every B tile
constexpr int kTcN = 256;
constexpr int kTcK = 32;                  // one packed word of A per row and K tile
constexpr int kATile = kCtaM * kTcK * 2;  // 16 KB: both halves of one K tile
constexpr int kAHalf = kTcM * kTcK * 2;   // 8 KB
constexpr int kBTile = kTcK * kTcN * 2;   // 16 KB
// Each operand has a 96 KB ring of stages.  A stage carries TPS occupied K
// tiles (a kernel template parameter): 2 tiles in 3 stages of 32 KB, or 3
// tiles in 2 stages of 48 KB (a third fewer hand-offs per MMA, one stage
// less in flight).  The SDDMM runs 3 stages of one 32 KB box per operand.
constexpr int kRingBytes = 96 * 1024;
constexpr int kMaxStages = 3;
// Producers: one group of 256 threads (one per row of the CTA tile) per tile
// of the stage, so a warp expands one tile per stage; then a TMA warp and an
// MMA warp (allocates TMEM, issues the MMAs).
constexpr int kGroupThreads = kCtaM;
constexpr __host__ __device__ int tc_threads(int tps) { return kGroupThreads * tps + 64; }
constexpr int kWordAhead = 4;                 // A words are loaded this many stages ahead
// Occupied K tiles of the CTA, listed once in shared memory: tile index in
// bits 0-27, which 128-row halves have bits in bits 28-29.
constexpr int kListMax = 4096;
constexpr uint32_t kTmemCols = 512;       // two 128x256 FP32 accumulators
// Epilogue staging: a warp's 32 rows x 32 columns of FP32 in the idle stage
// memory, rows 36 floats apart (16-byte aligned; the row-wise float4 writes
// and the column-block float4 reads are both free of bank conflicts).
constexpr int kEpiStride = 36;
constexpr int kEpiWarps = 16;  // 4 TMEM lane quarters x 2 accumulators x 2 column halves
using tc::kLbo;
using tc::kSbo;
using tc::kLayoutSw128;
constexpr int kFwd = 0, kTrans = 1, kSddmm = 2, kBatch = 3, kBatchT = 4, kBatchS = 5;
// kBatch / kBatchT / kBatchS: the forward product, Aᵀ·G and the SDDMM of a
// batch, CTA b running work item b with its problem's record
__host__ __device__ constexpr bool batched_mode(int m) { return m == kBatch || m == kBatchT || m == kBatchS; }
__host__ __device__ constexpr bool trans_mode(int m) { return m == kTrans || m == kBatchT; }
__host__ __device__ constexpr bool sddmm_mode(int m) { return m == kSddmm || m == kBatchS; }
// B (fwd) / G (trans) tile: four TMA boxes of 64 columns x 32 reduction rows,
// 128-byte swizzle, kBox bytes apart (the LBO); 8-row groups 1 KB apart (SBO).
constexpr int kBoxCols = 64;
constexpr uint32_t kBox = kBoxCols * kTcK * 2;  // 4 KB
// SDDMM: a stage is 64 columns of N: the G tile (256 rows) and the X tile
// (256 rows) are one box each, K-major with 128-byte swizzle (rows 128 B,
// 8-row groups 1 KB apart); the four K=16 steps start 32 B apart.
constexpr int kSdK = 64;
constexpr int kSdTile = kCtaM * kSdK * 2;  // one G or X box of a stage: 32 KB
constexpr uint32_t kSdSbo = 1024;
// Shared memory is requested with this much slack so the stage buffers can
// be aligned to the 1 KB swizzle atom.
constexpr size_t kSmemAlign = 1024;

struct __align__(1024) TcSmem {
  uint8_t a[kRingBytes];  // stage s at s * stage bytes
  uint8_t b[kRingBytes];
  int list[kListMax];
  int nlist, seen, lo;
  uint64_t full[kMaxStages];   // producer warps + the TMA transaction arrival
  uint64_t empty[kMaxStages];  // tcgen05.commit of the stage's MMAs
  uint64_t done;
  uint32_t tmem_addr;
  int abort;
};


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
  // split-K (gridDim.z > 1): CTA z sums list slice z into part + z*part_stride
  // (row stride ldp); a reduction kernel adds the slices into C
  float* part;
  int64_t ldp, part_stride;
  // fwd / trans: B (or G) already in shared-memory order (k_tile_b), one
  // 16 KB block per (32-row tile, 256-column block), bt_cb blocks per tile
  // row; nullptr = B by TMA tensor boxes
  const uint8_t* bt;
  int64_t bt_cb;
  // batched form (kBatch): CTA b runs work item b of the batch
  const BatchProblemTc* bprobs;
  // fwd / trans: A's words column by column ([Kw][M]) for coalesced loads, or null
  const uint32_t* At;
  const int4* items;  // {problem, 256-row block, 256-column block, K tiles}
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
template <typename BT, int MODE, int TPS>
__global__ void __launch_bounds__(tc_threads(TPS), 1) k_spmm_tc(TcArgs a, const __grid_constant__ CUtensorMap mapA,
                                                               const __grid_constant__ CUtensorMap mapB) {
  constexpr int kTilesPerStage = TPS;
  constexpr bool kSd = sddmm_mode(MODE), kTr = trans_mode(MODE), kBat = batched_mode(MODE);
  constexpr int kStageBytes = kSd ? kSdTile : TPS * kATile;
  constexpr int kStages = kRingBytes / kStageBytes;
  constexpr int kProducerWarps = kGroupThreads * TPS / 32;
  constexpr int kTmaWarp = kProducerWarps;
  constexpr int kMmaWarp = kProducerWarps + 1;
  static_assert(kStages >= 2 && kStages <= kMaxStages, "stage ring");
  static_assert(kProducerWarps >= kEpiWarps, "the epilogue runs on producer warps");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(
      smem_raw + ((kSmemAlign - (ptx::smem_addr(smem_raw) & (kSmemAlign - 1))) & (kSmemAlign - 1)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr bool kFwdLike = MODE == kFwd || MODE == kBatch;
  // the CTA's problem: the launch's (fwd / trans / sddmm) or its work item's (batch)
  const uint32_t* gA = a.A;
  int64_t gM = a.M, gK = a.K, gKw = a.Kw, gldc = a.ldc;
  float* gC = a.C;
  const void* bmap = &mapB;
  const void* amap = &mapA;
  int64_t row0 = (int64_t)blockIdx.x * kCtaM;  // output rows: M (fwd, sddmm) or K (trans)
  int64_t col0 = (int64_t)blockIdx.y * kTcN;   // output columns: N (fwd, trans) or K (sddmm)
  if (kBat) {
    const int4 it = a.items[blockIdx.x];
    const BatchProblemTc& p = a.bprobs[it.x];
    gA = p.A;
    gM = p.M;
    gK = p.K;
    gKw = p.Kw;
    gC = p.C;
    gldc = p.ldc;
    bmap = kSd ? &p.map2 : &p.map;  // SDDMM: X [K][N] (the B side), G [M][N] (the A side)
    amap = &p.map;
    row0 = (int64_t)it.y * kCtaM;
    col0 = (int64_t)it.z * kTcN;
  }
  const int64_t out_rows = kTr ? gK : gM;
  const int64_t out_cols = kSd ? gK : a.N;
  // B boxes (64 columns) holding output columns of this CTA: a narrow last
  // column tile loads, multiplies and stores only those (MMA N = 64·nbox)
  const int nbox = kSd ? kTcN / kBoxCols
                                  : (int)min((int64_t)(kTcN / kBoxCols), (out_cols - col0 + kBoxCols - 1) / kBoxCols);
  const int dense_halves = row0 + kTcM < out_rows ? 3 : 1;

  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      // one arrival per producer warp + the TMA warp's (SDDMM: TMA only)
      ptx::mbar_init(&sm.full[s], kSd ? 1 : kProducerWarps + 1);
      ptx::mbar_init(&sm.empty[s], 1);
    }
    ptx::mbar_init(&sm.done, 1);
    sm.abort = 0;
    ptx::fence_mbar_init();
  }
  if (warp == kMmaWarp) {
    ptx::tmem_alloc(&sm.tmem_addr, kTmemCols);
    ptx::tmem_relinquish();
  }
  if ((MODE == kBatch || MODE == kBatchT) && warp == 0) {
    // every reduction tile (a batch has no occupancy plan): K tiles of the
    // forward product, 32-row tiles of A for Aᵀ·G; both halves that hold rows
    const int64_t red = MODE == kBatch ? gKw : (gM + kTcK - 1) / kTcK;
    const int ntot = (int)min(red, (int64_t)kListMax);
    for (int k = lane; k < ntot; k += 32) sm.list[k] = k | (dense_halves << 28);
    __syncwarp();
    if (lane == 0) {
      sm.lo = 0;
      sm.nlist = ntot;
      sm.seen = ntot > 0 ? dense_halves : 0;
    }
  }
  if ((MODE == kFwd || MODE == kTrans) && warp == 0) {
    // List the occupied K tiles of the two 128-row blocks (ascending), with
    // the halves that have bits in each; the launcher guarantees that the
    // list fits (at most kListMax reduction tiles).
    const int nblk = (int)((out_rows + kTcM - 1) / kTcM);
    const uint32_t* occ0 = a.occ + (int64_t)blockIdx.x * kHalves * a.occ_words;
    const bool has1 = (int)blockIdx.x * kHalves + 1 < nblk;
    int n = 0;
    for (int ow0 = 0; ow0 < a.occ_words; ow0 += 32) {
      const int ow = ow0 + lane;
      const uint32_t b0 = ow < a.occ_words ? __ldg(occ0 + ow) : 0u;
      const uint32_t b1 = (has1 && ow < a.occ_words) ? __ldg(occ0 + a.occ_words + ow) : 0u;
      uint32_t bits = b0 | b1;
      const int c = __popc(bits);
      int incl = c;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += y;
      }
      int pos = n + incl - c;
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1;
        if (pos < kListMax)
          sm.list[pos] = (ow * 32 + b) | (int)((((b0 >> b) & 1u) | (((b1 >> b) & 1u) << 1)) << 28);
        pos++;
      }
      n += __shfl_sync(kFull, incl, 31);
    }
    // this CTA's slice of the list (all of it without split-K) and the
    // halves that slice touches
    __syncwarp();
    const int ntot = min(n, kListMax);
    const int lo = (int)((int64_t)ntot * blockIdx.z / gridDim.z);
    const int hi = (int)((int64_t)ntot * (blockIdx.z + 1) / gridDim.z);
    uint32_t hs = 0;
    for (int k = lo + lane; k < hi; k += 32) hs |= ((uint32_t)sm.list[k] >> 28) & 3u;
    hs = __reduce_or_sync(kFull, hs);
    if (lane == 0) {
      sm.lo = lo;
      sm.nlist = hi - lo;
      sm.seen = (int)hs;
    }
  }
  // SDDMM: a block of A without set bits needs no product at all
  if (kSd) {
    uint32_t acc = 0;
    if (tid < kCtaM && row0 + tid < gM) {
      const uint32_t* arow = gA + (row0 + tid) * gKw;
      for (int64_t w = col0 / 32; w < min(gKw, (col0 + kTcN) / 32); w++) acc |= __ldg(arow + w);
    }
    const int any = __syncthreads_or(acc != 0u);
    if (tid == 0) {
      sm.nlist = any ? (int)((a.N + kSdK - 1) / kSdK) : 0;  // steps of kSdK columns of N
      sm.seen = any ? dense_halves : 0;
      sm.lo = 0;
    }
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  ptx::tc_fence_after_sync();
  const uint32_t tmem = sm.tmem_addr;
  const int n = sm.nlist;
  const int* lst = sm.list + sm.lo;  // this CTA's occupied tiles (fwd / trans)
  // stage i: list entries 2i and 2i+1 (fwd / trans) or N columns [64i, 64i+64) (SDDMM)
  const int nstages = kSd ? n : (n + kTilesPerStage - 1) / kTilesPerStage;

  if (warp < kProducerWarps) {
    // ---------------- A producers (fwd / trans) ----------------
    // Group u (warps 8u..8u+7) expands tile u of every stage, one row (fwd)
    // or one (A row, word) pair (trans) per thread, from words loaded
    // kWordAhead stages ahead; each warp arrives once per stage after its
    // lanes' writes are fenced.  Lane 0 waits for the slot for the warp.
    if (!kSd) {
      const int u = warp / (kGroupThreads / 32);
      const int r = tid % kGroupThreads;
      auto load_word = [&](int k) -> uint32_t {
        if (k >= n) return 0u;
        const int t = lst[k] & 0x0fffffff;
        if (kFwdLike) {
          const int64_t arow = row0 + r;
          if (arow >= gM) return 0u;
          return (!kBat && a.At) ? __ldg(a.At + (int64_t)t * gM + arow) : __ldg(gA + arow * gKw + t);
        }
        const int64_t arow = (int64_t)t * kTcK + (r & 31);
        const int64_t wcol = row0 / 32 + (r >> 5);
        if (arow >= gM || wcol >= gKw) return 0u;
        return (!kBat && a.At) ? __ldg(a.At + wcol * gM + arow) : __ldg(gA + arow * gKw + wcol);
      };
      uint32_t wq[kWordAhead];
#pragma unroll
      for (int j = 0; j < kWordAhead; j++) wq[j] = load_word(kTilesPerStage * j + u);
      for (int i = 0; i < nstages; i++) {
        const int s = i % kStages;
        const uint32_t w0 = wq[0];
        const uint32_t wnew = load_word(kTilesPerStage * (i + kWordAhead) + u);
        // (no abort poll on this path: a role that gives up stops arriving,
        // and every other role's own bounded wait then ends its loop)
        int go = 1;
        if (lane == 0 && i >= kStages && !ptx::mbar_wait(&sm.empty[s], ((i / kStages) - 1) & 1)) {
          atomicCAS(&g_tc_error, 0, 3);
          sm.abort = 1;
          go = 0;
        }
        if (!__shfl_sync(kFull, go, 0)) break;
        if (kTilesPerStage * i + u < n) {
          uint8_t* at = sm.a + s * kStageBytes + u * kATile;
          uint4 e[4];
          tc::expand32_two(w0, e);
          if (kFwdLike) {
            // row r of the tile: half r/128 at 8 KB, then core matrices
            uint8_t* as = at + (r >> 3) * kSbo + (r & 7) * 16;
#pragma unroll
            for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(as + c * kLbo) = e[c];
          } else {
            // A row j of the tile, word wk of the block: output rows wk*32 + 8c ..
            const int j = r & 31, wk = r >> 5;
            uint8_t* as = at + (j >> 3) * kLbo + (j & 7) * 16;
#pragma unroll
            for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(as + (wk * 4 + c) * kSbo) = e[c];
          }
        }
        ptx::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&sm.full[s]);
#pragma unroll
        for (int j = 0; j < kWordAhead - 1; j++) wq[j] = wq[j + 1];
        wq[kWordAhead - 1] = wnew;
      }
    }
  } else if (warp == kTmaWarp && lane == 0) {
    // ---------------- TMA issuer ----------------
    // Shared-memory addresses are formed once; a stage adds its offset.
    const uint32_t a0 = ptx::smem_addr(sm.a), b0 = ptx::smem_addr(sm.b), f0 = ptx::smem_addr(&sm.full[0]);
    if (kBat) {  // written by the host into global memory
      ptx::tensormap_acquire(bmap);
      if (kSd) ptx::tensormap_acquire(amap);
    }
    for (int i = 0; i < nstages; i++) {
      const int s = i % kStages;
      if (i >= kStages && !ptx::mbar_wait(&sm.empty[s], ((i / kStages) - 1) & 1)) {
        atomicCAS(&g_tc_error, 0, 3);
        sm.abort = 1;
        break;
      }
      const uint32_t fb = f0 + s * 8, as = a0 + s * kStageBytes, bs = b0 + s * kStageBytes;
      if (kSd) {
        // G rows row0.. and X rows col0.. (256 each), N columns i*64..
        ptx::mbar_arrive_expect_tx(&sm.full[s], 2 * kSdTile);
        ptx::tma_load_2d_u32(as, amap, i * kSdK, (int)row0, fb);
        ptx::tma_load_2d_u32(bs, bmap, i * kSdK, (int)col0, fb);
      } else {
        // B (fwd) / G (trans) rows t*32.. of the stage's tiles, columns col0 + 64*j
        const int k0 = kTilesPerStage * i;
        const int cnt = min(kTilesPerStage, n - k0);  // tiles in this stage
        ptx::mbar_arrive_expect_tx(&sm.full[s], cnt * nbox * kBox);
        if (!kBat && a.bt) {
          // tiled B: each tile's first nbox atoms are one contiguous copy
#pragma unroll
          for (int u = 0; u < kTilesPerStage; u++)
            if (u < cnt)
              ptx::bulk_g2s(sm.b + s * kStageBytes + u * kBTile,
                            a.bt + ((int64_t)(lst[k0 + u] & 0x0fffffff) * a.bt_cb + blockIdx.y) * kBTile,
                            nbox * kBox, &sm.full[s]);
          continue;
        }
#pragma unroll
        for (int u = 0; u < kTilesPerStage; u++) {
          if (u >= cnt) break;
          const int t = lst[k0 + u] & 0x0fffffff;
#pragma unroll
          for (int j = 0; j < kTcN / kBoxCols; j++)
            if (j < nbox)
              ptx::tma_load_2d_u32(bs + u * kBTile + j * kBox, bmap, (int)col0 + j * kBoxCols, t * kTcK, fb);
        }
      }
    }
  } else if (warp == kMmaWarp && lane == 0) {
    // ---------------- MMA issuer ----------------
    // Descriptors of stage 0 are built once; every MMA adds a compile-time
    // offset (plus the stage's) to the 14-bit start-address field (>> 4).
    const uint32_t ab = std::is_same<BT, __nv_bfloat16>::value ? 1u : 0u;
    const uint32_t idesc = tc::idesc_f16(ab, kTr ? 1u : 0u, kSd ? 0u : 1u,
                                         (uint32_t)(nbox * kBoxCols), kTcM);
    const uint32_t a0 = ptx::smem_addr(sm.a), b0 = ptx::smem_addr(sm.b);
    const uint64_t adesc = kSd ? ptx::smem_desc_noswizzle_u32(a0, 16, kSdSbo) | ((uint64_t)kLayoutSw128 << 61)
                                          : ptx::smem_desc_noswizzle_u32(a0, kLbo, kSbo);
    const uint64_t bdesc = kSd ? ptx::smem_desc_noswizzle_u32(b0, 16, kSdSbo) | ((uint64_t)kLayoutSw128 << 61)
                                          : ptx::smem_desc_noswizzle_u32(b0, kBox, 1024) | ((uint64_t)kLayoutSw128 << 61);
    // The tensor pipe queues about one MMA beyond the one it runs, so every
    // cycle this thread spends between stages is idle tensor time: the next
    // stage's halves are read from the list while this stage issues, and the
    // abort flag is not polled here either.
    auto halves = [&](int st, int (&hv)[kTilesPerStage]) {
#pragma unroll
      for (int u = 0; u < kTilesPerStage; u++) {
        const int k = kTilesPerStage * st + u;
        hv[u] = kSd ? (u == 0 ? dense_halves : 0)
                               : (st < nstages && k < n ? (lst[k] >> 28) & 3 : 0);
      }
    };
    uint32_t started = 0;
    int i = 0;
    int hn[kTilesPerStage];
    halves(0, hn);
    for (; i < nstages; i++) {
      const int s = i % kStages;
      int hv[kTilesPerStage];
#pragma unroll
      for (int u = 0; u < kTilesPerStage; u++) hv[u] = hn[u];
      halves(i + 1, hn);
      const int hv0 = hv[0];
      if (!ptx::mbar_wait(&sm.full[s], (i / kStages) & 1)) {
        atomicCAS(&g_tc_error, 0, 3);
        sm.abort = 1;
        break;
      }
      ptx::tc_fence_after_sync();
      const uint64_t soff = (uint64_t)((s * kStageBytes) >> 4);
      const uint64_t as = adesc + soff, bs = bdesc + soff;
      if (kSd) {
#pragma unroll
        for (int h = 0; h < kHalves; h++) {
          if (!((hv0 >> h) & 1)) continue;
#pragma unroll
          for (int j = 0; j < kSdK / 16; j++)  // K step j starts 32 B into the 128-byte rows
            ptx::tc_mma_f16(tmem + (uint32_t)(h * kTcN), as + (uint64_t)((h * kTcM * 128 + j * 32) >> 4),
                            bs + (uint64_t)((j * 32) >> 4), idesc, ((started >> h) & 1u) || j > 0);
          started |= 1u << h;
        }
      } else {
#pragma unroll
        for (int u = 0; u < kTilesPerStage; u++) {
          const int hu = hv[u];
#pragma unroll
          for (int h = 0; h < kHalves; h++) {
            if (!((hu >> h) & 1)) continue;
#pragma unroll
            for (int j = 0; j < 2; j++)  // K half j: A two core-matrix columns on, B two 8-row groups on
              ptx::tc_mma_f16(tmem + (uint32_t)(h * kTcN),
                              as + (uint64_t)((u * kATile + h * kAHalf + j * 2 * kLbo) >> 4),
                              bs + (uint64_t)((u * kBTile + j * 2 * 1024) >> 4), idesc, ((started >> h) & 1u) || j > 0);
            started |= 1u << h;
          }
        }
      }
      ptx::tc_commit(&sm.empty[s]);
    }
    if (i > 0) ptx::tc_commit(&sm.done);
    else ptx::mbar_arrive(&sm.done);
  }

  // ---------------- epilogue (producer warps) ----------------
  // Warp w reads TMEM lanes 32*(w%4).. (a warp may only touch its own
  // quarter of the lanes) of accumulator (w/4)%2, column half w/8 of the
  // tile's 64·nbox live columns (so a narrow tile keeps all 16 warps busy);
  // a thread holds 32 columns of one output row at a time and passes them
  // through a 32x32 tile of the (now idle) stage memory, so that each store
  // instruction writes four whole 128-byte rows of C instead of 16 bytes in
  // each of 32 rows.  The SDDMM first keeps only the set bits of A's row,
  // from the row's four words loaded once.
  if (warp < kEpiWarps) {
    const int h = (warp >> 2) & 1, q = warp & 3, cg = warp >> 3;
    const bool have = (sm.seen >> h) & 1;
    // warp-uniform flags: the TMEM loads and the tile hand-off below are
    // collective over the warp
    const bool ok = __all_sync(kFull, ptx::mbar_wait(&sm.done, 0));
    if (!ok && lane == 0) {
      atomicCAS(&g_tc_error, 0, 3);
      sm.abort = 1;
    }
    ptx::tc_fence_after_sync();
    const bool wlive = __all_sync(kFull, ok && !*(volatile int*)&sm.abort);
    const int64_t rbase = row0 + h * kTcM + q * 32;  // the warp's first row
    const int64_t row = rbase + lane;
    const bool split = gridDim.z > 1;
    float* cbase = split ? a.part + (int64_t)blockIdx.z * a.part_stride : gC;
    const int64_t cld = split ? a.ldp : gldc;
    const int cspan = nbox * (kBoxCols / 2);      // live columns per column half (a multiple of 32)
    const int64_t ccol = col0 + cg * cspan;         // the warp's first column
    const bool live = row < out_rows && wlive;
    const uint32_t* arow = gA + row * gKw;
    const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * kTcN + cg * cspan);
    float* tile = reinterpret_cast<float*>(sm.a) + warp * 32 * kEpiStride;
    const int c8_end = cspan / 8;
    // SDDMM: the row's A words of this warp's columns (cspan = 128: four
    // words), loaded once before the stores instead of once per 32 columns
    uint32_t aw[4] = {0u, 0u, 0u, 0u};
    if (kSd && live) {
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int64_t w = ccol / 32 + i;
        if (i * 32 < cspan && w < gKw) aw[i] = __ldg(arow + w);
      }
    }
    for (int c8 = 0; c8 < c8_end; c8 += 4) {
      uint32_t r[4][8];
      if (have && ok) {
#pragma unroll
        for (int u = 0; u < 4; u++) ptx::tmem_ld_32x32b_x8(tbase + (uint32_t)((c8 + u) * 8), r[u]);
        ptx::tmem_wait_ld();
      } else {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int v = 0; v < 8; v++) r[u][v] = 0u;
      }
      if (kSd) {
        // keep the set bits of A's row only (the row's word of these 32 columns)
        const uint32_t wbits = aw[(c8 / 4) & 3];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int v = 0; v < 8; v++)
            if (!((wbits >> (u * 8 + v)) & 1u)) r[u][v] = 0u;
      }
      if (!wlive) continue;
      // the bit operand held 2.0 per set bit (the SDDMM's operands are both
      // dense: no scale); row `lane` of the tile
      constexpr float kScale = kSd ? 1.0f : tc::kTwoScale;
#pragma unroll
      for (int u = 0; u < 4; u++) {
        float4* t4 = reinterpret_cast<float4*>(tile + lane * kEpiStride + u * 8);
        t4[0] = make_float4(__uint_as_float(r[u][0]) * kScale, __uint_as_float(r[u][1]) * kScale,
                            __uint_as_float(r[u][2]) * kScale, __uint_as_float(r[u][3]) * kScale);
        t4[1] = make_float4(__uint_as_float(r[u][4]) * kScale, __uint_as_float(r[u][5]) * kScale,
                            __uint_as_float(r[u][6]) * kScale, __uint_as_float(r[u][7]) * kScale);
      }
      __syncwarp();
      // 8 lanes per row: rows 4*it + lane/8, 16 bytes each
      const int c4 = (lane & 7) * 4;
      const int64_t gcol = ccol + c8 * 8 + c4;
#pragma unroll
      for (int it = 0; it < 8; it++) {
        const int j = it * 4 + (lane >> 3);
        const int64_t grow = rbase + j;
        if (grow < out_rows && gcol < out_cols)
          *reinterpret_cast<float4*>(cbase + grow * cld + gcol) =
              *reinterpret_cast<const float4*>(tile + j * kEpiStride + c4);
      }
      __syncwarp();
    }
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  if (warp == kMmaWarp) {
    ptx::tc_fence_after_sync();
    ptx::tmem_dealloc(tmem, kTmemCols);
  }
}

// B (fwd) or G (trans) [R][N] of 16-bit values -> the shared-memory order
// of the tensor-core kernel's B stage, so that a tile arrives by one
// contiguous bulk copy instead of four tensor boxes of 32 rows: block (t, cb)
// (16 KB, t = 32-row tile, cb = 256-column block) holds four 64-column atoms
// of 4 KB; in atom j, row r occupies 128 bytes whose 16-byte chunk c sits at
// position c ^ (r % 8) (the 128-byte swizzle, as a TMA load into a
// 1024-byte aligned stage writes it).  Rows past R and columns past N are
// zero.  One thread per 16-byte chunk: a warp reads 512 contiguous bytes of
// one row and writes four 128-byte runs.
__global__ void __launch_bounds__(256) k_tile_b(const uint8_t* __restrict__ B, int64_t R, int64_t N, int64_t ldb,
                                                int64_t ntiles, int64_t ncb, uint4* __restrict__ bt) {
  const int64_t total = ntiles * ncb * (kBTile / 16);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t blk = e >> 10;
    const int in = (int)(e & 1023);
    const int r = in >> 5, j = (in >> 3) & 3, c = in & 7;
    const int64_t t = blk / ncb, cb = blk - t * ncb;
    const int64_t row = t * kTcK + r, col = cb * kTcN + j * kBoxCols + c * 8;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (row < R && col < N) v = __ldg(reinterpret_cast<const uint4*>(B + (row * ldb + col) * 2));
    bt[blk * 1024 + j * 256 + r * 8 + (c ^ (r & 7))] = v;
  }
}

// Both occupancy bitmaps in one pass over A's words.  A block of 4 warps
// covers 128 rows x 32 word columns: thread (warp j, lane l) ORs the 32 rows
// of row tile 4·blockIdx.y + j in word column 32·blockIdx.x + l (coalesced
// across the lanes).  Forward: the OR of the 4 warps is the (128-row block,
// K tile) bit, and the 32 lanes' bits are one occupancy word (one ballot).
// Transposed: the OR of 4 neighbouring lanes is the (row tile, 128-column
// block) bit of Aᵀ's bitmap, set with atomicOr (the bitmap is zeroed first;
// a bit that was not yet set is counted).
__global__ void __launch_bounds__(128) k_occupancy_both(const uint32_t* __restrict__ A, int64_t M, int64_t Kw,
                                                        int ow, uint32_t* __restrict__ occ, int owt, int64_t nkb,
                                                        uint32_t* __restrict__ occT, unsigned long long* count,
                                                        unsigned long long* countT) {
  __shared__ uint32_t s_or[4][32];
  const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
  const int64_t w = (int64_t)blockIdx.x * 32 + lane;
  const int64_t rb = blockIdx.y, rt = rb * 4 + j;
  uint32_t acc = 0;
  if (w < Kw) {
    const int64_t r0 = rt * 32, r1 = min(M, r0 + 32);
    for (int64_t r = r0; r < r1; r++) acc |= __ldg(A + r * Kw + w);
  }
  s_or[j][lane] = acc;
  // transposed bitmap: 8 column blocks of 4 words per warp
  uint32_t g = acc | __shfl_xor_sync(kFull, acc, 1);
  g |= __shfl_xor_sync(kFull, g, 2);
  const int64_t kb = w >> 2;
  if ((lane & 3) == 0 && g != 0u && kb < nkb && rt * 32 < M) {
    const uint32_t bit = 1u << (rt & 31);
    const uint32_t old = atomicOr(occT + kb * owt + (rt >> 5), bit);
    if (countT && !(old & bit)) atomicAdd(countT, 1ull);
  }
  __syncthreads();
  if (j == 0) {
    const uint32_t v = s_or[0][lane] | s_or[1][lane] | s_or[2][lane] | s_or[3][lane];
    const uint32_t m = __ballot_sync(kFull, v != 0u);
    if (lane == 0) {
      occ[rb * ow + blockIdx.x] = m;
      if (count && m) atomicAdd(count, (unsigned long long)__popc(m));
    }
  }
}

}  // namespace

int tc_occupancy_words(int64_t K) { return (int)ceil_div(ceil_div(K, 32), 32); }
int64_t tc_max_reduction() { return (int64_t)kListMax * kTcK; }
int tc_occupancy_t_words(int64_t M) { return (int)ceil_div(ceil_div(M, 32), 32); }

// words [M][Kw] -> At [Kw][M] through 32x32 shared-memory tiles (coalesced
// on both sides).
__global__ void __launch_bounds__(256) k_transpose_words(const uint32_t* __restrict__ w, int64_t M, int64_t Kw,
                                                         uint32_t* __restrict__ At) {
  __shared__ uint32_t tile[32][33];
  const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r0 + k, c = c0 + tx;
    tile[k][tx] = (r < M && c < Kw) ? __ldg(w + r * Kw + c) : 0u;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int64_t c = c0 + k, r = r0 + tx;
    if (c < Kw && r < M) At[c * M + r] = tile[tx][k];
  }
}

int launch_transpose_words(const uint32_t* words, int64_t M, int64_t Kw, uint32_t* At, cudaStream_t s) {
  if (M == 0 || Kw == 0) return BSP_OK;
  if (ceil_div(M, 32) > 65535) return BSP_ERR_CAPACITY;
  k_transpose_words<<<dim3((unsigned)ceil_div(Kw, 32), (unsigned)ceil_div(M, 32)), 256, 0, s>>>(words, M, Kw, At);
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_occupancy(const uint32_t* A, int64_t M, int64_t K, uint32_t* occ, uint32_t* occT,
                     unsigned long long* count, unsigned long long* countT, cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32);
  const int ow = tc_occupancy_words(K), owt = tc_occupancy_t_words(M);
  const int64_t nkb = ceil_div(K, kTcM), nrb = ceil_div(M, kTcM);
  if (M == 0 || K == 0) return BSP_OK;
  if (nrb > 65535) return BSP_ERR_CAPACITY;
  BSP_CUDA(cudaMemsetAsync(occT, 0, sizeof(uint32_t) * (size_t)nkb * owt, s));
  k_occupancy_both<<<dim3((unsigned)ow, (unsigned)nrb), 128, 0, s>>>(A, M, Kw, ow, occ, owt, nkb, occT, count,
                                                                      countT);
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

static_assert(sizeof(TcSmem) + kSmemAlign <= 232448, "stage ring exceeds the shared memory of a CTA");
static_assert(kEpiWarps * 32 * kEpiStride * (int)sizeof(float) <= kRingBytes,
              "epilogue tiles exceed the stage memory");

template <typename BT, int MODE, int TPS>
int launch_mode(const TcArgs& a, const CUtensorMap& ma, const CUtensorMap& mb, dim3 grid, cudaStream_t s) {
  const size_t smem = sizeof(TcSmem) + kSmemAlign;
  static bool configured[64] = {};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(k_spmm_tc<BT, MODE, TPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured[dev] = true;
  }
  k_spmm_tc<BT, MODE, TPS><<<grid, tc_threads(TPS), smem, s>>>(a, ma, mb);
  BSP_LAUNCHED();
  return BSP_OK;
}

// C = Σ_z part[z] in ascending z (deterministic), four columns per thread
// (the tensor-core path needs N % 8 == 0 and 16-byte aligned C rows).
__global__ void __launch_bounds__(256) k_split_reduce(const float* __restrict__ part, int64_t ldp, int64_t stride,
                                                      int splits, int64_t rows, int64_t cols, float* __restrict__ C,
                                                      int64_t ldc) {
  const int64_t q = cols / 4, total = rows * q;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / q, c = (e - r * q) * 4;
    float4 acc = __ldg(reinterpret_cast<const float4*>(part + r * ldp + c));
    for (int z = 1; z < splits; z++) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(part + z * stride + r * ldp + c));
      acc.x += v.x;
      acc.y += v.y;
      acc.z += v.z;
      acc.w += v.w;
    }
    *reinterpret_cast<float4*>(C + r * ldc + c) = acc;
  }
}

}  // namespace

// Split-K for the tensor-core products: when the output has fewer CTA tiles
// than half the SMs, the reduction (list of occupied tiles) is cut into S
// slices, up to 8 and at least 16 reduction tiles each, so that about one CTA
// per SM runs; every slice's FP32 partial needs rows x round4(cols) floats.
int tc_split_count(int64_t out_rows, int64_t out_cols, int64_t red_tiles) {
  const int64_t tiles = ceil_div(out_rows, kCtaM) * ceil_div(out_cols, kTcN);
  const int64_t sms = num_sms();
  if (tiles == 0 || tiles * 2 > sms) return 1;
  int64_t S = sms / tiles;
  if (S > 8) S = 8;
  if (S > red_tiles / 16) S = red_tiles / 16;
  return S < 1 ? 1 : (int)S;
}

size_t tc_split_bytes(int64_t out_rows, int64_t out_cols, int64_t red_tiles) {
  const int S = tc_split_count(out_rows, out_cols, red_tiles);
  return S > 1 ? (size_t)S * (size_t)out_rows * (size_t)(ceil_div(out_cols, 4) * 4) * sizeof(float) + 256 : 0;
}

// B (or G) in tile order: every (32-row tile, 256-column block) is 16 KB.
size_t tc_tiled_b_bytes(int64_t red_rows, int64_t cols) {
  return (size_t)ceil_div(red_rows, kTcK) * (size_t)ceil_div(cols, kTcN) * kBTile + 1024;
}

// Tiling B costs a read and a write of it; it pays where many row blocks
// read every B tile (measured on GB300: 16384 rows, 64 blocks, 0.84 -> 0.80
// ms; 4096 rows, 16 blocks, forward + backward 0.76 -> 0.79 ms).
constexpr int64_t kTiledMinRowBlocks = 32;

bool tc_tiles_b(int64_t out_rows) { return ceil_div(out_rows, kCtaM) >= kTiledMinRowBlocks; }

size_t tc_preferred_bytes(int64_t out_rows, int64_t out_cols, int64_t red_rows) {
  return tc_split_bytes(out_rows, out_cols, ceil_div(red_rows, kTcK)) +
         (tc_tiles_b(out_rows) ? tc_tiled_b_bytes(red_rows, out_cols) : 0);
}

namespace {

// Three K tiles per stage (two stages) where the output has this many row
// blocks; BSP_TC_TPS=2 or 3 forces one form.
constexpr int64_t kThreeTileMinRowBlocks = 32;
bool three_tiles(int64_t out_rows) {
  static const int force = [] {
    const char* e = getenv("BSP_TC_TPS");
    return e && *e ? atoi(e) : 0;
  }();
  if (force == 2 || force == 3) return force == 3;
  return ceil_div(out_rows, kCtaM) >= kThreeTileMinRowBlocks;
}

// BSP_TC_TILED_B=0 keeps B on tensor boxes even with room for the tiled copy.
bool tiled_b_enabled() {
  static const bool on = [] {
    const char* e = getenv("BSP_TC_TILED_B");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <int MODE>
int launch_tc(TcArgs a, cudaStream_t s, void* ws = nullptr, size_t ws_bytes = 0, TcForm form = TcForm{}) {
  const int64_t rows = MODE == kTrans ? a.K : a.M;
  const int64_t cols = MODE == kSddmm ? a.K : a.N;
  if (rows == 0 || cols == 0) return BSP_OK;
  int splits = 1;
  size_t used = 0;
  if (MODE != kSddmm && ws && form.split != 0) {
    const int64_t red_tiles = ceil_div(MODE == kFwd ? a.K : a.M, kTcK);
    const int S = tc_split_count(rows, cols, red_tiles);
    if (S > 1 && ws_bytes >= tc_split_bytes(rows, cols, red_tiles)) {
      splits = S;
      a.part = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
      a.ldp = ceil_div(cols, 4) * 4;
      a.part_stride = rows * a.ldp;
      used = tc_split_bytes(rows, cols, red_tiles);
    }
  }
  // B in tile order when the rest of the workspace holds it (else tensor boxes)
  const int64_t red_rows = MODE == kFwd ? a.K : a.M;
  const bool room = MODE != kSddmm && ws && ws_bytes >= used + tc_tiled_b_bytes(red_rows, cols);
  const bool tiled = room && (form.tiled >= 0 ? form.tiled == 1 : tc_tiles_b(rows) && tiled_b_enabled());
  const dim3 grid((unsigned)ceil_div(rows, kCtaM), (unsigned)ceil_div(cols, kTcN), (unsigned)splits);
  if (ceil_div(cols, kTcN) > 65535 || ceil_div(rows, kCtaM) > 0x7fffffff) return BSP_ERR_CAPACITY;
  if (a.N > INT32_MAX || a.M > INT32_MAX || a.K > INT32_MAX) return BSP_ERR_CAPACITY;
  // the tile list of a CTA holds every reduction tile (fwd: K, trans: M)
  if (MODE != kSddmm && ceil_div(MODE == kFwd ? a.K : a.M, kTcK) > kListMax) return BSP_ERR_CAPACITY;
  CUtensorMap ma, mb;
  memset(&ma, 0, sizeof(ma));
  if (MODE == kSddmm) {
    BSP_TRY(make_map(&ma, a.G, a.bdt, a.M, a.N, a.ldg, kSdK, kCtaM, CU_TENSOR_MAP_SWIZZLE_128B));  // G [M][N]
    BSP_TRY(make_map(&mb, a.B, a.bdt, a.K, a.N, a.ldb, kSdK, kTcN, CU_TENSOR_MAP_SWIZZLE_128B));   // X [K][N]
  } else {
    // B [K][N] (fwd) or G [M][N] (trans), 64 columns x 32 reduction rows per box
    BSP_TRY(make_map(&mb, a.B, a.bdt, MODE == kFwd ? a.K : a.M, a.N, a.ldb, kBoxCols, kTcK,
                     CU_TENSOR_MAP_SWIZZLE_128B));
  }
  if (tiled) {
    const int64_t ntiles = ceil_div(red_rows, kTcK), ncb = ceil_div(cols, kTcN);
    uint8_t* bt = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(static_cast<char*>(ws) + used) + 1023) & ~(uintptr_t)1023);
    const int64_t work = ntiles * ncb * (kBTile / 16);
    const int64_t cap = (int64_t)num_sms() * 16;
    k_tile_b<<<(unsigned)(ceil_div(work, 256) < cap ? ceil_div(work, 256) : cap), 256, 0, s>>>(
        static_cast<const uint8_t*>(a.B), red_rows, cols, a.ldb, ntiles, ncb, reinterpret_cast<uint4*>(bt));
    BSP_LAUNCHED();
    a.bt = bt;
    a.bt_cb = ncb;
  }
  if (a.bdt != BSP_BF16 && a.bdt != BSP_F16) return BSP_ERR_UNSUPPORTED;
  bool launched = false;
  if constexpr (MODE != kSddmm) {  // (the SDDMM has one stage form)
    if (form.tps ? form.tps == 3 : three_tiles(rows)) {
      if (a.bdt == BSP_BF16) BSP_TRY((launch_mode<__nv_bfloat16, MODE, 3>(a, ma, mb, grid, s)));
      else BSP_TRY((launch_mode<__half, MODE, 3>(a, ma, mb, grid, s)));
      launched = true;
    }
  }
  if (!launched) {
    if (a.bdt == BSP_BF16) BSP_TRY((launch_mode<__nv_bfloat16, MODE, 2>(a, ma, mb, grid, s)));
    else BSP_TRY((launch_mode<__half, MODE, 2>(a, ma, mb, grid, s)));
  }
  if (splits > 1) {
    const int64_t work = rows * (cols / 4);
    const int64_t cap = (int64_t)num_sms() * 8;
    k_split_reduce<<<(unsigned)(ceil_div(work, 256) < cap ? ceil_div(work, 256) : cap), 256, 0, s>>>(
        a.part, a.ldp, a.part_stride, splits, rows, cols, a.C, a.ldc);
    BSP_LAUNCHED();
  }
  return BSP_OK;
}
}  // namespace

int launch_spmm_tc(const SpmmArgs& sa, const uint32_t* occ, const uint32_t* At, cudaStream_t s, void* ws,
                   size_t ws_bytes, TcForm form) {
  TcArgs a = {};
  a.At = At;
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
  return launch_tc<kFwd>(a, s, ws, ws_bytes, form);
}

int launch_spmm_t_tc(const uint32_t* A, int64_t M, int64_t K, const void* G, int gdt, int64_t ldg, int64_t N,
                     float* dX, int64_t lddx, const uint32_t* occT, const uint32_t* At, cudaStream_t s, void* ws,
                     size_t ws_bytes) {
  TcArgs a = {};
  a.At = At;
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
  return launch_tc<kTrans>(a, s, ws, ws_bytes);
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

int make_batch_map(CUtensorMap* m, const void* B, int bdt, int64_t K, int64_t N, int64_t ldb) {
  return make_map(m, B, bdt, K, N, ldb, kBoxCols, kTcK, CU_TENSOR_MAP_SWIZZLE_128B);
}

int make_batch_map_sddmm(CUtensorMap* m, const void* T, int bdt, int64_t rows, int64_t N, int64_t ld,
                         int box_rows) {
  return make_map(m, T, bdt, rows, N, ld, kSdK, (uint32_t)box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

int launch_batched_tc(const BatchProblemTc* probs, const int4* items, int n_items, int64_t N, int bdt,
                      cudaStream_t s, int kind) {
  if (n_items == 0 || N == 0) return BSP_OK;
  TcArgs a = {};
  a.N = N;
  a.bdt = bdt;
  a.bprobs = probs;
  a.items = items;
  CUtensorMap unused;
  memset(&unused, 0, sizeof(unused));
  const dim3 grid((unsigned)n_items, 1, 1);
  if (bdt != BSP_BF16 && bdt != BSP_F16) return BSP_ERR_UNSUPPORTED;
  const bool bf = bdt == BSP_BF16;
  switch (kind) {
    case 0: return bf ? launch_mode<__nv_bfloat16, kBatch, 2>(a, unused, unused, grid, s)
                      : launch_mode<__half, kBatch, 2>(a, unused, unused, grid, s);
    case 1: return bf ? launch_mode<__nv_bfloat16, kBatchT, 2>(a, unused, unused, grid, s)
                      : launch_mode<__half, kBatchT, 2>(a, unused, unused, grid, s);
    case 2: return bf ? launch_mode<__nv_bfloat16, kBatchS, 2>(a, unused, unused, grid, s)
                      : launch_mode<__half, kBatchS, 2>(a, unused, unused, grid, s);
    default: return BSP_ERR_INVALID_ARG;
  }
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
