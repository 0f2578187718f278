// spmm_batched.cu — many independent bitmap SpMMs in one tensor-core launch.
//
// A batch (bsp_batch_create) holds, in device memory, one record per problem
// (B's tensor map, encoded once on the host, and A, C, sizes), a work list
// with one item per (problem, 256-row block, 256-column block), sorted by
// reduction length, longest first, and a work-queue counter.
// bsp_batched_spmm runs the list in one launch, with no host synchronisation
// and no allocation: for N ≤ 128 with the persistent kernel below (a CTA
// per SM pulls items from the queue); for wider N with the tensor-core SpMM
// kernel in batch mode (spmm_tc.cu: one CTA per item).  Both read the item's
// problem from its record, run every K tile of its rows (a batch has no
// occupancy plan) and stream B by TMA through the problem's own tensor map.
#include <algorithm>
#include <new>
#include <type_traits>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bsp_internal.cuh"
#include "ptx.cuh"
#include "spmm.cuh"
#include "tc_common.cuh"

namespace bsp {

// Kept for bsp_device_status: the tensor-core kernel reports its own waits.
__device__ int g_batch_error;

int batched_device_error(int* out, bool clear) {
  BSP_CUDA(cudaMemcpyFromSymbol(out, g_batch_error, sizeof(int)));
  if (clear) {
    const int zero = 0;
    BSP_CUDA(cudaMemcpyToSymbol(g_batch_error, &zero, sizeof(int)));
  }
  return BSP_OK;
}

namespace {
constexpr int64_t kItemRows = 256, kItemCols = 256;  // the tensor-core kernel's CTA tile

// ---- persistent batched kernel (N ≤ 128) ----------------------------------
// One CTA per SM takes work items from a device-side queue (an atomic
// counter over the longest-first item list) until the list is exhausted.
// An item is 256 rows of one problem (two 128-row halves) times all N ≤ 128
// columns, reduced over every 32-column K tile of its rows.  Roles:
//   warps 0-7 (producers): thread r expands row r of both K tiles of a stage
//     (2.0 per set bit, K-major core matrices), words loaded 4 stages ahead;
//   warp 8 (TMA, lane 0): fetches the next item into a 4-slot ring in shared
//     memory for every role, then loads each stage's B rows as 64x32 boxes
//     (128-byte swizzle) through the problem's tensor map;
//   warp 9 (MMA, lane 0): allocates TMEM, issues tcgen05.mma (M128 N≤128
//     K16) into accumulator set j % 2 of item j and commits each stage to
//     its "empty" barrier and each item to "tfull";
//   warps 10-17 (epilogue): read set j % 2 back (warp w touches TMEM lanes
//     32·(w%4)..; warps 10-13 and 14-17 split the columns), scale by 0.5,
//     store C through a 32x32 staging tile per warp, then free the set
//     ("tempty") and the item's ring slot ("qempty").
// With two accumulator sets the epilogue of item j runs under the MMAs of
// item j+1, and the producers and TMA run up to three stages ahead across
// item boundaries, so an item costs its MMAs, not its set-up.  Stage and
// item counters run over the whole launch, so every mbarrier phase follows
// from a counter.  Every wait is bounded: on timeout the role records error
// 4 in g_batch_error and stops; the others' bounded waits then end.
constexpr int kPRows = 256, kPM = 128, kPK = 32, kPMaxN = 128;
constexpr int kPTps = 2, kPQ = 4;
constexpr int kPATile = kPRows * kPK * 2;  // 16 KB: both halves of one K tile
constexpr int kPAHalf = kPM * kPK * 2;     // 8 KB
constexpr int kPBox = 64 * kPK * 2;        // 4 KB: 64 columns x 32 rows
constexpr int kPBTile = 2 * kPBox;         // 8 KB: up to 128 columns
constexpr int kPAStage = kPTps * kPATile, kPBStage = kPTps * kPBTile;
constexpr int kPProdWarps = kPRows / 32;  // 8
constexpr int kPTmaWarp = kPProdWarps, kPMmaWarp = kPProdWarps + 1;
constexpr int kPEpiWarp0 = kPProdWarps + 2;
constexpr int kPEpiStride = 36;       // staging rows 36 floats apart (16-byte aligned, conflict-free)
constexpr uint32_t kPTmemCols = 512;  // two sets x two halves x 128 columns
constexpr int kPErr = 4;

// STAGES pipeline stages (32 KB of A + 16 KB of B each), EPIW epilogue warps
template <int STAGES, int EPIW>
struct __align__(1024) PersistSmem {
  uint8_t a[STAGES * kPAStage];
  uint8_t b[STAGES * kPBStage];  // 1 KB-aligned (128-byte swizzle atoms)
  float epi[EPIW][32 * kPEpiStride];
  uint64_t full[STAGES], empty[STAGES];
  uint64_t tfull[2], tempty[2];
  uint64_t qfull[kPQ], qempty[kPQ];
  int qitem[kPQ];
  uint32_t tmem_addr;
};
constexpr size_t kPSmemAlign = 1024;

__device__ __forceinline__ void persist_fail() { atomicCAS(&g_batch_error, 0, kPErr); }

// lane 0 waits on `bar` (bounded) and reads *val; the warp gets both
__device__ __forceinline__ bool warp_wait_read(uint64_t* bar, uint32_t parity, const int* val, int* out) {
  int ok = 1, v = 0;
  if ((threadIdx.x & 31) == 0) {
    ok = ptx::mbar_wait(bar, parity) ? 1 : 0;
    if (ok && val) v = *(volatile const int*)val;
  }
  ok = __shfl_sync(kFull, ok, 0);
  if (out) *out = __shfl_sync(kFull, v, 0);
  return ok != 0;
}

template <typename BT, int STAGES, int EPIW, int WA, bool TR>
__global__ void __launch_bounds__((kPEpiWarp0 + EPIW) * 32, 1)
    k_batched_persist(const BatchProblemTc* __restrict__ probs, const int4* __restrict__ items, int n_items,
                      int* next_item, int64_t N) {
  constexpr int kPStages = STAGES, kPEpiWarps = EPIW, kPWordAhead = WA;
  using Smem = PersistSmem<STAGES, EPIW>;
  static_assert(sizeof(Smem) + kPSmemAlign <= 232448, "persistent batched kernel: shared memory");
  static_assert(EPIW == 4 || EPIW == 8, "epilogue warps cover the four TMEM lane quarters");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(
      smem_raw + ((kPSmemAlign - (ptx::smem_addr(smem_raw) & (kPSmemAlign - 1))) & (kPSmemAlign - 1)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nbox = (int)((min(N, (int64_t)kPMaxN) + 63) / 64);  // 64-column boxes holding output columns
  if (tid == 0) {
    for (int s = 0; s < kPStages; s++) {
      ptx::mbar_init(&sm.full[s], kPProdWarps + 1);  // producer warps + the TMA transaction arrival
      ptx::mbar_init(&sm.empty[s], 1);               // tcgen05.commit of the stage's MMAs
    }
    for (int b = 0; b < 2; b++) {
      ptx::mbar_init(&sm.tfull[b], 1);
      ptx::mbar_init(&sm.tempty[b], kPEpiWarps);
    }
    for (int q = 0; q < kPQ; q++) {
      ptx::mbar_init(&sm.qfull[q], 1);
      ptx::mbar_init(&sm.qempty[q], kPEpiWarps);
    }
    ptx::fence_mbar_init();
  }
  if (warp == kPMmaWarp) {
    ptx::tmem_alloc(&sm.tmem_addr, kPTmemCols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  ptx::tc_fence_after_sync();
  const uint32_t tmem = sm.tmem_addr;

  if (warp < kPProdWarps) {
    // ---------------- A producers ----------------
    const int r = tid;  // row of the item
    uint32_t g = 0;     // stages produced so far (whole launch)
    for (int j = 0;; j++) {
      int it = -1;
      if (!warp_wait_read(&sm.qfull[j % kPQ], (uint32_t)(j / kPQ) & 1u, &sm.qitem[j % kPQ], &it)) {
        if (lane == 0) persist_fail();
        break;
      }
      if (it < 0) break;
      const int4 w4 = __ldg(items + it);
      const BatchProblemTc* p = probs + w4.x;
      const uint32_t* A = p->A;
      const int64_t M = p->M, Kw = p->Kw;
      const int64_t arow = (int64_t)w4.y * kPRows + r;
      const int nt = w4.w, nst = (nt + kPTps - 1) / kPTps;
      // forward: word k (a 32-column K tile) of row arow; Aᵀ·G: the words of
      // the item's 256 A columns in A rows 32k.. (thread r: row 32k + r % 32,
      // word r / 32 of the block)
      auto load_word = [&](int k) -> uint32_t {
        if (k >= nt) return 0u;
        if (!TR) return arow < M ? __ldg(A + arow * Kw + k) : 0u;
        const int64_t ar = (int64_t)k * kPK + (r & 31);
        const int64_t wc = (int64_t)w4.y * (kPRows / 32) + (r >> 5);
        return (ar < M && wc < Kw) ? __ldg(A + ar * Kw + wc) : 0u;
      };
      uint32_t wq[kPWordAhead][kPTps];
#pragma unroll
      for (int a = 0; a < kPWordAhead; a++)
#pragma unroll
        for (int u = 0; u < kPTps; u++) wq[a][u] = load_word(kPTps * a + u);
      bool fail = false;
      for (int i = 0; i < nst; i++, g++) {
        const int s = (int)(g % kPStages);
        uint32_t wn[kPTps];
#pragma unroll
        for (int u = 0; u < kPTps; u++) wn[u] = load_word(kPTps * (i + kPWordAhead) + u);
        if (g >= (uint32_t)kPStages &&
            !warp_wait_read(&sm.empty[s], ((g / kPStages) - 1) & 1u, nullptr, nullptr)) {
          if (lane == 0) persist_fail();
          fail = true;
          break;
        }
#pragma unroll
        for (int u = 0; u < kPTps; u++) {
          if (kPTps * i + u >= nt) continue;
          uint4 e[4];
          tc::expand32_two(wq[0][u], e);
          uint8_t* at = sm.a + s * kPAStage + u * kPATile;
          if (!TR) {  // row r of the tile: half r/128 at 8 KB, then core matrices
            uint8_t* as = at + (r >> 3) * tc::kSbo + (r & 7) * 16;
#pragma unroll
            for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(as + c * tc::kLbo) = e[c];
          } else {  // A row j of the tile, word wk of the block: output rows wk*32 + 8c ..
            const int j = r & 31, wk = r >> 5;
            uint8_t* as = at + (j >> 3) * tc::kLbo + (j & 7) * 16;
#pragma unroll
            for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(as + (wk * 4 + c) * tc::kSbo) = e[c];
          }
        }
        ptx::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&sm.full[s]);
#pragma unroll
        for (int a = 0; a < kPWordAhead - 1; a++)
#pragma unroll
          for (int u = 0; u < kPTps; u++) wq[a][u] = wq[a + 1][u];
#pragma unroll
        for (int u = 0; u < kPTps; u++) wq[kPWordAhead - 1][u] = wn[u];
      }
      if (fail) break;
    }
  } else if (warp == kPTmaWarp) {
    // ---------------- item queue + B by TMA ----------------
    if (lane == 0) {
      const uint32_t b0 = ptx::smem_addr(sm.b), f0 = ptx::smem_addr(&sm.full[0]);
      uint32_t g = 0;
      for (int j = 0;; j++) {
        const int q = j % kPQ;
        if (j >= kPQ && !ptx::mbar_wait(&sm.qempty[q], (uint32_t)((j / kPQ) - 1) & 1u)) {
          persist_fail();
          break;
        }
        const int it = atomicAdd(next_item, 1);
        sm.qitem[q] = it < n_items ? it : -1;
        ptx::mbar_arrive(&sm.qfull[q]);
        if (it >= n_items) break;
        const int4 w4 = __ldg(items + it);
        const void* map = &probs[w4.x].map;
        ptx::tensormap_acquire(map);  // written by the host into global memory
        const int nt = w4.w, nst = (nt + kPTps - 1) / kPTps;
        bool fail = false;
        for (int i = 0; i < nst; i++, g++) {
          const int s = (int)(g % kPStages);
          if (g >= (uint32_t)kPStages && !ptx::mbar_wait(&sm.empty[s], ((g / kPStages) - 1) & 1u)) {
            persist_fail();
            fail = true;
            break;
          }
          const int cnt = min(kPTps, nt - kPTps * i);
          ptx::mbar_arrive_expect_tx(&sm.full[s], (uint32_t)(cnt * nbox * kPBox));
          for (int u = 0; u < cnt; u++) {
            const int t = kPTps * i + u;
            for (int jb = 0; jb < nbox; jb++)
              ptx::tma_load_2d_u32(b0 + (uint32_t)(s * kPBStage + u * kPBTile + jb * kPBox), map, jb * 64, t * kPK,
                                   f0 + (uint32_t)s * 8u);
          }
        }
        if (fail) break;
      }
    }
  } else if (warp == kPMmaWarp) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t ab = std::is_same<BT, __nv_bfloat16>::value ? 1u : 0u;
      const uint32_t idesc = tc::idesc_f16(ab, TR ? 1u : 0u, 1u, (uint32_t)(nbox * 64), kPM);
      const uint64_t adesc = ptx::smem_desc_noswizzle_u32(ptx::smem_addr(sm.a), tc::kLbo, tc::kSbo);
      const uint64_t bdesc = ptx::smem_desc_noswizzle_u32(ptx::smem_addr(sm.b), kPBox, 1024) |
                             ((uint64_t)tc::kLayoutSw128 << 61);
      uint32_t g = 0;
      for (int j = 0;; j++) {
        if (!ptx::mbar_wait(&sm.qfull[j % kPQ], (uint32_t)(j / kPQ) & 1u)) {
          persist_fail();
          break;
        }
        const int it = *(volatile const int*)&sm.qitem[j % kPQ];
        if (it < 0) break;
        const int4 w4 = __ldg(items + it);
        const int64_t out_rows = TR ? probs[w4.x].K : probs[w4.x].M;  // rows of C (dX: A's columns)
        const int halves = (int64_t)w4.y * kPRows + kPM < out_rows ? 3 : 1;
        const int nt = w4.w, nst = (nt + kPTps - 1) / kPTps;
        const int set = j & 1;
        if (j >= 2 && !ptx::mbar_wait(&sm.tempty[set], (uint32_t)((j >> 1) - 1) & 1u)) {
          persist_fail();
          break;
        }
        ptx::tc_fence_after_sync();
        const uint32_t dset = tmem + (uint32_t)(set * 256);
        uint32_t started = 0;
        bool fail = false;
        for (int i = 0; i < nst; i++, g++) {
          const int s = (int)(g % kPStages);
          if (!ptx::mbar_wait(&sm.full[s], (g / kPStages) & 1u)) {
            persist_fail();
            fail = true;
            break;
          }
          ptx::tc_fence_after_sync();
#pragma unroll
          for (int u = 0; u < kPTps; u++) {
            if (kPTps * i + u >= nt) continue;
#pragma unroll
            for (int h = 0; h < 2; h++) {
              if (!((halves >> h) & 1)) continue;
#pragma unroll
              for (int k = 0; k < 2; k++)  // K half k: A two core-matrix columns on, B two 8-row groups on
                ptx::tc_mma_f16(dset + (uint32_t)(h * kPM),
                                adesc + (uint64_t)((s * kPAStage + u * kPATile + h * kPAHalf + k * 2 * tc::kLbo) >> 4),
                                bdesc + (uint64_t)((s * kPBStage + u * kPBTile + k * 2 * 1024) >> 4), idesc,
                                ((started >> h) & 1u) || k > 0);
              started |= 1u << h;
            }
          }
          ptx::tc_commit(&sm.empty[s]);
        }
        if (fail) break;
        if (nst > 0) ptx::tc_commit(&sm.tfull[set]);
        else ptx::mbar_arrive(&sm.tfull[set]);
      }
    }
  } else {
    // ---------------- epilogue ----------------
    const int e = warp - kPEpiWarp0;  // 0..EPIW-1
    const int q4 = warp & 3;          // the TMEM lane quarter this warp may access
    // column halves of this warp: one of the two with 8 epilogue warps, both with 4
    const int ch0 = EPIW == 8 ? e >> 2 : 0, ch1 = EPIW == 8 ? (e >> 2) + 1 : 2;
    const int cspan = nbox * 32;      // live columns per half (a multiple of 32)
    float* tile = sm.epi[e];
    for (int j = 0;; j++) {
      int it = -1;
      if (!warp_wait_read(&sm.qfull[j % kPQ], (uint32_t)(j / kPQ) & 1u, &sm.qitem[j % kPQ], &it)) {
        if (lane == 0) persist_fail();
        break;
      }
      if (it < 0) break;
      const int4 w4 = __ldg(items + it);
      const BatchProblemTc* p = probs + w4.x;
      const int64_t M = TR ? p->K : p->M, ldc = p->ldc;  // rows of C (dX: A's columns)
      float* C = p->C;
      const int nt = w4.w;
      const int set = j & 1;
      if (!warp_wait_read(&sm.tfull[set], (uint32_t)(j >> 1) & 1u, nullptr, nullptr)) {
        if (lane == 0) persist_fail();
        break;
      }
      ptx::tc_fence_after_sync();
      for (int hc = 0; hc < 2 * (ch1 - ch0); hc++) {
        const int h = hc & 1, ch = ch0 + (hc >> 1);
        const int64_t rbase = (int64_t)w4.y * kPRows + h * kPM + q4 * 32;  // the warp's first row
        if (rbase >= M) continue;
        const uint32_t tb = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(set * 256 + h * kPM + ch * cspan);
        for (int c8 = 0; c8 < cspan / 8; c8 += 4) {
          uint32_t v[4][8];
          if (nt > 0) {
#pragma unroll
            for (int u = 0; u < 4; u++) ptx::tmem_ld_32x32b_x8(tb + (uint32_t)((c8 + u) * 8), v[u]);
            ptx::tmem_wait_ld();
          } else {
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
              for (int x = 0; x < 8; x++) v[u][x] = 0u;
          }
#pragma unroll
          for (int u = 0; u < 4; u++) {
            float4* t4 = reinterpret_cast<float4*>(tile + lane * kPEpiStride + u * 8);
            t4[0] = make_float4(__uint_as_float(v[u][0]) * tc::kTwoScale, __uint_as_float(v[u][1]) * tc::kTwoScale,
                                __uint_as_float(v[u][2]) * tc::kTwoScale, __uint_as_float(v[u][3]) * tc::kTwoScale);
            t4[1] = make_float4(__uint_as_float(v[u][4]) * tc::kTwoScale, __uint_as_float(v[u][5]) * tc::kTwoScale,
                                __uint_as_float(v[u][6]) * tc::kTwoScale, __uint_as_float(v[u][7]) * tc::kTwoScale);
          }
          __syncwarp();
          // 8 lanes per row: rows 4*k + lane/8, 16 bytes each
          const int c4 = (lane & 7) * 4;
          const int64_t gcol = (int64_t)ch * cspan + c8 * 8 + c4;
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const int jr = k * 4 + (lane >> 3);
            const int64_t grow = rbase + jr;
            if (grow < M && gcol < N)
              *reinterpret_cast<float4*>(C + grow * ldc + gcol) = *reinterpret_cast<const float4*>(tile + jr * kPEpiStride + c4);
          }
          __syncwarp();
        }
      }
      ptx::tc_fence_before_sync();
      __syncwarp();
      if (lane == 0) {
        ptx::mbar_arrive(&sm.tempty[set]);
        ptx::mbar_arrive(&sm.qempty[j % kPQ]);
      }
    }
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  if (warp == kPMmaWarp) {
    ptx::tc_fence_after_sync();
    ptx::tmem_dealloc(tmem, kPTmemCols);
  }
}

template <typename BT, int STAGES, int EPIW, int WA, bool TR>
int launch_persist_s(const BatchProblemTc* probs, const int4* items, int n_items, int* counter, int64_t N,
                     cudaStream_t st) {
  constexpr size_t smem = sizeof(PersistSmem<STAGES, EPIW>) + kPSmemAlign;
  auto kern = k_batched_persist<BT, STAGES, EPIW, WA, TR>;
  static bool configured[64] = {false};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (dev < 64) configured[dev] = true;
  }
  BSP_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
  const int grid = std::min(num_sms(), n_items);
  kern<<<grid, (kPEpiWarp0 + EPIW) * 32, smem, st>>>(probs, items, n_items, counter, N);
  BSP_LAUNCHED();
  return BSP_OK;
}

// Shapes of the persistent kernel (pipeline stages, epilogue warps, A words
// loaded ahead), chosen per batch by bsp_batch_tune.  At the 512-problem N =
// 128 set: 3/4/4 192.6 us, 3/8/4 196.8 (its 576 threads spill 44 bytes at
// 96 registers), 3/8/8 198.9, 4/4/4 202.3, 4/4/8 206.8.
constexpr int kPersistShapes = 4;
template <typename BT, bool TR = false>
int launch_persist_t(const BatchProblemTc* probs, const int4* items, int n_items, int* counter, int64_t N,
                     int shape, cudaStream_t st) {
  switch (shape) {
    case 1: return launch_persist_s<BT, 3, 8, 4, TR>(probs, items, n_items, counter, N, st);
    case 2: return launch_persist_s<BT, 4, 4, 4, TR>(probs, items, n_items, counter, N, st);
    case 3: return launch_persist_s<BT, 3, 4, 8, TR>(probs, items, n_items, counter, N, st);
    default: return launch_persist_s<BT, 3, 4, 4, TR>(probs, items, n_items, counter, N, st);
  }
}

// ---- persistent batched SDDMM (dA = (G·Xᵀ) ⊙ A of a gradient batch) -----
// One CTA per SM takes items — (problem, 128 rows of dA, 256 columns of dA)
// — from the batch's work queue.  Both operands are dense 16-bit tiles, so
// there are no producers: the TMA warp loads, per 64 columns of N, G's box
// (128 rows, 16 KB) and X's box (256 rows, 32 KB), K-major with the 128-byte
// swizzle; the MMA warp issues four M128 N256 K16 MMAs per stage into
// accumulator set j % 2 of item j; 8 epilogue warps (two per TMEM lane
// quarter, one per 128-column half) keep the set bits of A's rows, pass 32
// columns at a time through a staging tile and store dA rows whole.  With
// two accumulator sets an item's epilogue — the store of 128 KB of dA, the
// bound of this write-heavy product — runs under the next item's loads and
// MMAs instead of after them.  Every wait is bounded (error 4 in
// g_batch_error).
constexpr int kSdRows = 128, kSdCols = 256, kSdStep = 64, kSdStages = 3;
constexpr int kSdGBox = kSdRows * kSdStep * 2;  // 16 KB
constexpr int kSdXBox = kSdCols * kSdStep * 2;  // 32 KB
constexpr int kSdEpiWarps = 8, kSdEpiWarp0 = 2;
constexpr int kSdThreads = (kSdEpiWarp0 + kSdEpiWarps) * 32;  // 320

struct __align__(1024) SddmmSmem {
  uint8_t g[kSdStages * kSdGBox];  // 1 KB-aligned boxes (128-byte swizzle atoms)
  uint8_t x[kSdStages * kSdXBox];
  float epi[kSdEpiWarps][32 * kPEpiStride];
  uint64_t full[kSdStages], empty[kSdStages];
  uint64_t tfull[2], tempty[2];
  uint64_t qfull[kPQ], qempty[kPQ];
  int qitem[kPQ];
  uint32_t tmem_addr;
};
static_assert(sizeof(SddmmSmem) + kPSmemAlign <= 232448, "persistent SDDMM: shared memory");

template <typename BT>
__global__ void __launch_bounds__(kSdThreads, 1)
    k_batched_sddmm_persist(const BatchProblemTc* __restrict__ probs, const int4* __restrict__ items, int n_items,
                            int* next_item, int64_t N) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  SddmmSmem& sm = *reinterpret_cast<SddmmSmem*>(
      smem_raw + ((kPSmemAlign - (ptx::smem_addr(smem_raw) & (kPSmemAlign - 1))) & (kPSmemAlign - 1)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nst = (int)((N + kSdStep - 1) / kSdStep);  // stages of an item (every item reduces all of N)
  if (tid == 0) {
    for (int s = 0; s < kSdStages; s++) {
      ptx::mbar_init(&sm.full[s], 1);   // the TMA transaction arrival
      ptx::mbar_init(&sm.empty[s], 1);  // tcgen05.commit of the stage's MMAs
    }
    for (int b = 0; b < 2; b++) {
      ptx::mbar_init(&sm.tfull[b], 1);
      ptx::mbar_init(&sm.tempty[b], kSdEpiWarps);
    }
    for (int q = 0; q < kPQ; q++) {
      ptx::mbar_init(&sm.qfull[q], 1);
      ptx::mbar_init(&sm.qempty[q], kSdEpiWarps);
    }
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(&sm.tmem_addr, kPTmemCols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  ptx::tc_fence_after_sync();
  const uint32_t tmem = sm.tmem_addr;

  if (warp == 0) {
    // ---------------- item queue + G and X by TMA ----------------
    if (lane == 0) {
      const uint32_t g0 = ptx::smem_addr(sm.g), x0 = ptx::smem_addr(sm.x), f0 = ptx::smem_addr(&sm.full[0]);
      uint32_t g = 0;
      for (int j = 0;; j++) {
        const int q = j % kPQ;
        if (j >= kPQ && !ptx::mbar_wait(&sm.qempty[q], (uint32_t)((j / kPQ) - 1) & 1u)) {
          persist_fail();
          break;
        }
        const int it = atomicAdd(next_item, 1);
        sm.qitem[q] = it < n_items ? it : -1;
        ptx::mbar_arrive(&sm.qfull[q]);
        if (it >= n_items) break;
        const int4 w4 = __ldg(items + it);
        const BatchProblemTc* p = probs + w4.x;
        ptx::tensormap_acquire(&p->map3);  // written by the host into global memory
        ptx::tensormap_acquire(&p->map2);
        bool fail = false;
        for (int i = 0; i < nst; i++, g++) {
          const int s = (int)(g % kSdStages);
          if (g >= (uint32_t)kSdStages && !ptx::mbar_wait(&sm.empty[s], ((g / kSdStages) - 1) & 1u)) {
            persist_fail();
            fail = true;
            break;
          }
          ptx::mbar_arrive_expect_tx(&sm.full[s], (uint32_t)(kSdGBox + kSdXBox));
          ptx::tma_load_2d_u32(g0 + (uint32_t)(s * kSdGBox), &p->map3, i * kSdStep, w4.y * kSdRows, f0 + (uint32_t)s * 8u);
          ptx::tma_load_2d_u32(x0 + (uint32_t)(s * kSdXBox), &p->map2, i * kSdStep, w4.z * kSdCols, f0 + (uint32_t)s * 8u);
        }
        if (fail) break;
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t ab = std::is_same<BT, __nv_bfloat16>::value ? 1u : 0u;
      const uint32_t idesc = tc::idesc_f16(ab, 0u, 0u, (uint32_t)kSdCols, (uint32_t)kSdRows);
      const uint64_t gdesc = ptx::smem_desc_noswizzle_u32(ptx::smem_addr(sm.g), 16, 1024) |
                             ((uint64_t)tc::kLayoutSw128 << 61);
      const uint64_t xdesc = ptx::smem_desc_noswizzle_u32(ptx::smem_addr(sm.x), 16, 1024) |
                             ((uint64_t)tc::kLayoutSw128 << 61);
      uint32_t g = 0;
      for (int j = 0;; j++) {
        if (!ptx::mbar_wait(&sm.qfull[j % kPQ], (uint32_t)(j / kPQ) & 1u)) {
          persist_fail();
          break;
        }
        if (*(volatile const int*)&sm.qitem[j % kPQ] < 0) break;
        const int set = j & 1;
        if (j >= 2 && !ptx::mbar_wait(&sm.tempty[set], (uint32_t)((j >> 1) - 1) & 1u)) {
          persist_fail();
          break;
        }
        ptx::tc_fence_after_sync();
        const uint32_t dset = tmem + (uint32_t)(set * kSdCols);
        bool fail = false;
        for (int i = 0; i < nst; i++, g++) {
          const int s = (int)(g % kSdStages);
          if (!ptx::mbar_wait(&sm.full[s], (g / kSdStages) & 1u)) {
            persist_fail();
            fail = true;
            break;
          }
          ptx::tc_fence_after_sync();
#pragma unroll
          for (int k = 0; k < kSdStep / 16; k++)  // K step k starts 32 B into the 128-byte rows
            ptx::tc_mma_f16(dset, gdesc + (uint64_t)((s * kSdGBox + k * 32) >> 4),
                            xdesc + (uint64_t)((s * kSdXBox + k * 32) >> 4), idesc, i > 0 || k > 0);
          ptx::tc_commit(&sm.empty[s]);
        }
        if (fail) break;
        if (nst > 0) ptx::tc_commit(&sm.tfull[set]);
        else ptx::mbar_arrive(&sm.tfull[set]);
      }
    }
  } else {
    // ---------------- epilogue ----------------
    const int e = warp - kSdEpiWarp0;  // 0..7
    const int q4 = warp & 3;           // the TMEM lane quarter this warp may access
    const int ch = e >> 2;             // 128-column half of the item
    float* tile = sm.epi[e];
    for (int j = 0;; j++) {
      int it = -1;
      if (!warp_wait_read(&sm.qfull[j % kPQ], (uint32_t)(j / kPQ) & 1u, &sm.qitem[j % kPQ], &it)) {
        if (lane == 0) persist_fail();
        break;
      }
      if (it < 0) break;
      const int4 w4 = __ldg(items + it);
      const BatchProblemTc* p = probs + w4.x;
      const int64_t M = p->M, K = p->K, Kw = p->Kw, ldc = p->ldc;
      float* C = p->C;
      const int64_t rbase = (int64_t)w4.y * kSdRows + q4 * 32;  // the warp's first row
      const int64_t cbase = (int64_t)w4.z * kSdCols + ch * 128;  // its first column
      // the row's A words of these 128 columns
      uint32_t aw[4] = {0u, 0u, 0u, 0u};
      if (rbase + lane < M) {
        const uint32_t* arow = p->A + (rbase + lane) * Kw;
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (cbase / 32 + i < Kw) aw[i] = __ldg(arow + cbase / 32 + i);
      }
      const int set = j & 1;
      if (!warp_wait_read(&sm.tfull[set], (uint32_t)(j >> 1) & 1u, nullptr, nullptr)) {
        if (lane == 0) persist_fail();
        break;
      }
      ptx::tc_fence_after_sync();
      const uint32_t tb = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(set * kSdCols + ch * 128);
      for (int c32 = 0; c32 < 4; c32++) {
        uint32_t v[4][8];
#pragma unroll
        for (int u = 0; u < 4; u++) ptx::tmem_ld_32x32b_x8(tb + (uint32_t)(c32 * 32 + u * 8), v[u]);
        ptx::tmem_wait_ld();
        const uint32_t wbits = aw[c32];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          float4* t4 = reinterpret_cast<float4*>(tile + lane * kPEpiStride + u * 8);
          float f[8];
#pragma unroll
          for (int x = 0; x < 8; x++) f[x] = ((wbits >> (u * 8 + x)) & 1u) ? __uint_as_float(v[u][x]) : 0.f;
          t4[0] = make_float4(f[0], f[1], f[2], f[3]);
          t4[1] = make_float4(f[4], f[5], f[6], f[7]);
        }
        __syncwarp();
        // 8 lanes per row: rows 4*k + lane/8, 16 bytes each
        const int c4 = (lane & 7) * 4;
        const int64_t gcol = cbase + c32 * 32 + c4;
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int jr = k * 4 + (lane >> 3);
          const int64_t grow = rbase + jr;
          if (grow < M && gcol < K)
            *reinterpret_cast<float4*>(C + grow * ldc + gcol) = *reinterpret_cast<const float4*>(tile + jr * kPEpiStride + c4);
        }
        __syncwarp();
      }
      ptx::tc_fence_before_sync();
      __syncwarp();
      if (lane == 0) {
        ptx::mbar_arrive(&sm.tempty[set]);
        ptx::mbar_arrive(&sm.qempty[j % kPQ]);
      }
    }
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after_sync();
    ptx::tmem_dealloc(tmem, kPTmemCols);
  }
}

template <typename BT>
int launch_sddmm_persist_t(const BatchProblemTc* probs, const int4* items, int n_items, int* counter, int64_t N,
                           cudaStream_t st) {
  constexpr size_t smem = sizeof(SddmmSmem) + kPSmemAlign;
  static bool configured[64] = {false};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(k_batched_sddmm_persist<BT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (dev < 64) configured[dev] = true;
  }
  BSP_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
  const int grid = std::min(num_sms(), n_items);
  k_batched_sddmm_persist<BT><<<grid, kSdThreads, smem, st>>>(probs, items, n_items, counter, N);
  BSP_LAUNCHED();
  return BSP_OK;
}

}  // namespace


}  // namespace bsp

struct bsp_batch {
  int n = 0;
  int64_t N = 0;
  int bdt = BSP_BF16;
  int grad = 0;         // 0: forward batch (bsp_batch_create), 1: gradient batch (bsp_batch_grad_create)
  int n_items = 0;      // forward items, or the Aᵀ·G items of a gradient batch
  int n_items_s = 0;    // SDDMM items of a gradient batch
  int device = 0;
  void* dev = nullptr;  // records, items, the work-queue counter
  bsp::BatchProblemTc* probs = nullptr;    // forward, or Aᵀ·G (map = G)
  bsp::BatchProblemTc* probs_s = nullptr;  // SDDMM (map = G, map2 = X)
  int4* items = nullptr;
  int4* items_s = nullptr;
  int4* items_sp = nullptr;  // SDDMM items of the persistent kernel: (problem, 128 rows, 256 columns)
  int n_items_sp = 0;
  int* counter = nullptr;  // next item of the persistent kernel (reset by every run)
  int shape = 0;           // persistent kernel's shape (bsp_batch_tune)
};

namespace {

// Uploads records and items into one device block and fills the batch.
int batch_upload(bsp_batch* b, const std::vector<bsp::BatchProblemTc>& p1, const std::vector<int4>& i1,
                 const std::vector<bsp::BatchProblemTc>& p2, const std::vector<int4>& i2, cudaStream_t s,
                 const std::vector<int4>& i3 = {}) {
  using namespace bsp;
  auto up = [](size_t bytes) { return (std::max<size_t>(bytes, 1) + 255) & ~size_t(255); };
  const size_t o_p1 = 0, o_i1 = o_p1 + up(sizeof(BatchProblemTc) * p1.size());
  const size_t o_p2 = o_i1 + up(sizeof(int4) * i1.size()), o_i2 = o_p2 + up(sizeof(BatchProblemTc) * p2.size());
  const size_t o_i3 = o_i2 + up(sizeof(int4) * i2.size());
  const size_t o_c = o_i3 + up(sizeof(int4) * i3.size()), total = o_c + 256;
  cudaError_t e = cudaMalloc(&b->dev, total);
  if (e != cudaSuccess) {
    cuda_status(e);
    b->dev = nullptr;
    return BSP_ERR_ALLOC;
  }
  char* base = static_cast<char*>(b->dev);
  b->probs = reinterpret_cast<BatchProblemTc*>(base + o_p1);
  b->items = reinterpret_cast<int4*>(base + o_i1);
  b->probs_s = reinterpret_cast<BatchProblemTc*>(base + o_p2);
  b->items_s = reinterpret_cast<int4*>(base + o_i2);
  b->items_sp = reinterpret_cast<int4*>(base + o_i3);
  b->counter = reinterpret_cast<int*>(base + o_c);
  b->n_items = (int)i1.size();
  b->n_items_s = (int)i2.size();
  b->n_items_sp = (int)i3.size();
  struct Part { void* dst; const void* src; size_t bytes; };
  const Part parts[5] = {{b->probs, p1.data(), sizeof(BatchProblemTc) * p1.size()},
                         {b->items, i1.data(), sizeof(int4) * i1.size()},
                         {b->probs_s, p2.data(), sizeof(BatchProblemTc) * p2.size()},
                         {b->items_s, i2.data(), sizeof(int4) * i2.size()},
                         {b->items_sp, i3.data(), sizeof(int4) * i3.size()}};
  for (const Part& q : parts)
    if (q.bytes && (e = cudaMemcpyAsync(q.dst, q.src, q.bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_status(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
  return BSP_OK;
}

// longest reduction first (LPT), ties by problem order: stable
void sort_items(std::vector<int4>& items) {
  std::stable_sort(items.begin(), items.end(), [](const int4& x, const int4& y) { return x.w > y.w; });
}

}  // namespace

extern "C" {

int bsp_batch_create(const bsp_problem* problems, int n, int64_t N, int b_dtype, bsp_batch** batch,
                     bsp_stream_t stream) {
  using namespace bsp;
  if (!batch) return BSP_ERR_INVALID_ARG;
  *batch = nullptr;
  if (n < 0 || N < 0 || N > ((int64_t)1 << 30)) return BSP_ERR_INVALID_ARG;
  if (n > 0 && !problems) return BSP_ERR_INVALID_ARG;
  if (b_dtype != BSP_BF16 && b_dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (N % 8 != 0) return BSP_ERR_ALIGNMENT;
  std::vector<BatchProblemTc> hp((size_t)n);
  std::vector<int4> items;
  for (int i = 0; i < n; i++) {
    const bsp_problem& p = problems[i];
    if (p.M < 0 || p.K < 0 || p.M > INT32_MAX || p.K > ((int64_t)1 << 30)) return BSP_ERR_INVALID_ARG;
    if (p.K > tc_max_reduction()) return BSP_ERR_CAPACITY;
    if (p.ldb < N || p.ldc < N) return BSP_ERR_INVALID_ARG;
    if ((p.M > 0 && p.K > 0 && !p.A_words) || (p.K > 0 && N > 0 && !p.B) || (p.M > 0 && N > 0 && !p.C))
      return BSP_ERR_INVALID_ARG;
    if (!is_aligned(p.A_words, 4) || !is_aligned(p.B, 16) || (p.ldb * 2) % 16 != 0 || !is_aligned(p.C, 16) ||
        p.ldc % 4 != 0)
      return BSP_ERR_ALIGNMENT;
    const int64_t Kw = ceil_div(p.K, 32);
    BatchProblemTc& r = hp[(size_t)i];
    std::memset(&r, 0, sizeof(r));
    if (p.K > 0 && N > 0) BSP_TRY(make_batch_map(&r.map, p.B, b_dtype, p.K, N, p.ldb));
    r.A = p.A_words;
    r.M = p.M;
    r.K = p.K;
    r.Kw = Kw;
    r.C = p.C;
    r.ldc = p.ldc;
    for (int64_t rb = 0; rb < ceil_div(p.M, kItemRows); rb++)
      for (int64_t nb = 0; nb < ceil_div(N, kItemCols); nb++) items.push_back(make_int4(i, (int)rb, (int)nb, (int)Kw));
  }
  if (items.size() > (size_t)INT32_MAX) return BSP_ERR_CAPACITY;
  sort_items(items);
  bsp_batch* b = new (std::nothrow) bsp_batch();
  if (!b) return BSP_ERR_ALLOC;
  b->n = n;
  b->N = N;
  b->bdt = b_dtype;
  cudaGetDevice(&b->device);
  const int st = batch_upload(b, hp, items, {}, {}, (cudaStream_t)stream);
  if (st != BSP_OK) {
    if (b->dev) cudaFree(b->dev);
    delete b;
    return st;
  }
  *batch = b;
  return BSP_OK;
}

int bsp_batch_grad_create(const bsp_problem_grad* problems, int n, int64_t N, int dtype, bsp_batch** batch,
                          bsp_stream_t stream) {
  using namespace bsp;
  if (!batch) return BSP_ERR_INVALID_ARG;
  *batch = nullptr;
  if (n < 0 || N < 0 || N > ((int64_t)1 << 30)) return BSP_ERR_INVALID_ARG;
  if (n > 0 && !problems) return BSP_ERR_INVALID_ARG;
  if (dtype != BSP_BF16 && dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (N % 8 != 0) return BSP_ERR_ALIGNMENT;
  std::vector<BatchProblemTc> pt, ps;
  std::vector<int4> it, is, isp;
  for (int i = 0; i < n; i++) {
    const bsp_problem_grad& p = problems[i];
    if (p.M < 0 || p.K < 0 || p.M > INT32_MAX || p.K > INT32_MAX) return BSP_ERR_INVALID_ARG;
    if (p.ldx < N || p.ldg < N) return BSP_ERR_INVALID_ARG;
    if (p.dX && p.lddx < N) return BSP_ERR_INVALID_ARG;
    if (p.dA && p.ldda < p.K) return BSP_ERR_INVALID_ARG;
    const bool work = p.M > 0 && p.K > 0;
    if (work && (!p.A_words || (N > 0 && (!p.X || !p.G)))) return BSP_ERR_INVALID_ARG;
    if (!is_aligned(p.A_words, 4) || !is_aligned(p.X, 16) || !is_aligned(p.G, 16) || (p.ldx * 2) % 16 != 0 ||
        (p.ldg * 2) % 16 != 0)
      return BSP_ERR_ALIGNMENT;
    const int64_t Kw = ceil_div(p.K, 32);
    if (p.dX && p.K > 0) {  // dX = Aᵀ·G: output rows K, reduction over M in 32-row tiles
      if (ceil_div(p.M, 32) * 32 > tc_max_reduction()) return BSP_ERR_CAPACITY;
      if (!is_aligned(p.dX, 16) || p.lddx % 4 != 0) return BSP_ERR_ALIGNMENT;
      BatchProblemTc r;
      std::memset(&r, 0, sizeof(r));
      if (p.M > 0 && N > 0) BSP_TRY(make_batch_map(&r.map, p.G, dtype, p.M, N, p.ldg));
      r.A = p.A_words;
      r.M = p.M;
      r.K = p.K;
      r.Kw = Kw;
      r.C = p.dX;
      r.ldc = p.lddx;
      const int idx = (int)pt.size();
      pt.push_back(r);
      for (int64_t rb = 0; rb < ceil_div(p.K, kItemRows); rb++)
        for (int64_t nb = 0; nb < ceil_div(N, kItemCols); nb++)
          it.push_back(make_int4(idx, (int)rb, (int)nb, (int)ceil_div(p.M, 32)));
    }
    if (p.dA && p.M > 0) {  // dA = (G·Xᵀ) ⊙ A: output [M][K], reduction over N in 64-column steps
      if (p.K % 8 != 0 || !is_aligned(p.dA, 16) || p.ldda % 4 != 0) return BSP_ERR_ALIGNMENT;
      if (ceil_div(p.K, kItemCols) > INT32_MAX) return BSP_ERR_CAPACITY;
      BatchProblemTc r;
      std::memset(&r, 0, sizeof(r));
      if (p.K > 0 && N > 0) {
        BSP_TRY(make_batch_map_sddmm(&r.map, p.G, dtype, p.M, N, p.ldg));
        BSP_TRY(make_batch_map_sddmm(&r.map2, p.X, dtype, p.K, N, p.ldx));
        BSP_TRY(make_batch_map_sddmm(&r.map3, p.G, dtype, p.M, N, p.ldg, 128));
      }
      r.A = p.A_words;
      r.M = p.M;
      r.K = p.K;
      r.Kw = Kw;
      r.C = p.dA;
      r.ldc = p.ldda;
      const int idx = (int)ps.size();
      ps.push_back(r);
      for (int64_t rb = 0; rb < ceil_div(p.M, kItemRows); rb++)
        for (int64_t kb = 0; kb < ceil_div(p.K, kItemCols); kb++)
          is.push_back(make_int4(idx, (int)rb, (int)kb, (int)ceil_div(N, 64)));
      for (int64_t rb = 0; rb < ceil_div(p.M, (int64_t)kSdRows); rb++)
        for (int64_t kb = 0; kb < ceil_div(p.K, (int64_t)kSdCols); kb++)
          isp.push_back(make_int4(idx, (int)rb, (int)kb, (int)ceil_div(N, 64)));
    }
  }
  if (it.size() > (size_t)INT32_MAX || is.size() > (size_t)INT32_MAX || isp.size() > (size_t)INT32_MAX)
    return BSP_ERR_CAPACITY;
  sort_items(it);
  sort_items(is);
  bsp_batch* b = new (std::nothrow) bsp_batch();
  if (!b) return BSP_ERR_ALLOC;
  b->n = n;
  b->N = N;
  b->bdt = dtype;
  b->grad = 1;
  cudaGetDevice(&b->device);
  const int st = batch_upload(b, pt, it, ps, is, (cudaStream_t)stream, isp);
  if (st != BSP_OK) {
    if (b->dev) cudaFree(b->dev);
    delete b;
    return st;
  }
  *batch = b;
  return BSP_OK;
}

int bsp_batch_destroy(bsp_batch* batch) {
  if (!batch) return BSP_OK;
  if (batch->dev) cudaFree(batch->dev);
  delete batch;
  return BSP_OK;
}

int bsp_batched_spmm(const bsp_batch* b, bsp_stream_t stream) {
  using namespace bsp;
  if (!b || b->grad) return BSP_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) return BSP_ERR_INVALID_ARG;
  if (b->n_items == 0 || b->N == 0) return BSP_OK;
  const cudaStream_t s = (cudaStream_t)stream;
  // N ≤ 128: the persistent kernel (BSP_BATCH_PERSIST=0 selects the CTA-per-item
  // launch, for comparisons); wider N: a CTA per (256-row, 256-column) item
  const char* e = getenv("BSP_BATCH_PERSIST");
  if (b->N <= kPMaxN && !(e && e[0] == '0')) {
    if (b->bdt == BSP_BF16)
      return launch_persist_t<__nv_bfloat16>(b->probs, b->items, b->n_items, b->counter, b->N, b->shape, s);
    if (b->bdt == BSP_F16)
      return launch_persist_t<__half>(b->probs, b->items, b->n_items, b->counter, b->N, b->shape, s);
    return BSP_ERR_UNSUPPORTED;
  }
  return launch_batched_tc(b->probs, b->items, b->n_items, b->N, b->bdt, s);
}

int bsp_batch_tune(bsp_batch* b, bsp_stream_t stream, int* shape, float* ms) {
  using namespace bsp;
  if (!b || b->grad || !shape || !ms) return BSP_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) return BSP_ERR_INVALID_ARG;
  const cudaStream_t s = (cudaStream_t)stream;
  const char* e = getenv("BSP_BATCH_PERSIST");
  const int n_shapes = (b->N <= kPMaxN && !(e && e[0] == '0')) ? kPersistShapes : 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int best = 0;
  float best_ms = 0.f;
  const int keep = b->shape;
  auto sweep = [&]() -> int {
    BSP_CUDA(cudaEventCreate(&e0));
    BSP_CUDA(cudaEventCreate(&e1));
    for (int v = 0; v < n_shapes; v++) {
      b->shape = v;
      BSP_TRY(bsp_batched_spmm(b, stream));  // warm-up (first launch of this shape)
      BSP_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < 3; r++) BSP_TRY(bsp_batched_spmm(b, stream));
      BSP_CUDA(cudaEventRecord(e1, s));
      BSP_CUDA(cudaEventSynchronize(e1));
      float t = 0.f;
      BSP_CUDA(cudaEventElapsedTime(&t, e0, e1));
      t /= 3.f;
      if (v == 0 || t < best_ms) {
        best = v;
        best_ms = t;
      }
    }
    return BSP_OK;
  };
  const int rc = sweep();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc != BSP_OK) {
    b->shape = keep;
    return rc;
  }
  b->shape = best;
  *shape = best;
  *ms = best_ms;
  return BSP_OK;
}

int bsp_batched_spmm_grad(const bsp_batch* b, bsp_stream_t stream) {
  using namespace bsp;
  if (!b || !b->grad) return BSP_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) return BSP_ERR_INVALID_ARG;
  if (b->N == 0) return BSP_OK;
  const cudaStream_t s = (cudaStream_t)stream;
  // dX = Aᵀ·G: for N ≤ 128 the persistent kernel in its transposed form
  // (BSP_BATCH_PERSIST=0 selects the CTA per item, for comparisons)
  const char* ep = getenv("BSP_BATCH_PERSIST");
  if (b->N <= kPMaxN && !(ep && ep[0] == '0')) {
    if (b->n_items > 0) {
      const int rc = b->bdt == BSP_BF16
                         ? launch_persist_t<__nv_bfloat16, true>(b->probs, b->items, b->n_items, b->counter, b->N, 0, s)
                         : launch_persist_t<__half, true>(b->probs, b->items, b->n_items, b->counter, b->N, 0, s);
      BSP_TRY(rc);
    }
  } else {
    BSP_TRY(launch_batched_tc(b->probs, b->items, b->n_items, b->N, b->bdt, s, 1));
  }
  // dA: the persistent SDDMM (BSP_BATCH_SDDMM_PERSIST=0 selects the CTA per
  // 256x256 item, for comparisons)
  const char* e = getenv("BSP_BATCH_SDDMM_PERSIST");
  if (!(e && e[0] == '0')) {
    if (b->n_items_sp == 0) return BSP_OK;
    if (b->bdt == BSP_BF16)
      return launch_sddmm_persist_t<__nv_bfloat16>(b->probs_s, b->items_sp, b->n_items_sp, b->counter, b->N, s);
    return launch_sddmm_persist_t<__half>(b->probs_s, b->items_sp, b->n_items_sp, b->counter, b->N, s);
  }
  return launch_batched_tc(b->probs_s, b->items_s, b->n_items_s, b->N, b->bdt, s, 2);
}

}  // extern "C"
