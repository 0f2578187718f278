// spmm_batched.cu — many independent bitmap SpMMs in one persistent
// tensor-core launch.
//
// A batch (bsp_batch_create) holds a device array of problem descriptors and
// a work queue: one item per (problem, 128-row block, column block of TN),
// sorted by reduction length, longest first.  One persistent kernel walks
// the queue (CTA b takes items b, b + grid, b + 2·grid, …) with three roles
// that run concurrently:
//   warps 0-3  producers: expand the item's 32-column bit tile of A into 0/1
//              16-bit operands (K-major core matrices) and stream the 32 x TN
//              B tile with 16-byte cp.async (MN-major), 4-stage ring;
//   warp 4     TMEM owner; lane 0 issues tcgen05.mma (M=128, N=TN, K=16) into
//              one of two TMEM accumulators and commits the stages;
//   warps 5-8  epilogue: tcgen05.ld the finished accumulator, store C, and
//              hand the accumulator back — so the epilogue of item j
//              overlaps the MMAs of item j+1.
// All barriers are mbarriers with bounded waits (timeout → error 4 in
// g_batch_error and the CTA stops at the next check).
#include <algorithm>
#include <new>
#include <type_traits>
#include <vector>

#include "ptx.cuh"
#include "spmm_dev.cuh"
#include "tc_common.cuh"

namespace bsp {

__device__ int g_batch_error;

namespace {

using tc::expand8;
using tc::kLbo;
using tc::kSbo;

constexpr int kBM = 128;
constexpr int kBK = 32;
constexpr int kBStages = 4;
constexpr int kBThreads = 288;  // 9 warps
constexpr int kBProducers = 128;

struct DevProblem {
  const uint32_t* A;
  int64_t M, K, Kw;
  const void* B;
  int64_t ldb;
  float* C;
  int64_t ldc;
};

struct BatchArgs {
  const DevProblem* probs;
  const int4* items;  // {problem, row block, column block, reduction tiles}
  int n_items;
  int64_t N;
};

template <int TN>
struct __align__(1024) BatchSmem {
  uint8_t a[kBStages][kBM * kBK * 2];
  uint8_t b[kBStages][kBK * TN * 2];
  uint64_t full[kBStages];
  uint64_t empty[kBStages];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint32_t tmem_addr;
  int abort;
};

__device__ __forceinline__ bool bwait(uint64_t* bar, uint32_t parity, int* abort) {
  if (ptx::mbar_wait(bar, parity)) return true;
  atomicCAS(&g_batch_error, 0, 4);
  *(volatile int*)abort = 1;
  return false;
}

template <typename BT, int TN>
__global__ void __launch_bounds__(kBThreads, 1) k_spmm_batched_tc(BatchArgs ba) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  BatchSmem<TN>& sm = *reinterpret_cast<BatchSmem<TN>*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t one = std::is_same<BT, __nv_bfloat16>::value ? 0x3f80u : 0x3c00u;
  constexpr uint32_t kCols = 2 * TN;  // two accumulators

  if (tid == 0) {
    for (int s = 0; s < kBStages; s++) {
      ptx::mbar_init(&sm.full[s], kBProducers);
      ptx::mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      ptx::mbar_init(&sm.tfull[b], 1);
      ptx::mbar_init(&sm.tempty[b], 128);
    }
    sm.abort = 0;
    ptx::fence_mbar_init();
  }
  if (warp == 4) {
    ptx::tmem_alloc(&sm.tmem_addr, kCols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  ptx::tc_fence_after_sync();
  const uint32_t tmem = sm.tmem_addr;

  if (warp < 4) {
    // ---------------- producers ----------------
    int i = 0;
    for (int q = blockIdx.x; q < ba.n_items && !*(volatile int*)&sm.abort; q += gridDim.x) {
      const int4 it = ba.items[q];
      const DevProblem p = ba.probs[it.x];
      const BT* B = static_cast<const BT*>(p.B);
      const int64_t arow = (int64_t)it.y * kBM + tid;
      const int64_t col0 = (int64_t)it.z * TN;
      for (int kt = 0; kt < it.w; kt++, i++) {
        const int s = i % kBStages;
        if (i >= kBStages && !bwait(&sm.empty[s], ((i / kBStages) - 1) & 1, &sm.abort)) break;
        const uint32_t w = arow < p.M ? __ldg(p.A + arow * p.Kw + kt) : 0u;
        uint8_t* as = sm.a[s] + (tid >> 3) * kSbo + (tid & 7) * 16;
#pragma unroll
        for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(as + c * kLbo) = expand8((w >> (8 * c)) & 0xffu, one);
#pragma unroll
        for (int j = 0; j < TN / 32; j++) {
          const int qq = tid + kBProducers * j;
          const int k = qq / (TN / 8), n8 = qq % (TN / 8);
          const int64_t krow = (int64_t)kt * kBK + k;
          const int64_t ncol = col0 + n8 * 8;
          const bool ok = krow < p.K && ncol < ba.N;
          ptx::cp_async_16(sm.b[s] + n8 * kSbo + (k >> 3) * kLbo + (k & 7) * 16,
                           ok ? B + krow * p.ldb + ncol : B, ok ? 16u : 0u);
        }
        ptx::cp_async_commit();
        ptx::cp_async_wait_group<2>();
        if (i >= 2) {
          ptx::fence_proxy_async_smem();
          ptx::mbar_arrive(&sm.full[(i - 2) % kBStages]);
        }
      }
    }
    ptx::cp_async_wait_group<0>();
    ptx::fence_proxy_async_smem();
    for (int j = (i >= 2 ? i - 2 : 0); j < i; j++) ptx::mbar_arrive(&sm.full[j % kBStages]);
  } else if (warp == 4) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t ab = std::is_same<BT, __nv_bfloat16>::value ? 1u : 0u;
      const uint32_t idesc = tc::idesc_f16(ab, 0u, 1u, TN, kBM);
      int i = 0, j = 0;
      for (int q = blockIdx.x; q < ba.n_items && !*(volatile int*)&sm.abort; q += gridDim.x, j++) {
        const int kts = ba.items[q].w;
        const int buf = j & 1;
        if (j >= 2 && !bwait(&sm.tempty[buf], ((j >> 1) - 1) & 1, &sm.abort)) break;
        ptx::tc_fence_after_sync();
        const uint32_t d = tmem + (uint32_t)(buf * TN);
        bool ok = true;
        for (int kt = 0; kt < kts; kt++, i++) {
          const int s = i % kBStages;
          if (!bwait(&sm.full[s], (i / kBStages) & 1, &sm.abort)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after_sync();
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const uint64_t ad = ptx::smem_desc_noswizzle(sm.a[s] + h * 2 * kLbo, kLbo, kSbo);
            const uint64_t bd = ptx::smem_desc_noswizzle(sm.b[s] + h * 2 * kLbo, kLbo, kSbo);
            ptx::tc_mma_f16(d, ad, bd, idesc, (kt > 0) || (h > 0));
          }
          ptx::tc_commit(&sm.empty[s]);
        }
        if (!ok) break;
        if (kts > 0) ptx::tc_commit(&sm.tfull[buf]);
        else ptx::mbar_arrive(&sm.tfull[buf]);
      }
    }
  } else {
    // ---------------- epilogue (warps 5-8) ----------------
    const int quarter = warp & 3;  // TMEM lanes 32*quarter .. +31
    int j = 0;
    for (int q = blockIdx.x; q < ba.n_items && !*(volatile int*)&sm.abort; q += gridDim.x, j++) {
      const int4 it = ba.items[q];
      const DevProblem p = ba.probs[it.x];
      const int buf = j & 1;
      if (!bwait(&sm.tfull[buf], (j >> 1) & 1, &sm.abort)) break;
      ptx::tc_fence_after_sync();
      const int64_t row = (int64_t)it.y * kBM + quarter * 32 + lane;
      const int64_t col0 = (int64_t)it.z * TN;
      float* crow = p.C + row * p.ldc + col0;
      const bool live = row < p.M;
      for (int c8 = 0; c8 < TN / 8; c8 += 4) {
        uint32_t r[4][8];
        if (it.w > 0) {
#pragma unroll
          for (int u = 0; u < 4; u++)
            ptx::tmem_ld_32x32b_x8(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * TN + (c8 + u) * 8),
                                   r[u]);
          ptx::tmem_wait_ld();
        } else {
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int e = 0; e < 8; e++) r[u][e] = 0u;
        }
        if (!live) continue;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int col = (c8 + u) * 8;
          if (col0 + col >= ba.N) continue;
          *reinterpret_cast<float4*>(crow + col) = make_float4(
              __uint_as_float(r[u][0]), __uint_as_float(r[u][1]), __uint_as_float(r[u][2]), __uint_as_float(r[u][3]));
          *reinterpret_cast<float4*>(crow + col + 4) = make_float4(
              __uint_as_float(r[u][4]), __uint_as_float(r[u][5]), __uint_as_float(r[u][6]), __uint_as_float(r[u][7]));
        }
      }
      ptx::tc_fence_before_sync();
      ptx::mbar_arrive(&sm.tempty[buf]);
    }
  }
  ptx::tc_fence_before_sync();
  __syncthreads();
  if (warp == 4) {
    ptx::tc_fence_after_sync();
    ptx::tmem_dealloc(tmem, kCols);
  }
}

}  // namespace
}  // namespace bsp

// ---------------------------------------------------------------------------
// host side: the batch object and its launch

struct bsp_batch {
  int n = 0;
  int64_t N = 0;
  int bdt = BSP_BF16;
  int tn = 128;
  int n_items = 0;
  int device = 0;
  int grid = 0;
  void* dev = nullptr;  // DevProblem[n] followed by int4 items[n_items]
  bsp::DevProblem* probs = nullptr;
  int4* items = nullptr;
  int64_t nnz_hint = 0;
};

namespace bsp {
namespace {

template <typename BT, int TN>
int launch_batched_t(const bsp_batch* b, cudaStream_t s) {
  const size_t smem = sizeof(BatchSmem<TN>);
  static bool configured[64] = {};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(k_spmm_batched_tc<BT, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured[dev] = true;
  }
  BatchArgs a = {b->probs, b->items, b->n_items, b->N};
  k_spmm_batched_tc<BT, TN><<<b->grid, kBThreads, smem, s>>>(a);
  BSP_LAUNCHED();
  return BSP_OK;
}

template <typename BT, int TN>
int batched_occupancy() {
  int occ = 0;
  if (cudaFuncSetAttribute(k_spmm_batched_tc<BT, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(BatchSmem<TN>)) != cudaSuccess)
    return 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_spmm_batched_tc<BT, TN>, kBThreads,
                                                    sizeof(BatchSmem<TN>)) != cudaSuccess)
    return 1;
  // two TMEM accumulators of TN columns each: at most 512 / (2*TN) CTAs per SM
  const int tmem_cap = 512 / (2 * TN);
  return std::max(1, std::min(occ, tmem_cap));
}

}  // namespace

int batched_device_error(int* out, bool clear) {
  BSP_CUDA(cudaMemcpyFromSymbol(out, g_batch_error, sizeof(int)));
  if (clear) {
    const int zero = 0;
    BSP_CUDA(cudaMemcpyToSymbol(g_batch_error, &zero, sizeof(int)));
  }
  return BSP_OK;
}

}  // namespace bsp

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
  const int tn = N <= 128 ? 128 : 256;
  std::vector<DevProblem> hp((size_t)n);
  std::vector<int4> items;
  for (int i = 0; i < n; i++) {
    const bsp_problem& p = problems[i];
    if (p.M < 0 || p.K < 0 || p.M > INT32_MAX || p.K > ((int64_t)1 << 30)) return BSP_ERR_INVALID_ARG;
    if (p.ldb < N || p.ldc < N) return BSP_ERR_INVALID_ARG;
    if ((p.M > 0 && p.K > 0 && !p.A_words) || (p.K > 0 && N > 0 && !p.B) || (p.M > 0 && N > 0 && !p.C))
      return BSP_ERR_INVALID_ARG;
    if (!is_aligned(p.A_words, 4) || !is_aligned(p.B, 16) || (p.ldb * 2) % 16 != 0 || !is_aligned(p.C, 16) ||
        p.ldc % 4 != 0)
      return BSP_ERR_ALIGNMENT;
    const int64_t Kw = ceil_div(p.K, 32);
    hp[(size_t)i] = DevProblem{p.A_words, p.M, p.K, Kw, p.B, p.ldb, p.C, p.ldc};
    for (int64_t rb = 0; rb < ceil_div(p.M, kBM); rb++)
      for (int64_t nb = 0; nb < ceil_div(N, tn); nb++) items.push_back(make_int4(i, (int)rb, (int)nb, (int)Kw));
  }
  if (items.size() > (size_t)INT32_MAX) return BSP_ERR_CAPACITY;
  // longest reduction first (LPT), ties by problem order: stable
  std::stable_sort(items.begin(), items.end(), [](const int4& x, const int4& y) { return x.w > y.w; });
  bsp_batch* b = new (std::nothrow) bsp_batch();
  if (!b) return BSP_ERR_ALLOC;
  b->n = n;
  b->N = N;
  b->bdt = b_dtype;
  b->tn = tn;
  b->n_items = (int)items.size();
  cudaGetDevice(&b->device);
  const size_t pbytes = sizeof(DevProblem) * (size_t)std::max(n, 1);
  const size_t ibytes = sizeof(int4) * std::max<size_t>(items.size(), 1);
  const size_t poff = (pbytes + 255) & ~size_t(255);
  cudaError_t e = cudaMalloc(&b->dev, poff + ibytes);
  if (e != cudaSuccess) {
    cuda_status(e);
    delete b;
    return BSP_ERR_ALLOC;
  }
  b->probs = static_cast<DevProblem*>(b->dev);
  b->items = reinterpret_cast<int4*>(static_cast<char*>(b->dev) + poff);
  const cudaStream_t s = (cudaStream_t)stream;
  int st = BSP_OK;
  if (n > 0 && (e = cudaMemcpyAsync(b->probs, hp.data(), sizeof(DevProblem) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    st = cuda_status(e);
  if (st == BSP_OK && !items.empty() &&
      (e = cudaMemcpyAsync(b->items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    st = cuda_status(e);
  if (st == BSP_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) st = cuda_status(e);
  if (st != BSP_OK) {
    cudaFree(b->dev);
    delete b;
    return st;
  }
  int occ = 1;
  if (tn == 128) occ = b_dtype == BSP_BF16 ? batched_occupancy<__nv_bfloat16, 128>() : batched_occupancy<__half, 128>();
  else occ = b_dtype == BSP_BF16 ? batched_occupancy<__nv_bfloat16, 256>() : batched_occupancy<__half, 256>();
  b->grid = std::max(1, std::min(b->n_items, num_sms() * occ));
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
  if (!b) return BSP_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) return BSP_ERR_INVALID_ARG;
  if (b->n_items == 0 || b->N == 0) return BSP_OK;
  const cudaStream_t s = (cudaStream_t)stream;
  if (b->tn == 128)
    return b->bdt == BSP_BF16 ? launch_batched_t<__nv_bfloat16, 128>(b, s) : launch_batched_t<__half, 128>(b, s);
  return b->bdt == BSP_BF16 ? launch_batched_t<__nv_bfloat16, 256>(b, s) : launch_batched_t<__half, 256>(b, s);
}

}  // extern "C"
