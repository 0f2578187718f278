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
//     operand (K-major core-matrix layout) and stream the 32x256 B tile with
//     16-byte cp.async into the MN-major core-matrix layout; then, after the
//     last stage, read the accumulator back with tcgen05.ld and store C;
//   warp 4: allocates TMEM; its lane 0 issues two tcgen05.mma (K=16) per
//     stage and commits them to the stage's "empty" mbarrier.
// Four stages of 24 KB; every mbarrier wait is bounded (timeout → error 3
// in g_tc_error, the CTA skips to freeing its TMEM).
#include <type_traits>

#include "ptx.cuh"
#include "spmm_dev.cuh"

namespace bsp {

__device__ int g_tc_error;

namespace {

constexpr int kTcM = 128;
constexpr int kTcN = 256;
constexpr int kTcK = 32;
constexpr int kStages = 4;
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
// Operands are stored as 8x16-byte core matrices (no swizzle).  In both
// descriptors the leading byte offset (LBO) is the distance between core
// matrices adjacent along K and the stride byte offset (SBO) the distance
// between core matrices adjacent along M (A) or N (B) — measured on GB300
// with one-hot A rows and position-encoding B values.
// A (K-major):  element (m, k) at (m/8)*kASbo + (k/8)*kALbo + (m%8)*16 + (k%8)*2
constexpr uint32_t kALbo = 128, kASbo = 512;
// B (MN-major): element (k, n) at (n/8)*kBSbo + (k/8)*kBLbo + (k%8)*16 + (n%8)*2
constexpr uint32_t kBLbo = 128, kBSbo = 512;

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

// Instruction descriptor for kind::f16: D f32, A and B of the same 16-bit
// type (bf16 = 1, f16 = 0), A K-major, B MN-major, N = 256, M = 128.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t ab_type) {
  return (1u << 4) | (ab_type << 7) | (ab_type << 10) | (0u << 15) | (1u << 16) |
         ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
}

// 8 bits of a word → 8 16-bit values 0 / one, packed little-endian.
__device__ __forceinline__ uint4 expand8(uint32_t byte, uint32_t one) {
  uint32_t w[4];
#pragma unroll
  for (int j = 0; j < 4; j++)
    w[j] = (((byte >> (2 * j)) & 1u) ? one : 0u) | ((((byte >> (2 * j + 1)) & 1u) ? one : 0u) << 16);
  return make_uint4(w[0], w[1], w[2], w[3]);
}

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

template <typename BT>
__global__ void __launch_bounds__(kTcThreads, 1) k_spmm_tc(SpmmArgs a, const uint32_t* __restrict__ occ,
                                                          int occ_words) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * kTcM;
  const int n0 = (int)blockIdx.y * kTcN;
  const uint32_t one = std::is_same<BT, __nv_bfloat16>::value ? 0x3f80u : 0x3c00u;
  const uint32_t* block_occ = occ + (int64_t)blockIdx.x * occ_words;

  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      ptx::mbar_init(&sm.full[s], kProducers);
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
  ptx::tc_fence_before_sync();
  __syncthreads();
  ptx::tc_fence_after_sync();
  const uint32_t tmem = sm.tmem_addr;
  int ntiles = 0;

  if (warp < 4) {
    // ---------------- producers ----------------
    const BT* __restrict__ B = static_cast<const BT*>(a.B);
    const int64_t arow = row0 + tid;
    const uint32_t* awords = a.A + arow * a.Kw;
    TileIter it;
    it.init(block_occ, occ_words);
    int i = 0;
    for (int kt = it.next(); kt >= 0; kt = it.next(), i++) {
      const int s = i % kStages;
      if (i >= kStages && !ptx::mbar_wait(&sm.empty[s], ((i / kStages) - 1) & 1)) {
        atomicCAS(&g_tc_error, 0, 3);
        sm.abort = 1;
        break;
      }
      if (*(volatile int*)&sm.abort) break;
      // A operand: row tid, 32 columns → 4 core-matrix rows of 8 values
      const uint32_t w = arow < a.M ? __ldg(awords + kt) : 0u;
      uint8_t* as = sm.a[s] + (tid >> 3) * kASbo + (tid & 7) * 16;
#pragma unroll
      for (int c = 0; c < 4; c++)
        *reinterpret_cast<uint4*>(as + c * kALbo) = expand8((w >> (8 * c)) & 0xffu, one);
      // B tile rows k0..k0+31, columns n0..n0+255: 1024 chunks of 16 bytes
      const int64_t k0 = (int64_t)kt * kTcK;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int q = tid + kProducers * j;
        const int k = q >> 5, n8 = q & 31;
        const int64_t krow = k0 + k;
        const int ncol = n0 + n8 * 8;
        const bool ok = krow < a.K && ncol < a.N;
        const BT* src = ok ? B + krow * a.ldb + ncol : B;
        ptx::cp_async_16(sm.b[s] + n8 * kBSbo + (k >> 3) * kBLbo + (k & 7) * 16, src, ok ? 16u : 0u);
      }
      ptx::cp_async_commit();
      // stage i-2 is now complete: publish it to the MMA issuer
      ptx::cp_async_wait_group<2>();
      if (i >= 2) {
        ptx::fence_proxy_async_smem();
        ptx::mbar_arrive(&sm.full[(i - 2) % kStages]);
      }
    }
    ntiles = i;
    ptx::cp_async_wait_group<0>();
    ptx::fence_proxy_async_smem();
    for (int j = (ntiles >= 2 ? ntiles - 2 : 0); j < ntiles; j++) ptx::mbar_arrive(&sm.full[j % kStages]);
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = idesc_f16(std::is_same<BT, __nv_bfloat16>::value ? 1u : 0u);
    TileIter it;
    it.init(block_occ, occ_words);
    int i = 0;
    for (int kt = it.next(); kt >= 0; kt = it.next(), i++) {
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
        const uint64_t ad = ptx::smem_desc_noswizzle(sm.a[s] + j * 2 * kALbo, kALbo, kASbo);
        const uint64_t bd = ptx::smem_desc_noswizzle(sm.b[s] + j * 2 * kBLbo, kBLbo, kBSbo);
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
    float* crow = a.C + row * a.ldc + n0;
    const bool live = row < a.M && ok && !*(volatile int*)&sm.abort;
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
      if (live) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int col = (c8 + u) * 8;
          if (n0 + col < a.N) {
            *reinterpret_cast<float4*>(crow + col) =
                make_float4(__uint_as_float(r[u][0]), __uint_as_float(r[u][1]), __uint_as_float(r[u][2]),
                            __uint_as_float(r[u][3]));
            *reinterpret_cast<float4*>(crow + col + 4) =
                make_float4(__uint_as_float(r[u][4]), __uint_as_float(r[u][5]), __uint_as_float(r[u][6]),
                            __uint_as_float(r[u][7]));
          }
        }
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

int launch_tile_occupancy(const uint32_t* A, int64_t M, int64_t K, uint32_t* occ,
                          unsigned long long* count, cudaStream_t s) {
  const int ow = tc_occupancy_words(K);
  const int64_t warps = ceil_div(M, kTcM) * ow;
  if (warps == 0) return BSP_OK;
  k_tile_occupancy<<<(unsigned)ceil_div(warps, 8), 256, 0, s>>>(A, M, ceil_div(K, 32), ow, occ, count);
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_spmm_tc(const SpmmArgs& a, const uint32_t* occ, cudaStream_t s) {
  if (a.M == 0 || a.N == 0) return BSP_OK;
  const size_t smem = sizeof(TcSmem);
  const dim3 grid((unsigned)ceil_div(a.M, kTcM), (unsigned)ceil_div(a.N, kTcN));
  if (grid.y > 65535) return BSP_ERR_CAPACITY;
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  static bool configured[2][64] = {};
  const int t = a.bdt == BSP_BF16 ? 0 : 1;
  if (dev < 64 && !configured[t][dev]) {
    if (t == 0)
      BSP_CUDA(cudaFuncSetAttribute(k_spmm_tc<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    else
      BSP_CUDA(cudaFuncSetAttribute(k_spmm_tc<__half>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured[t][dev] = true;
  }
  const int ow = tc_occupancy_words(a.K);
  if (t == 0) k_spmm_tc<__nv_bfloat16><<<grid, kTcThreads, smem, s>>>(a, occ, ow);
  else k_spmm_tc<__half><<<grid, kTcThreads, smem, s>>>(a, occ, ow);
  BSP_LAUNCHED();
  return BSP_OK;
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
