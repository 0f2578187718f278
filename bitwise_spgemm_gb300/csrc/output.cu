// output.cu — the steps around the SpMM when the operands are themselves
// bitmaps or multi-bit values:
//
//  * symbolic output masks: for A (M×K) and B (K×N) both given as packed
//    bit rows, row i of C's mask is the OR of B's row masks at A's set bits
//    (the symbolic half of pre_spgemm, reference source/src/transform.cuh:
//    1028-1057, which walked a CSR copy of A one thread per row and kept the
//    mask in shared memory).  The first-fit grouping of the output rows that
//    follows it there is bsp_group_rows on the result.
//  * bit-plane products: C = Σ_b w_b · (P_b · B) for the 0/1 planes P_b of
//    an 8-bit matrix, w_b = 2^b and, for two's complement values, −2^7 for
//    the top plane — the recombination of spgemm_compute_1dthread_tcore_v3
//    (transform.cuh:2199-2246) with the weights of initialize_multiplicand
//    (main.cu:895-910).  There every plane went through a wmma tile of half
//    values and shared-memory atomics; here one warp walks the planes of a
//    row, sums each plane in FP32 (TwoSum compensated) and adds it, scaled by
//    its power-of-two weight (exact), to the row's total.
#include <climits>

#include "ptx.cuh"
#include "spmm_dev.cuh"

namespace bsp {
namespace {

constexpr int kSymWords = 4;  // output words per lane (128 per warp)
constexpr int kSymDepth = 8;  // B row masks in flight per warp

// One warp per (row of C, 128-word chunk of its mask).  The walker yields
// A's set bits in ascending order; columns at or past K (stray bits in the
// padding of A's last word) are ignored.
__global__ void __launch_bounds__(256) k_symbolic_rows(const uint32_t* __restrict__ A, int64_t M, int64_t K,
                                                       int64_t Kw, const uint32_t* __restrict__ Bw, int64_t Nw,
                                                       uint32_t* __restrict__ Cw) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= M) return;
  const int64_t w0 = (int64_t)blockIdx.y * (32 * kSymWords);
  uint32_t acc[kSymWords] = {};
  BitWalker wk;
  wk.init(A + row * Kw, 0, (int)Kw, lane);
  while (true) {
    uint32_t idx[kSymDepth];
#pragma unroll
    for (int s = 0; s < kSymDepth; s++) idx[s] = wk.next();
    if (idx[0] == kEnd) break;
    uint32_t v[kSymDepth][kSymWords];
#pragma unroll
    for (int s = 0; s < kSymDepth; s++)
#pragma unroll
      for (int q = 0; q < kSymWords; q++) {
        const int64_t w = w0 + q * 32 + lane;
        v[s][q] = (idx[s] != kEnd && (int64_t)idx[s] < K && w < Nw) ? __ldg(Bw + (int64_t)idx[s] * Nw + w) : 0u;
      }
#pragma unroll
    for (int s = 0; s < kSymDepth; s++)
#pragma unroll
      for (int q = 0; q < kSymWords; q++) acc[q] |= v[s][q];
    if (idx[kSymDepth - 1] == kEnd) break;
  }
#pragma unroll
  for (int q = 0; q < kSymWords; q++) {
    const int64_t w = w0 + q * 32 + lane;
    if (w < Nw) Cw[row * Nw + w] = acc[q];
  }
}

// ---- symbolic masks through a prototype plan ------------------------------
// For a row i of cluster c, the number of A_i's columns k whose B mask has
// column j set is  n_c[j] + #adds_i with j − #removes_i with j, where n_c
// counts over the cluster's consensus columns: every removed column is in
// the consensus, so the running count never goes below zero, and the mask
// bit is n > 0 — exact.  Counts are kept bit-sliced: plane p of a word holds
// bit p of its 32 columns' counts (16 planes: counts < 65536, which K <
// 65536 guarantees), so adding or removing one row's mask word is a ripple
// carry or borrow over the planes.  A row then reads its cluster's planes
// and its delta rows' masks (≈16 for the clustered workload) instead of the
// mask of every set bit (≈425).
constexpr int kSymPlanes = 16;
constexpr int kSymCWords = 64;   // output words per CTA of the plane kernel
constexpr int kSymCGroups = 8;   // consensus parts per CTA of the plane kernel
constexpr int kSymPWords = 2;    // output words per lane of the planned row kernel (64 per warp)

__device__ __forceinline__ void planes_add(uint32_t (&pl)[kSymPlanes], uint32_t x) {
#pragma unroll
  for (int p = 0; p < kSymPlanes; p++) {
    const uint32_t carry = pl[p] & x;
    pl[p] ^= x;
    x = carry;
    if (!x) break;
  }
}
__device__ __forceinline__ void planes_sub(uint32_t (&pl)[kSymPlanes], uint32_t x) {
#pragma unroll
  for (int p = 0; p < kSymPlanes; p++) {
    const uint32_t borrow = ~pl[p] & x;
    pl[p] ^= x;
    x = borrow;
    if (!x) break;
  }
}

// planes[c][p][w] for cluster c = blockIdx.x, words w of chunk blockIdx.y:
// thread (g, wl) counts its word's column bits over part g of the consensus
// columns (bit-sliced, 8 masks in flight), the parts meet as per-column
// counts in shared memory, and 64 threads write the planes of the total.
__global__ void __launch_bounds__(kSymCWords * kSymCGroups) k_sym_cluster_planes(
    const uint32_t* __restrict__ cons, int64_t Kw, int64_t K, const uint32_t* __restrict__ Bw, int64_t Nw,
    uint32_t* __restrict__ planes, int* __restrict__ top) {
  __shared__ int cnt[32][kSymCWords];
  const int lane = threadIdx.x & 31;
  const int g = threadIdx.x / kSymCWords, wl = threadIdx.x % kSymCWords;
  const int64_t c = blockIdx.x;
  const int64_t w = (int64_t)blockIdx.y * kSymCWords + wl;
  for (int i = threadIdx.x; i < 32 * kSymCWords; i += blockDim.x) (&cnt[0][0])[i] = 0;
  __syncthreads();
  uint32_t pl[kSymPlanes];
#pragma unroll
  for (int p = 0; p < kSymPlanes; p++) pl[p] = 0u;
  BitWalker wk;
  wk.init(cons + c * Kw, (int)(Kw * g / kSymCGroups), (int)(Kw * (g + 1) / kSymCGroups), lane);
  while (true) {
    uint32_t idx[kSymDepth], v[kSymDepth];
#pragma unroll
    for (int s = 0; s < kSymDepth; s++) idx[s] = wk.next();
    if (idx[0] == kEnd) break;
#pragma unroll
    for (int s = 0; s < kSymDepth; s++)
      v[s] = (idx[s] != kEnd && (int64_t)idx[s] < K && w < Nw) ? __ldg(Bw + (int64_t)idx[s] * Nw + w) : 0u;
#pragma unroll
    for (int s = 0; s < kSymDepth; s++) planes_add(pl, v[s]);
    if (idx[kSymDepth - 1] == kEnd) break;
  }
  int np = 0;  // this thread's planes in use
#pragma unroll
  for (int p = 0; p < kSymPlanes; p++)
    if (pl[p]) np = p + 1;
  if (np) {
    for (int b = 0; b < 32; b++) {
      int n = 0;
      for (int p = 0; p < np; p++) n |= (int)((pl[p] >> b) & 1u) << p;
      if (n) atomicAdd(&cnt[b][wl], n);
    }
  }
  __syncthreads();
  if (g == 0 && w < Nw) {
    int mx = 0;  // the largest count of this word's columns
    for (int b = 0; b < 32; b++) mx = max(mx, cnt[b][wl]);
    const int used = mx ? 32 - __clz(mx) : 0;  // planes up to the highest nonzero one
    for (int p = 0; p < kSymPlanes; p++) {
      uint32_t word = 0u;
      if (p < used)
        for (int b = 0; b < 32; b++) word |= (uint32_t)((cnt[b][wl] >> p) & 1) << b;
      planes[(c * kSymPlanes + p) * Nw + w] = word;
    }
    const int cu = __reduce_max_sync(__activemask(), used);
    if ((threadIdx.x & 31) == __ffs(__activemask()) - 1 && cu) atomicMax(top + c, cu);
  }
}

// One warp per (row of C, 64-word chunk): clustered rows start from their
// cluster's planes and apply their delta rows; other rows OR the masks of
// their set bits.
__global__ void __launch_bounds__(256, 4) k_sym_rows_planned(const uint32_t* __restrict__ A, int64_t M, int64_t K,
                                                          int64_t Kw, const uint32_t* __restrict__ Bw, int64_t Nw,
                                                          const int32_t* __restrict__ row_cluster,
                                                          const int32_t* __restrict__ delta_ptr,
                                                          const uint32_t* __restrict__ delta_idx,
                                                          const uint32_t* __restrict__ planes,
                                                          const int* __restrict__ top, uint32_t* __restrict__ Cw) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= M) return;
  const int64_t w0 = (int64_t)blockIdx.y * (32 * kSymPWords);
  int64_t wq[kSymPWords];
  bool wv[kSymPWords];
#pragma unroll
  for (int q = 0; q < kSymPWords; q++) {
    wq[q] = w0 + q * 32 + lane;
    wv[q] = wq[q] < Nw;
  }
  const int cl = __ldg(row_cluster + row);
  uint32_t out[kSymPWords];
  if (cl < 0) {
#pragma unroll
    for (int q = 0; q < kSymPWords; q++) out[q] = 0u;
    BitWalker wk;
    wk.init(A + row * Kw, 0, (int)Kw, lane);
    while (true) {
      uint32_t idx[kSymDepth];
#pragma unroll
      for (int s = 0; s < kSymDepth; s++) idx[s] = wk.next();
      if (idx[0] == kEnd) break;
#pragma unroll
      for (int s = 0; s < kSymDepth; s++)
#pragma unroll
        for (int q = 0; q < kSymPWords; q++)
          out[q] |= (idx[s] != kEnd && (int64_t)idx[s] < K && wv[q]) ? __ldg(Bw + (int64_t)idx[s] * Nw + wq[q]) : 0u;
      if (idx[kSymDepth - 1] == kEnd) break;
    }
  } else {
    // planes this row's counts can reach: the cluster's counts are below
    // 2^top, and the row adds at most one per delta entry
    const int d0 = __ldg(delta_ptr + row), d1 = __ldg(delta_ptr + row + 1);
    const uint32_t bound = ((1u << __ldg(top + cl)) - 1u) + (uint32_t)(d1 - d0);
    const int np = bound ? min(kSymPlanes, 32 - __clz(bound)) : 0;
    uint32_t pl[kSymPWords][kSymPlanes];
    const uint32_t* pc = planes + (int64_t)cl * kSymPlanes * Nw;
#pragma unroll
    for (int q = 0; q < kSymPWords; q++)
#pragma unroll
      for (int p = 0; p < kSymPlanes; p++) pl[q][p] = (wv[q] && p < np) ? __ldg(pc + (int64_t)p * Nw + wq[q]) : 0u;
    ListWalker wk;
    wk.init(delta_idx, d0, d1, lane);
    while (true) {
      uint32_t idx[kSymDepth];
#pragma unroll
      for (int s = 0; s < kSymDepth; s++) idx[s] = wk.next();
      if (idx[0] == kEnd) break;
      uint32_t v[kSymDepth][kSymPWords];
#pragma unroll
      for (int s = 0; s < kSymDepth; s++)
#pragma unroll
        for (int q = 0; q < kSymPWords; q++)
          v[s][q] = (idx[s] != kEnd && wv[q]) ? __ldg(Bw + (int64_t)(idx[s] & 0x7fffffffu) * Nw + wq[q]) : 0u;
#pragma unroll
      for (int s = 0; s < kSymDepth; s++) {
        if (idx[s] == kEnd) continue;
        const bool sub = (idx[s] >> 31) != 0u;
#pragma unroll
        for (int q = 0; q < kSymPWords; q++) {
          if (sub) planes_sub(pl[q], v[s][q]);
          else planes_add(pl[q], v[s][q]);
        }
      }
      if (idx[kSymDepth - 1] == kEnd) break;
    }
#pragma unroll
    for (int q = 0; q < kSymPWords; q++) {
      uint32_t m = 0u;
#pragma unroll
      for (int p = 0; p < kSymPlanes; p++) m |= pl[q][p];
      out[q] = m;
    }
  }
#pragma unroll
  for (int q = 0; q < kSymPWords; q++)
    if (wv[q]) Cw[row * Nw + wq[q]] = out[q];
}

struct PlaneArgs {
  const uint32_t* planes;  // [nplanes][M][Kw]
  int64_t M, K, Kw;
  int nplanes, signed_top;
  const void* B;
  int64_t ldb, N;
  float* C;
  int64_t ldc;
};

__device__ __forceinline__ float plane_weight(int b, int nplanes, int signed_top) {
  const float w = (float)(1u << b);
  return (signed_top && b == nplanes - 1) ? -w : w;
}

// One warp per (row, column chunk of 32*VPL*COLS), 16-byte vectors of B.
template <typename BT, int VPL, int D>
__global__ void __launch_bounds__(256) k_bitplane_rows(PlaneArgs a) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = 32 * VPL * COLS;
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= a.M) return;
  const int n0 = (int)blockIdx.y * CW;
  const BT* __restrict__ B = static_cast<const BT*>(a.B);
  int col[VPL];
  bool cvalid[VPL];
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    col[v] = n0 + (v * 32 + lane) * COLS;
    cvalid[v] = col[v] < a.N;
  }
  Acc<VPL, COLS, false> tot;
  tot.zero();
  for (int b = 0; b < a.nplanes; b++) {
    BitWalker wk;
    wk.init(a.planes + ((int64_t)b * a.M + row) * a.Kw, 0, (int)a.Kw, lane);
    Acc<VPL, COLS, true> acc;
    acc.zero();
    accumulate_walk<BT, VPL, D, true>(wk, B, a.ldb, col, cvalid, acc);
    const float w = plane_weight(b, a.nplanes, a.signed_top);
#pragma unroll
    for (int v = 0; v < VPL; v++)
#pragma unroll
      for (int j = 0; j < COLS; j++) tot.s[v][j] += w * acc.result(v, j);
  }
  store_vecs<VPL, COLS, false>(a.C + row * a.ldc, col, cvalid, tot, nullptr);
}

// Any layout: one warp per (row, 32 columns), a lane per column.
template <typename BT>
__global__ void __launch_bounds__(256) k_bitplane_rows_scalar(PlaneArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= a.M) return;
  const BT* __restrict__ B = static_cast<const BT*>(a.B);
  for (int64_t c0 = (int64_t)blockIdx.y * 32; c0 < a.N; c0 += (int64_t)gridDim.y * 32) {
    const int64_t c = c0 + lane;
    float tot = 0.f;
    for (int b = 0; b < a.nplanes; b++) {
      BitWalker wk;
      wk.init(a.planes + ((int64_t)b * a.M + row) * a.Kw, 0, (int)a.Kw, lane);
      float s = 0.f, e = 0.f;
      for (uint32_t k = wk.next(); k != kEnd; k = wk.next()) {
        const float x = c < a.N ? to_f32(B[(int64_t)k * a.ldb + c]) : 0.f;
        const float t = s + x, bp = t - s;
        e += (s - (t - bp)) + (x - bp);
        s = t;
      }
      tot += plane_weight(b, a.nplanes, a.signed_top) * (s + e);
    }
    if (c < a.N) a.C[row * a.ldc + c] = tot;
  }
}

template <typename BT>
int launch_planes_t(const PlaneArgs& a, bool vec, cudaStream_t s) {
  const unsigned gx = (unsigned)ceil_div(a.M, 8);
  if (!vec) {
    const int64_t gy = ceil_div(a.N, 32) < 65535 ? ceil_div(a.N, 32) : 65535;
    k_bitplane_rows_scalar<BT><<<dim3(gx, (unsigned)gy), 256, 0, s>>>(a);
  } else {
    constexpr int COLS = Vec<BT>::COLS;
    constexpr int VPL = COLS == 4 ? 2 : 1;
    const int64_t gy = ceil_div(a.N, 32 * VPL * COLS);
    if (gy > 65535) return BSP_ERR_CAPACITY;
    k_bitplane_rows<BT, VPL, 8><<<dim3(gx, (unsigned)gy), 256, 0, s>>>(a);
  }
  BSP_LAUNCHED();
  return BSP_OK;
}

// B stacked for the planes-along-K form: row b*Kp + k of out is w_b·B[k]
// (k < K) or 0 (K ≤ k < Kp, Kp = 32·ceil(K/32)).  A power-of-two factor
// only changes the exponent, so the 16-bit values stay exact.  A CTA per
// output row (grid-stride), its threads along the columns.
template <typename BT>
__global__ void __launch_bounds__(256) k_stack_planes_b(const BT* __restrict__ B, int64_t ldb, int64_t K,
                                                        int64_t Kp, int64_t N, int nplanes, int signed_top,
                                                        BT* __restrict__ out, int64_t ldo) {
  const int64_t rows = (int64_t)nplanes * Kp;
  for (int64_t rr = blockIdx.x; rr < rows; rr += gridDim.x) {
    const int b = (int)(rr / Kp);
    const int64_t k = rr - (int64_t)b * Kp;
    const float w = plane_weight(b, nplanes, signed_top);
    BT* o = out + rr * ldo;
    if (k < K) {
      const BT* src = B + k * ldb;
      for (int64_t c = threadIdx.x; c < N; c += blockDim.x) o[c] = from_f32<BT>(to_f32(src[c]) * w);
    } else {
      for (int64_t c = threadIdx.x; c < N; c += blockDim.x) o[c] = from_f32<BT>(0.f);
    }
  }
}

}  // namespace

int launch_stack_planes_b(const void* B, int bdt, int64_t ldb, int64_t K, int64_t N, int nplanes, int signed_top,
                          void* out, int64_t ldo, cudaStream_t s) {
  const int64_t Kp = ceil_div(K, 32) * 32;
  const int64_t total = (int64_t)nplanes * Kp * N;
  if (total == 0) return BSP_OK;
  const int64_t rows = (int64_t)nplanes * Kp, cap = (int64_t)num_sms() * 32;
  const unsigned grid = (unsigned)(rows < cap ? rows : cap);
  if (bdt == BSP_F32)
    k_stack_planes_b<float><<<grid, 256, 0, s>>>((const float*)B, ldb, K, Kp, N, nplanes, signed_top, (float*)out, ldo);
  else if (bdt == BSP_BF16)
    k_stack_planes_b<__nv_bfloat16><<<grid, 256, 0, s>>>((const __nv_bfloat16*)B, ldb, K, Kp, N, nplanes, signed_top,
                                                         (__nv_bfloat16*)out, ldo);
  else if (bdt == BSP_F16)
    k_stack_planes_b<__half><<<grid, 256, 0, s>>>((const __half*)B, ldb, K, Kp, N, nplanes, signed_top, (__half*)out,
                                                  ldo);
  else
    return BSP_ERR_UNSUPPORTED;
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_symbolic_rows(const uint32_t* A, int64_t M, int64_t K, const uint32_t* Bw, int64_t N, uint32_t* Cw,
                         cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32), Nw = ceil_div(N, 32);
  const int64_t gy = ceil_div(Nw, 32 * kSymWords);
  if (M == 0 || Nw == 0) return BSP_OK;
  if (gy > 65535) return BSP_ERR_CAPACITY;
  k_symbolic_rows<<<dim3((unsigned)ceil_div(M, 8), (unsigned)gy), 256, 0, s>>>(A, M, K, Kw, Bw, Nw, Cw);
  BSP_LAUNCHED();
  return BSP_OK;
}

size_t symbolic_planes_bytes(int64_t n_proto, int64_t N) {
  // planes, then one int per cluster: the number of planes in use
  const size_t pb = sizeof(uint32_t) * (size_t)n_proto * kSymPlanes * (size_t)ceil_div(N, 32);
  return ((pb + 255) & ~size_t(255)) + sizeof(int) * (size_t)n_proto;
}

int launch_symbolic_planned(const uint32_t* A, int64_t M, int64_t K, const uint32_t* Bw, int64_t N, uint32_t* Cw,
                            const int32_t* row_cluster, const int32_t* delta_ptr, const uint32_t* delta_idx,
                            const uint32_t* cons, int64_t n_proto, uint32_t* planes, cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32), Nw = ceil_div(N, 32);
  if (M == 0 || Nw == 0) return BSP_OK;
  const int64_t gpy = ceil_div(Nw, kSymCWords), gry = ceil_div(Nw, 32 * kSymPWords);
  if (gpy > 65535 || gry > 65535 || n_proto > INT32_MAX) return BSP_ERR_CAPACITY;
  const size_t pb = sizeof(uint32_t) * (size_t)n_proto * kSymPlanes * (size_t)Nw;
  int* top = reinterpret_cast<int*>(reinterpret_cast<uint8_t*>(planes) + ((pb + 255) & ~size_t(255)));
  if (n_proto > 0) {
    BSP_CUDA(cudaMemsetAsync(top, 0, sizeof(int) * (size_t)n_proto, s));
    k_sym_cluster_planes<<<dim3((unsigned)n_proto, (unsigned)gpy), kSymCWords * kSymCGroups, 0, s>>>(cons, Kw, K, Bw,
                                                                                                    Nw, planes, top);
  }
  k_sym_rows_planned<<<dim3((unsigned)ceil_div(M, 8), (unsigned)gry), 256, 0, s>>>(
      A, M, K, Kw, Bw, Nw, row_cluster, delta_ptr, delta_idx, planes, top, Cw);
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_bitplane_spmm(const uint32_t* planes, int nplanes, int signed_top, int64_t M, int64_t K,
                         const void* B, int bdt, int64_t ldb, int64_t N, float* C, int64_t ldc, bool vec,
                         cudaStream_t s) {
  if (M == 0 || N == 0) return BSP_OK;
  PlaneArgs a = {planes, M, K, ceil_div(K, 32), nplanes, signed_top, B, ldb, N, C, ldc};
  if (bdt == BSP_F32) return launch_planes_t<float>(a, vec, s);
  if (bdt == BSP_BF16) return launch_planes_t<__nv_bfloat16>(a, vec, s);
  if (bdt == BSP_F16) return launch_planes_t<__half>(a, vec, s);
  return BSP_ERR_UNSUPPORTED;
}

}  // namespace bsp
