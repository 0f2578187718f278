// group.cu — reference-compatible first-fit row grouping, group→dense scatter
// and a device-wide exclusive scan used by the plan builder.
#include "bsp_internal.cuh"

namespace bsp {
namespace {

// One warp per tile t = rb*Kw + w (rows rb*TR .. rb*TR+TR-1, word column w).
// Lane g < G holds group g's mask.  Rows are visited in ascending order —
// the deterministic serialisation of generate_groups_large's atomicCAS race
// (reference source/src/main.cu:110-180): a zero word joins group 0 without
// touching the masks (:105-108); otherwise one ballot finds the first group
// whose mask does not intersect the word; if none, the row spills.
__global__ void __launch_bounds__(256) k_group_rows(const uint32_t* __restrict__ words, int64_t M,
                                                    int64_t Kw, int TR, int G,
                                                    int32_t* __restrict__ group_id,
                                                    uint32_t* __restrict__ group_mask,
                                                    int32_t* __restrict__ group_row,
                                                    int32_t* __restrict__ spill_cnt,
                                                    int32_t* __restrict__ spill_nnz,
                                                    int32_t* __restrict__ spill_rows,
                                                    unsigned long long* __restrict__ grouped_nnz,
                                                    int64_t n_tiles) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp; t < n_tiles; t += nwarps) {
    const int64_t rb = t / Kw;
    const int64_t w = t - rb * Kw;
    const int64_t row0 = rb * TR;
    if (group_row)
      for (int i = lane; i < G * 32; i += 32) group_row[t * G * 32 + i] = -1;
    if (spill_rows)
      for (int i = lane; i < TR; i += 32) spill_rows[t * TR + i] = -1;
    __syncwarp();
    uint32_t gm = 0;  // lane g < G: mask of group g
    int nsp = 0, nspnnz = 0;
    for (int c0 = 0; c0 < TR; c0 += 32) {
      const int64_t r = row0 + c0 + lane;
      const bool valid = (c0 + lane < TR) && (r < M);
      const uint32_t my = valid ? words[r * Kw + w] : 0u;
      int myg = 0;
      uint32_t pending = __ballot_sync(kFull, my != 0u);
      while (pending) {
        const int src = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t m = __shfl_sync(kFull, my, src);
        const uint32_t conflict = __ballot_sync(kFull, lane >= G || (gm & m) != 0u);
        const int g = (~conflict) ? __ffs(~conflict) - 1 : -1;
        if (g >= 0) {
          if (lane == g) gm |= m;
          if (group_row && ((m >> lane) & 1u))
            group_row[(t * G + g) * 32 + lane] = c0 + src;
        } else {
          if (spill_rows && lane == 0) spill_rows[t * TR + nsp] = c0 + src;
          nsp++;
          nspnnz += __popc(m);
        }
        if (lane == src) myg = g;
      }
      if (valid) group_id[r * Kw + w] = myg;
    }
    if (lane < G) group_mask[t * G + lane] = gm;
    int pc = lane < G ? __popc(gm) : 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) pc += __shfl_xor_sync(kFull, pc, o);
    if (lane == 0) {
      if (spill_cnt) spill_cnt[t] = nsp;
      if (spill_nnz) spill_nnz[t] = nspnnz;
      if (grouped_nnz) atomicAdd(grouped_nnz, (unsigned long long)pc);
    }
  }
}

// Warp per (row, word), lane = bit: the scatter of group2dense
// (reference source/src/main.cu:829-850) with LSB-first bits.
__global__ void __launch_bounds__(256) k_group_to_dense(const float* __restrict__ gv,
                                                        const int32_t* __restrict__ gid,
                                                        const uint32_t* __restrict__ words,
                                                        int64_t M, int64_t K, int64_t Kw, int TR,
                                                        int G, float* __restrict__ dense,
                                                        int64_t ldd) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp; t < M * Kw; t += nwarps) {
    const int64_t r = t / Kw;
    const int64_t w = t - r * Kw;
    const int g = gid[t];
    if (g < 0) continue;
    const uint32_t m = words[t];
    const int64_t c = w * 32 + lane;
    if (((m >> lane) & 1u) && c < K) {
      const int64_t tile = (r / TR) * Kw + w;
      dense[r * ldd + c] = gv[(tile * G + g) * 32 + lane];
    }
  }
}

// ---- exclusive scan ------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int32_t* __restrict__ in, int64_t n,
                                                              int32_t* __restrict__ bsum) {
  __shared__ int sw[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  int s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + (int64_t)threadIdx.x * kScanItems + j;
    s += i < n ? in[i] : 0;
  }
  int total;
  block_exclusive_scan(s, sw, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(int32_t* __restrict__ bsum, int64_t nb,
                                                              int32_t* __restrict__ out_total) {
  __shared__ int sw[32];
  int carry = 0;
  for (int64_t c0 = 0; c0 < nb; c0 += kScanThreads) {
    const int64_t i = c0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    int total;
    const int ex = block_exclusive_scan(v, sw, &total);
    if (i < nb) bsum[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *out_total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int32_t* __restrict__ in, int64_t n,
                                                             const int32_t* __restrict__ boff,
                                                             int32_t* __restrict__ out) {
  __shared__ int sw[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + (int64_t)threadIdx.x * kScanItems + j;
    v[j] = i < n ? in[i] : 0;
    s += v[j];
  }
  int total;
  int run = block_exclusive_scan(s, sw, &total) + boff[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + (int64_t)threadIdx.x * kScanItems + j;
    if (i < n) out[i] = run;
    run += v[j];
  }
}

// Small inputs: one CTA walks the tiles in order with a running carry, so
// the scan is one launch instead of three.
constexpr int kScanSingleThreads = 1024;
constexpr int64_t kScanSingleMax = 32768;
__global__ void __launch_bounds__(kScanSingleThreads) k_scan_single(const int32_t* __restrict__ in, int64_t n,
                                                                    int32_t* __restrict__ out) {
  __shared__ int sw[32];
  constexpr int TILE = kScanSingleThreads * kScanItems;
  int carry = 0;
  for (int64_t base = 0; base < n; base += TILE) {
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
      const int64_t i = base + (int64_t)threadIdx.x * kScanItems + j;
      v[j] = i < n ? in[i] : 0;
      s += v[j];
    }
    int total;
    int run = block_exclusive_scan(s, sw, &total) + carry;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
      const int64_t i = base + (int64_t)threadIdx.x * kScanItems + j;
      if (i < n) out[i] = run;
      run += v[j];
    }
    carry += total;
  }
  if (threadIdx.x == 0) out[n] = carry;
}

int grid_for(int64_t warps_needed) {
  const int64_t blocks = ceil_div(warps_needed, 8);
  const int64_t cap = (int64_t)num_sms() * 16;
  return (int)(blocks < 1 ? 1 : (blocks > cap ? cap : blocks));
}

}  // namespace

int launch_group_rows(const uint32_t* words, int64_t M, int64_t Kw, int tile_rows,
                      int max_groups, int32_t* group_id, uint32_t* group_mask,
                      int32_t* group_row, int32_t* spill_cnt, int32_t* spill_nnz,
                      int32_t* spill_rows, int64_t* grouped_nnz, cudaStream_t s) {
  const int64_t n_tiles = ceil_div(M, tile_rows) * Kw;
  if (grouped_nnz) BSP_CUDA(cudaMemsetAsync(grouped_nnz, 0, sizeof(int64_t), s));
  if (n_tiles == 0) return BSP_OK;
  k_group_rows<<<grid_for(n_tiles), 256, 0, s>>>(words, M, Kw, tile_rows, max_groups, group_id,
                                                 group_mask, group_row, spill_cnt, spill_nnz,
                                                 spill_rows, (unsigned long long*)grouped_nnz,
                                                 n_tiles);
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_group_to_dense(const float* gv, const int32_t* gid, const uint32_t* words, int64_t M,
                          int64_t K, int tile_rows, int max_groups, float* dense, int64_t ldd,
                          cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32);
  if (M * Kw == 0) return BSP_OK;
  k_group_to_dense<<<grid_for(M * Kw), 256, 0, s>>>(gv, gid, words, M, K, Kw, tile_rows,
                                                    max_groups, dense, ldd);
  BSP_LAUNCHED();
  return BSP_OK;
}

size_t scan_workspace_bytes(int64_t n) {
  return sizeof(int32_t) * (size_t)(ceil_div(n, kScanTile) + 1);
}

int launch_scan_i32(const int32_t* in, int64_t n, int32_t* out, void* ws, cudaStream_t s) {
  const int64_t nb = ceil_div(n, kScanTile);
  if (nb == 0) {
    BSP_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), s));
    return BSP_OK;
  }
  if (n <= kScanSingleMax) {
    k_scan_single<<<1, kScanSingleThreads, 0, s>>>(in, n, out);
    BSP_LAUNCHED();
    return BSP_OK;
  }
  int32_t* bsum = static_cast<int32_t*>(ws);
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, bsum);
  k_scan_blocks<<<1, kScanThreads, 0, s>>>(bsum, nb, out + n);
  k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, bsum, out);
  BSP_LAUNCHED();
  return BSP_OK;
}

}  // namespace bsp
