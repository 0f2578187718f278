// formats.cu — interchange formats next to the packed-row layout.
//
//  * 8x8 bitmap tiles (the tSparse format the reference builds in
//    coo2bmp_noTuple_d, source/src/main.cu:692-779, with find_tile_index,
//    source/src/mm.h:83-104): one uint64 per nonzero 8x8 tile, bit
//    (r%8)*8 + c%8, tiles in ascending tile_row*ceil(K/8)+tile_col order, and
//    the exclusive scan of their popcounts (the offsets of each tile's values).
//    The reference got there with three thrust sorts of the COO entries; from
//    packed rows a tile is eight bytes already in place (byte tx of row r is
//    the tile's row r%8), so one pass builds every tile, a scan compacts them.
//  * tiled CSR (csr2tiledcsr, main.cu:499-588, one serial thread there): the
//    entries of each (tile_rows x tile_cols) tile contiguous, tiles in
//    row-major order, rows in order inside a tile and CSR order inside a
//    row, with local columns, a local row pointer per tile and the exclusive
//    scan of the tiles' entry counts.  Here a warp per CSR row ranks its
//    entries within their (row, tile) runs (match_any + one atomicAdd per
//    run, so CSR order is kept), a block scan per tile turns the per-row
//    counts into the local row pointer, and a second warp-per-row pass
//    scatters.
#include "bsp_internal.cuh"

namespace bsp {
size_t scan_workspace_bytes(int64_t n);

namespace {

// Every 8x8 tile: bitmap, and 1 / 0 for the compaction scan.
__global__ void __launch_bounds__(256) k_tiles8_build(const uint32_t* __restrict__ words, int64_t M, int64_t Kw,
                                                      int64_t Mt, int64_t Kt, uint64_t* __restrict__ all,
                                                      int32_t* __restrict__ flag) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Mt * Kt) return;
  const int64_t ty = t / Kt, tx = t - ty * Kt;
  uint64_t m = 0;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int64_t row = ty * 8 + r;
    if (row < M) {
      const uint32_t w = __ldg(words + row * Kw + (tx >> 2));
      m |= (uint64_t)((w >> (8 * (tx & 3))) & 0xffu) << (8 * r);
    }
  }
  all[t] = m;
  flag[t] = m != 0ull;
}

// Nonzero tiles to their compacted slots; pc[p] = popcount (pc zeroed first).
__global__ void __launch_bounds__(256) k_tiles8_scatter(const uint64_t* __restrict__ all,
                                                        const int32_t* __restrict__ pos, int64_t Kt, int64_t T,
                                                        uint64_t* __restrict__ bmp, int32_t* __restrict__ trow,
                                                        int32_t* __restrict__ tcol, int32_t* __restrict__ pc,
                                                        int64_t* __restrict__ n_tiles) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) *n_tiles = pos[T];
  if (t >= T) return;
  const uint64_t m = all[t];
  if (!m) return;
  const int p = pos[t];
  bmp[p] = m;
  trow[p] = (int32_t)(t / Kt);
  tcol[p] = (int32_t)(t % Kt);
  pc[p] = __popcll(m);
}

// Tile bytes back into packed rows (rows zeroed first).  Byte tx of a row's
// words is columns 8tx..8tx+7 (LSB-first, little-endian); tiles outside the
// matrix are skipped.
__global__ void __launch_bounds__(256) k_tiles8_to_rows(const uint64_t* __restrict__ bmp,
                                                        const int32_t* __restrict__ trow,
                                                        const int32_t* __restrict__ tcol, int64_t n, int64_t M,
                                                        int64_t K, int64_t Kw, uint8_t* __restrict__ bytes) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t ty = __ldg(trow + t), tx = __ldg(tcol + t);
  if (ty < 0 || tx < 0 || tx * 8 >= K || ty * 8 >= M) return;
  const uint64_t m = __ldg(bmp + t);
  const int keep = K - tx * 8 >= 8 ? 0xff : (1 << (K - tx * 8)) - 1;  // no bits past column K-1
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int64_t row = ty * 8 + r;
    const uint8_t b = (uint8_t)((m >> (8 * r)) & (uint64_t)keep);
    if (row < M && b) bytes[row * Kw * 4 + tx] = b;
  }
}

// Rank of every CSR entry within its (row, tile column) run, in CSR order;
// cnt[row*Kt + tx] ends as the run's length.  Entries with a column outside
// [0, K) get rank -1 and are left out everywhere.
__global__ void __launch_bounds__(256) k_csr_rank(const int32_t* __restrict__ row_ptr,
                                                  const int32_t* __restrict__ col, int64_t M, int64_t K, int tc,
                                                  int64_t Kt, int32_t* __restrict__ cnt, int32_t* __restrict__ rank) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= M) return;
  const int32_t b = __ldg(row_ptr + i), e = __ldg(row_ptr + i + 1);
  for (int32_t j0 = b; j0 < e; j0 += 32) {
    const int32_t j = j0 + lane;
    const int32_t c = j < e ? __ldg(col + j) : -1;
    const bool ok = j < e && c >= 0 && c < K;
    const int key = ok ? c / tc : -1;
    const unsigned grp = __match_any_sync(kFull, key);
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (ok && lane == leader) base = atomicAdd(cnt + i * Kt + key, __popc(grp));
    base = __shfl_sync(kFull, base, leader);
    if (j < e) rank[j] = ok ? base + __popc(grp & ((1u << lane) - 1u)) : -1;
  }
}

// One CTA per tile: the local row pointer (tile_rows+1 values) as a block
// scan of the rows' counts in chunks of 256 rows, and the tile's entry count.
__global__ void __launch_bounds__(256) k_tiled_offsets(const int32_t* __restrict__ cnt, int64_t M, int tr,
                                                       int64_t Kt, int32_t* __restrict__ toff,
                                                       int32_t* __restrict__ tnnz) {
  __shared__ int32_t wsum[8];
  const int64_t t = blockIdx.x;
  const int64_t ty = t / Kt, tx = t - ty * Kt;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t* o = toff + t * (tr + 1);
  int32_t carry = 0;
  for (int j0 = 0; j0 < tr; j0 += 256) {
    const int j = j0 + threadIdx.x;
    const int64_t row = ty * tr + j;
    const int32_t v = (j < tr && row < M) ? __ldg(cnt + row * Kt + tx) : 0;
    int32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t y = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    int32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) {
      const int32_t x = wsum[w];
      before += w < wid ? x : 0;
      total += x;
    }
    if (j < tr) o[j] = carry + before + incl - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    o[tr] = carry;
    tnnz[t] = carry;
  }
}

__global__ void __launch_bounds__(256) k_csr_fill(const int32_t* __restrict__ row_ptr,
                                                  const int32_t* __restrict__ col, const uint8_t* __restrict__ val,
                                                  int vbytes, int64_t M, int tr, int tc, int64_t Kt,
                                                  const int32_t* __restrict__ rank, const int32_t* __restrict__ acc,
                                                  const int32_t* __restrict__ toff, int32_t* __restrict__ tcol,
                                                  uint8_t* __restrict__ tval) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= M) return;
  const int64_t ty = i / tr;
  const int lr = (int)(i - ty * tr);
  const int32_t b = __ldg(row_ptr + i), e = __ldg(row_ptr + i + 1);
  for (int32_t j = b + lane; j < e; j += 32) {
    const int32_t rk = rank[j];
    if (rk < 0) continue;
    const int32_t c = __ldg(col + j);
    const int64_t t = ty * Kt + c / tc;
    const int64_t p = (int64_t)acc[t] + toff[t * (tr + 1) + lr] + rk;
    tcol[p] = c % tc;
    if (val && tval)
      for (int q = 0; q < vbytes; q++) tval[p * vbytes + q] = val[(int64_t)j * vbytes + q];
  }
}

}  // namespace

size_t tiles8_workspace_bytes(int64_t M, int64_t K) {
  const int64_t T = ceil_div(M, 8) * ceil_div(K, 8);
  // all[T] u64, flag[T], pos[T+1], pc[T] int32, scan blocks
  return (size_t)T * 8 + 3 * ((size_t)T + 1) * 4 + scan_workspace_bytes(T) + 4 * 256;
}

static inline uint8_t* carve(uint8_t*& p, size_t bytes) {
  uint8_t* r = p;
  p += (bytes + 255) & ~(size_t)255;
  return r;
}

int launch_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K, uint64_t* bmp, int32_t* trow, int32_t* tcol,
                          int32_t* offset, int64_t* n_tiles, void* ws, cudaStream_t s) {
  const int64_t Mt = ceil_div(M, 8), Kt = ceil_div(K, 8), T = Mt * Kt, Kw = ceil_div(K, 32);
  uint8_t* p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
  uint64_t* all = reinterpret_cast<uint64_t*>(carve(p, (size_t)T * 8));
  int32_t* flag = reinterpret_cast<int32_t*>(carve(p, (size_t)T * 4));
  int32_t* pos = reinterpret_cast<int32_t*>(carve(p, ((size_t)T + 1) * 4));
  int32_t* pc = reinterpret_cast<int32_t*>(carve(p, ((size_t)T + 1) * 4));
  void* sws = carve(p, scan_workspace_bytes(T));
  const unsigned g = (unsigned)ceil_div(T, 256);
  k_tiles8_build<<<g, 256, 0, s>>>(words, M, Kw, Mt, Kt, all, flag);
  BSP_LAUNCHED();
  BSP_TRY(launch_scan_i32(flag, T, pos, sws, s));
  BSP_CUDA(cudaMemsetAsync(pc, 0, (size_t)T * 4, s));
  k_tiles8_scatter<<<g, 256, 0, s>>>(all, pos, Kt, T, bmp, trow, tcol, pc, n_tiles);
  BSP_LAUNCHED();
  // offsets over all T slots: past the n-th they stay at the total
  return launch_scan_i32(pc, T, offset, sws, s);
}

int launch_tiles8_to_rows(const uint64_t* bmp, const int32_t* trow, const int32_t* tcol, int64_t n, int64_t M,
                          int64_t K, uint32_t* words, cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32);
  BSP_CUDA(cudaMemsetAsync(words, 0, sizeof(uint32_t) * (size_t)M * (size_t)Kw, s));
  if (n == 0) return BSP_OK;
  k_tiles8_to_rows<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(bmp, trow, tcol, n, M, K, Kw,
                                                              reinterpret_cast<uint8_t*>(words));
  BSP_LAUNCHED();
  return BSP_OK;
}

size_t csr_tiled_workspace_bytes(int64_t M, int64_t K, int64_t nnz, int tile_rows, int tile_cols) {
  const int64_t Kt = ceil_div(K, tile_cols), T = ceil_div(M, tile_rows) * Kt;
  // cnt[M*Kt], rank[nnz], tnnz[T] int32, scan blocks
  return ((size_t)M * Kt + (size_t)nnz + (size_t)T) * 4 + scan_workspace_bytes(T) + 4 * 256;
}

int launch_csr_to_tiled(const int32_t* row_ptr, const int32_t* col, const void* val, int vbytes, int64_t M,
                        int64_t K, int64_t nnz, int tr, int tc, int32_t* acc, int32_t* toff, int32_t* tcol,
                        void* tval, void* ws, cudaStream_t s) {
  const int64_t Kt = ceil_div(K, tc), T = ceil_div(M, tr) * Kt;
  uint8_t* p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
  int32_t* cnt = reinterpret_cast<int32_t*>(carve(p, (size_t)M * Kt * 4));
  int32_t* rank = reinterpret_cast<int32_t*>(carve(p, (size_t)(nnz > 0 ? nnz : 1) * 4));
  int32_t* tnnz = reinterpret_cast<int32_t*>(carve(p, (size_t)T * 4));
  void* sws = carve(p, scan_workspace_bytes(T));
  BSP_CUDA(cudaMemsetAsync(cnt, 0, (size_t)M * Kt * 4, s));
  const unsigned gr = (unsigned)ceil_div(M, 8);
  k_csr_rank<<<gr, 256, 0, s>>>(row_ptr, col, M, K, tc, Kt, cnt, rank);
  BSP_LAUNCHED();
  if (T > INT32_MAX) return BSP_ERR_CAPACITY;
  k_tiled_offsets<<<(unsigned)T, 256, 0, s>>>(cnt, M, tr, Kt, toff, tnnz);
  BSP_LAUNCHED();
  BSP_TRY(launch_scan_i32(tnnz, T, acc, sws, s));
  k_csr_fill<<<gr, 256, 0, s>>>(row_ptr, col, static_cast<const uint8_t*>(val), vbytes, M, tr, tc, Kt, rank, acc,
                                toff, tcol, static_cast<uint8_t*>(tval));
  BSP_LAUNCHED();
  return BSP_OK;
}

}  // namespace bsp
