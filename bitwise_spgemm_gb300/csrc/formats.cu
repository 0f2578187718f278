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

// Packed rows -> 8x8 tiles in three passes over A's words.  Work unit: a
// "quad" = word q of the 8 rows of tile row ty, i.e. the four tiles
// tx = 4q..4q+3 (byte j of each row's word is tile 4q+j's row); quads in
// (ty, q) order give tiles in ascending tile order.  A CTA takes kT8Span
// consecutive quads, thread t the quads base + k*256 + t (k < kT8Quads), so
// every load of a row's words is coalesced.
//   1. per CTA: nonzero tiles and their set bits;
//   2. one CTA scans both per-CTA totals (exclusive), writes *n_tiles;
//   3. per CTA again: the tiles are rebuilt, placed by a block scan of the
//      per-thread counts on top of the CTA's offsets, and written with their
//      popcount offset; then offset[n..T] = nnz.
// A's words are read twice; nothing of size T is written besides offset.
constexpr int kT8Threads = 256;
constexpr int kT8Quads = 4;
constexpr int kT8Span = kT8Threads * kT8Quads;

// 4x4 byte transpose: out[j] = bytes j of a, b, c, d (in that byte order).
__device__ __forceinline__ void byte_transpose4(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t (&out)[4]) {
  const uint32_t ab_lo = __byte_perm(a, b, 0x5140), ab_hi = __byte_perm(a, b, 0x7362);  // a0 b0 a1 b1 / a2 b2 a3 b3
  const uint32_t cd_lo = __byte_perm(c, d, 0x5140), cd_hi = __byte_perm(c, d, 0x7362);
  out[0] = __byte_perm(ab_lo, cd_lo, 0x5410);
  out[1] = __byte_perm(ab_lo, cd_lo, 0x7632);
  out[2] = __byte_perm(ab_hi, cd_hi, 0x5410);
  out[3] = __byte_perm(ab_hi, cd_hi, 0x7632);
}

// The four tiles of quad qd: tile j's byte r is byte j of row r's word.
__device__ __forceinline__ void quad_tiles(const uint32_t* __restrict__ words, int64_t M, int64_t Kw, int64_t qd,
                                           uint64_t (&m)[4]) {
  const int64_t ty = qd / Kw, q = qd - ty * Kw;
  uint32_t w[8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int64_t row = ty * 8 + r;
    w[r] = row < M ? __ldg(words + row * Kw + q) : 0u;
  }
  uint32_t lo[4], hi[4];
  byte_transpose4(w[0], w[1], w[2], w[3], lo);
  byte_transpose4(w[4], w[5], w[6], w[7], hi);
#pragma unroll
  for (int j = 0; j < 4; j++) m[j] = ((uint64_t)hi[j] << 32) | lo[j];
}

__global__ void __launch_bounds__(kT8Threads) k_t8_count(const uint32_t* __restrict__ words, int64_t M, int64_t Kw,
                                                         int64_t Q, int32_t* __restrict__ cnt_blk,
                                                         int32_t* __restrict__ pc_blk) {
  __shared__ int sw[32];
  int c = 0, pc = 0;
  for (int k = 0; k < kT8Quads; k++) {
    const int64_t qd = (int64_t)blockIdx.x * kT8Span + (int64_t)k * kT8Threads + threadIdx.x;
    if (qd >= Q) break;
    uint64_t m[4];
    quad_tiles(words, M, Kw, qd, m);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      c += m[j] != 0ull;
      pc += __popcll(m[j]);
    }
  }
  int tc, tp;
  block_exclusive_scan(c, sw, &tc);
  block_exclusive_scan(pc, sw, &tp);
  if (threadIdx.x == 0) {
    cnt_blk[blockIdx.x] = tc;
    pc_blk[blockIdx.x] = tp;
  }
}

// Exclusive scans of the per-CTA tile counts and popcounts, in place; the
// totals go to *n_tiles and tot[0].
__global__ void __launch_bounds__(1024) k_t8_scan(int32_t* __restrict__ cnt_blk, int32_t* __restrict__ pc_blk,
                                                  int64_t nb, int64_t* __restrict__ n_tiles,
                                                  int32_t* __restrict__ tot) {
  __shared__ int sw[32];
  int cc = 0, cp = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    const int c = i < nb ? cnt_blk[i] : 0, p = i < nb ? pc_blk[i] : 0;
    int tc, tp;
    const int ec = block_exclusive_scan(c, sw, &tc);
    const int ep = block_exclusive_scan(p, sw, &tp);
    if (i < nb) {
      cnt_blk[i] = cc + ec;
      pc_blk[i] = cp + ep;
    }
    cc += tc;
    cp += tp;
  }
  if (threadIdx.x == 0) {
    *n_tiles = cc;
    tot[0] = cp;
  }
}

__global__ void __launch_bounds__(kT8Threads) k_t8_write(const uint32_t* __restrict__ words, int64_t M, int64_t Kw,
                                                         int64_t Q, int64_t Kt, int64_t T,
                                                         const int32_t* __restrict__ cnt_off,
                                                         const int32_t* __restrict__ pc_off,
                                                         const int64_t* __restrict__ n_tiles,
                                                         const int32_t* __restrict__ tot, uint64_t* __restrict__ bmp,
                                                         int32_t* __restrict__ trow, int32_t* __restrict__ tcol,
                                                         int32_t* __restrict__ offset) {
  __shared__ int sw[32];
  int run_c = cnt_off[blockIdx.x], run_p = pc_off[blockIdx.x];
  for (int k = 0; k < kT8Quads; k++) {
    const int64_t qd = (int64_t)blockIdx.x * kT8Span + (int64_t)k * kT8Threads + threadIdx.x;
    uint64_t m[4] = {0ull, 0ull, 0ull, 0ull};
    if (qd < Q) quad_tiles(words, M, Kw, qd, m);
    int c = 0, pc = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      c += m[j] != 0ull;
      pc += __popcll(m[j]);
    }
    int tc, tp;
    int pos = block_exclusive_scan(c, sw, &tc) + run_c;
    int po = block_exclusive_scan(pc, sw, &tp) + run_p;
    if (c) {
      const int64_t ty = qd / Kw, q = qd - ty * Kw;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        if (!m[j]) continue;
        bmp[pos] = m[j];
        trow[pos] = (int32_t)ty;
        tcol[pos] = (int32_t)(4 * q + j);
        offset[pos] = po;
        pos++;
        po += __popcll(m[j]);
      }
    }
    run_c += tc;
    run_p += tp;
  }
  // offset[t] = nnz for t in [n, T]
  const int64_t n = *n_tiles;
  const int32_t nnz = tot[0];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = n + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= T; t += stride) offset[t] = nnz;
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
  // per-CTA tile counts and popcounts, the nnz total
  const int64_t nb = ceil_div(ceil_div(M, 8) * ceil_div(K, 32), kT8Span);
  return 2 * ((size_t)nb * 4 + 256) + 256;
}

static inline uint8_t* carve(uint8_t*& p, size_t bytes) {
  uint8_t* r = p;
  p += (bytes + 255) & ~(size_t)255;
  return r;
}

int launch_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K, uint64_t* bmp, int32_t* trow, int32_t* tcol,
                          int32_t* offset, int64_t* n_tiles, void* ws, cudaStream_t s) {
  const int64_t Mt = ceil_div(M, 8), Kt = ceil_div(K, 8), T = Mt * Kt, Kw = ceil_div(K, 32);
  const int64_t Q = Mt * Kw, nb = ceil_div(Q, kT8Span);
  uint8_t* p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
  int32_t* cnt_blk = reinterpret_cast<int32_t*>(carve(p, (size_t)nb * 4));
  int32_t* pc_blk = reinterpret_cast<int32_t*>(carve(p, (size_t)nb * 4));
  int32_t* tot = reinterpret_cast<int32_t*>(p);
  k_t8_count<<<(unsigned)nb, kT8Threads, 0, s>>>(words, M, Kw, Q, cnt_blk, pc_blk);
  k_t8_scan<<<1, 1024, 0, s>>>(cnt_blk, pc_blk, nb, n_tiles, tot);
  k_t8_write<<<(unsigned)nb, kT8Threads, 0, s>>>(words, M, Kw, Q, Kt, T, cnt_blk, pc_blk, n_tiles, tot, bmp, trow,
                                                 tcol, offset);
  BSP_LAUNCHED();
  return BSP_OK;
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
