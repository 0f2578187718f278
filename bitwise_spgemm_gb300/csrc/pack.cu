// pack.cu — bit packing, transposition, unpacking and bit-plane split.
//
// All kernels are HBM-bound streaming passes.  A word of 32 columns is built
// by one warp ballot (lane i tests column 32w+i), which replaces the
// per-nonzero global atomicOr of dense2bitmask (reference
// source/src/main.cu:611-621) and the one-int-per-bit output of
// uint8_layout_trans (backup/layout_trans.cu:87-97).
#include "bsp_internal.cuh"

namespace bsp {
namespace {

// Nonzero test with the reference's `x != 0` semantics (main.cu:617):
// -0.0 is zero, NaN is nonzero.
template <int DT> struct Elem;
template <> struct Elem<BSP_F32> {
  using T = float;
  __device__ static bool nz(T x) { return x != 0.0f; }
};
template <> struct Elem<BSP_F16> {
  using T = uint16_t;
  __device__ static bool nz(T x) { return (x & 0x7fffu) != 0; }
};
template <> struct Elem<BSP_BF16> {
  using T = uint16_t;
  __device__ static bool nz(T x) { return (x & 0x7fffu) != 0; }
};
template <> struct Elem<BSP_I8> {
  using T = int8_t;
  __device__ static bool nz(T x) { return x != 0; }
};
template <> struct Elem<BSP_U8> {
  using T = uint8_t;
  __device__ static bool nz(T x) { return x != 0; }
};

constexpr int kWordsPerWarpIter = 4;

// One warp builds kWordsPerWarpIter words per iteration (independent loads in
// flight), lane u < 4 stores word u.
template <int DT>
__global__ void __launch_bounds__(256) k_pack_rows(const typename Elem<DT>::T* __restrict__ dense,
                                                   int64_t M, int64_t K, int64_t ld,
                                                   uint32_t* __restrict__ words, int64_t Kw,
                                                   int msb) {
  using E = Elem<DT>;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t total = M * Kw;
  for (int64_t base = warp * kWordsPerWarpIter; base < total; base += nwarps * kWordsPerWarpIter) {
    bool nz[kWordsPerWarpIter];
#pragma unroll
    for (int u = 0; u < kWordsPerWarpIter; u++) {
      const int64_t t = base + u;
      nz[u] = false;
      if (t < total) {
        const int64_t r = t / Kw;
        const int64_t c = (t - r * Kw) * 32 + lane;
        if (c < K) nz[u] = E::nz(dense[r * ld + c]);
      }
    }
    uint32_t mine = 0;
#pragma unroll
    for (int u = 0; u < kWordsPerWarpIter; u++) {
      uint32_t b = __ballot_sync(kFull, nz[u]);
      if (msb) b = __brev(b);
      if (lane == u) mine = b;
    }
    if (lane < kWordsPerWarpIter && base + lane < total) words[base + lane] = mine;
  }
}

// Column packing: a warp owns rows 32*mw .. 32*mw+31 (lane = row) and 32
// consecutive columns; ballot over lanes for column k yields words_t[k][mw].
template <int DT>
__global__ void __launch_bounds__(256) k_pack_cols(const typename Elem<DT>::T* __restrict__ dense,
                                                   int64_t M, int64_t K, int64_t ld,
                                                   uint32_t* __restrict__ words_t, int64_t Mw,
                                                   int msb) {
  using E = Elem<DT>;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t Kc = (K + 31) / 32;
  const int64_t total = Mw * Kc;
  for (int64_t t = warp; t < total; t += nwarps) {
    const int64_t mw = t / Kc;
    const int64_t k0 = (t - mw * Kc) * 32;
    const int64_t r = mw * 32 + lane;
    uint32_t mine = 0;
#pragma unroll 8
    for (int j = 0; j < 32; j++) {
      const int64_t k = k0 + j;
      const bool nz = (r < M && k < K) ? E::nz(dense[r * ld + k]) : false;
      uint32_t b = __ballot_sync(kFull, nz);
      if (msb) b = __brev(b);
      if (lane == j) mine = b;
    }
    if (k0 + lane < K) words_t[(k0 + lane) * Mw + mw] = mine;
  }
}

// 32x32 bit-block transpose: lane i holds row 32*mw+i's word w; ballot of bit
// j across lanes is column 32w+j of the transpose.
__global__ void __launch_bounds__(256) k_transpose_bits(const uint32_t* __restrict__ words,
                                                        int64_t M, int64_t Kw, int64_t K,
                                                        uint32_t* __restrict__ words_t, int64_t Mw) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t total = Mw * Kw;
  for (int64_t t = warp; t < total; t += nwarps) {
    const int64_t mw = t / Kw;
    const int64_t w = t - mw * Kw;
    const int64_t r = mw * 32 + lane;
    const uint32_t my = r < M ? words[r * Kw + w] : 0u;
    uint32_t mine = 0;
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const uint32_t b = __ballot_sync(kFull, (my >> j) & 1u);
      if (lane == j) mine = b;
    }
    const int64_t k = w * 32 + lane;
    if (k < K) words_t[k * Mw + mw] = mine;
  }
}

// Thread per element; `one` is the dtype's bit pattern of 1.
template <typename T>
__global__ void __launch_bounds__(256) k_unpack_rows(const uint32_t* __restrict__ words, int64_t M,
                                                     int64_t K, int64_t Kw, T* __restrict__ dense,
                                                     int64_t ld, int msb, T one) {
  const int64_t n = M * K;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / K;
    const int64_t c = i - r * K;
    const uint32_t w = words[r * Kw + c / 32];
    const int bit = msb ? 31 - (int)(c & 31) : (int)(c & 31);
    dense[r * ld + c] = ((w >> bit) & 1u) ? one : T(0);
  }
}

// Warp per (row, word): lane c loads one byte, one ballot per plane.
__global__ void __launch_bounds__(256) k_bitplanes(const uint8_t* __restrict__ v, int64_t M,
                                                   int64_t K, int64_t ld, int planes,
                                                   uint32_t* __restrict__ words, int64_t Kw,
                                                   int msb, int rows_layout) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t total = M * Kw;
  for (int64_t t = warp; t < total; t += nwarps) {
    const int64_t r = t / Kw;
    const int64_t w = t - r * Kw;
    const int64_t c = w * 32 + lane;
    const uint32_t x = c < K ? v[r * ld + c] : 0u;
    uint32_t mine = 0;
#pragma unroll
    for (int b = 0; b < 8; b++) {
      if (b < planes) {
        uint32_t m = __ballot_sync(kFull, (x >> b) & 1u);
        if (msb) m = __brev(m);
        if (lane == b) mine = m;
      }
    }
    if (lane < planes)
      words[(rows_layout ? (r * planes + lane) : ((int64_t)lane * M + r)) * Kw + w] = mine;
  }
}

// 8x8 bit-matrix transpose of a uint64 (byte i = row i): afterwards byte b,
// bit i holds bit b of byte i (Hacker's Delight, section 7-3, transpose8).
__device__ __forceinline__ uint64_t transpose8x8(uint64_t x) {
  x = (x & 0xAA55AA55AA55AA55ull) | ((x & 0x00AA00AA00AA00AAull) << 7) | ((x >> 7) & 0x00AA00AA00AA00AAull);
  x = (x & 0xCCCC3333CCCC3333ull) | ((x & 0x0000CCCC0000CCCCull) << 14) | ((x >> 14) & 0x0000CCCC0000CCCCull);
  x = (x & 0xF0F0F0F00F0F0F0Full) | ((x & 0x00000000F0F0F0F0ull) << 28) | ((x >> 28) & 0x00000000F0F0F0F0ull);
  return x;
}

// Bit planes from 16-byte rows: a warp takes 512 columns of a row (lane l
// columns 16l..16l+15, one vector load), two 8x8 transposes give the lane's
// 16-bit mask of every plane, and the even lane of each pair joins its mask
// with its neighbour's into the 32-column word.  Rows must start 16-byte
// aligned (ld % 16 == 0); the ragged end of a row is read byte by byte.
__global__ void __launch_bounds__(256) k_bitplanes_v16(const uint8_t* __restrict__ v, int64_t M, int64_t K,
                                                       int64_t ld, int planes, uint32_t* __restrict__ words,
                                                       int64_t Kw, int msb, int rows_layout) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nch = (K + 511) / 512;
  for (int64_t t = warp; t < M * nch; t += nwarps) {
    const int64_t r = t / nch, ch = t - r * nch;
    const int64_t c = ch * 512 + lane * 16;
    const uint8_t* p = v + r * ld + c;
    uint64_t x0 = 0, x1 = 0;
    if (c + 16 <= K) {
      const uint4 q = __ldg(reinterpret_cast<const uint4*>(p));
      x0 = (uint64_t)q.x | ((uint64_t)q.y << 32);
      x1 = (uint64_t)q.z | ((uint64_t)q.w << 32);
    } else {
      for (int i = 0; i < 16; i++)
        if (c + i < K) {
          const uint64_t b = p[i];
          if (i < 8) x0 |= b << (8 * i);
          else x1 |= b << (8 * (i - 8));
        }
    }
    x0 = transpose8x8(x0);
    x1 = transpose8x8(x1);
    // m[q] = 16-bit masks of planes 2q (low half) and 2q+1 (high half)
    uint32_t m[4], n[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      m[q] = (uint32_t)((x0 >> (16 * q)) & 0xff) | ((uint32_t)((x1 >> (16 * q)) & 0xff) << 8) |
             ((uint32_t)((x0 >> (16 * q + 8)) & 0xff) << 16) | ((uint32_t)((x1 >> (16 * q + 8)) & 0xff) << 24);
      n[q] = __shfl_down_sync(kFull, m[q], 1);
    }
    const int64_t w = ch * 16 + (lane >> 1);
    if ((lane & 1) == 0 && w < Kw) {
#pragma unroll
      for (int b = 0; b < 8; b++) {
        if (b >= planes) break;
        const int sh = 16 * (b & 1);
        uint32_t word = ((m[b >> 1] >> sh) & 0xffffu) | (((n[b >> 1] >> sh) & 0xffffu) << 16);
        if (msb) word = __brev(word);
        words[(rows_layout ? (r * planes + b) : ((int64_t)b * M + r)) * Kw + w] = word;
      }
    }
  }
}

int grid_for(int64_t warps_needed) {
  const int64_t blocks = ceil_div(warps_needed, 8);
  const int64_t cap = (int64_t)num_sms() * 16;
  return (int)(blocks < 1 ? 1 : (blocks > cap ? cap : blocks));
}

}  // namespace

int launch_pack_rows(const void* dense, int dtype, int64_t M, int64_t K, int64_t ld,
                     uint32_t* words, int msb, cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32);
  const int grid = grid_for(ceil_div(M * Kw, kWordsPerWarpIter));
  switch (dtype) {
    case BSP_F32: k_pack_rows<BSP_F32><<<grid, 256, 0, s>>>((const float*)dense, M, K, ld, words, Kw, msb); break;
    case BSP_F16: k_pack_rows<BSP_F16><<<grid, 256, 0, s>>>((const uint16_t*)dense, M, K, ld, words, Kw, msb); break;
    case BSP_BF16: k_pack_rows<BSP_BF16><<<grid, 256, 0, s>>>((const uint16_t*)dense, M, K, ld, words, Kw, msb); break;
    case BSP_I8: k_pack_rows<BSP_I8><<<grid, 256, 0, s>>>((const int8_t*)dense, M, K, ld, words, Kw, msb); break;
    case BSP_U8: k_pack_rows<BSP_U8><<<grid, 256, 0, s>>>((const uint8_t*)dense, M, K, ld, words, Kw, msb); break;
    default: return BSP_ERR_INVALID_ARG;
  }
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_pack_cols(const void* dense, int dtype, int64_t M, int64_t K, int64_t ld,
                     uint32_t* words_t, int msb, cudaStream_t s) {
  const int64_t Mw = ceil_div(M, 32);
  const int grid = grid_for(Mw * ceil_div(K, 32));
  switch (dtype) {
    case BSP_F32: k_pack_cols<BSP_F32><<<grid, 256, 0, s>>>((const float*)dense, M, K, ld, words_t, Mw, msb); break;
    case BSP_F16: k_pack_cols<BSP_F16><<<grid, 256, 0, s>>>((const uint16_t*)dense, M, K, ld, words_t, Mw, msb); break;
    case BSP_BF16: k_pack_cols<BSP_BF16><<<grid, 256, 0, s>>>((const uint16_t*)dense, M, K, ld, words_t, Mw, msb); break;
    case BSP_I8: k_pack_cols<BSP_I8><<<grid, 256, 0, s>>>((const int8_t*)dense, M, K, ld, words_t, Mw, msb); break;
    case BSP_U8: k_pack_cols<BSP_U8><<<grid, 256, 0, s>>>((const uint8_t*)dense, M, K, ld, words_t, Mw, msb); break;
    default: return BSP_ERR_INVALID_ARG;
  }
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_transpose_bits(const uint32_t* words, int64_t M, int64_t K, uint32_t* words_t,
                          cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32), Mw = ceil_div(M, 32);
  k_transpose_bits<<<grid_for(Mw * Kw), 256, 0, s>>>(words, M, Kw, K, words_t, Mw);
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_unpack_rows(const uint32_t* words, int64_t M, int64_t K, void* dense, int dtype,
                       int64_t ld, int msb, cudaStream_t s) {
  const int64_t Kw = ceil_div(K, 32);
  const int grid = grid_for(ceil_div(M * K, 32));
  switch (dtype) {
    case BSP_F32: k_unpack_rows<float><<<grid, 256, 0, s>>>(words, M, K, Kw, (float*)dense, ld, msb, 1.0f); break;
    case BSP_F16: k_unpack_rows<uint16_t><<<grid, 256, 0, s>>>(words, M, K, Kw, (uint16_t*)dense, ld, msb, (uint16_t)0x3c00u); break;
    case BSP_BF16: k_unpack_rows<uint16_t><<<grid, 256, 0, s>>>(words, M, K, Kw, (uint16_t*)dense, ld, msb, (uint16_t)0x3f80u); break;
    case BSP_I8:
    case BSP_U8: k_unpack_rows<uint8_t><<<grid, 256, 0, s>>>(words, M, K, Kw, (uint8_t*)dense, ld, msb, (uint8_t)1u); break;
    default: return BSP_ERR_INVALID_ARG;
  }
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_bitplanes(const uint8_t* v, int64_t M, int64_t K, int64_t ld, int planes,
                     uint32_t* words, int msb, cudaStream_t s, int rows_layout) {
  const int64_t Kw = ceil_div(K, 32);
  if (is_aligned(v, 16) && ld % 16 == 0)
    k_bitplanes_v16<<<grid_for(M * ceil_div(K, 512)), 256, 0, s>>>(v, M, K, ld, planes, words, Kw, msb,
                                                                  rows_layout);
  else
    k_bitplanes<<<grid_for(M * Kw), 256, 0, s>>>(v, M, K, ld, planes, words, Kw, msb, rows_layout);
  BSP_LAUNCHED();
  return BSP_OK;
}

}  // namespace bsp
