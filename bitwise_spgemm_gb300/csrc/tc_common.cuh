// tc_common.cuh — helpers shared by the tcgen05 kernels.
#pragma once
#include <stdint.h>

namespace bsp {
namespace tc {

// Operands are stored as 8x16-byte core matrices (no swizzle).  In every
// descriptor the leading byte offset (LBO) is the distance between core
// matrices adjacent along the reduction (K) and the stride byte offset (SBO)
// the distance between core matrices adjacent along M (operand A) or N
// (operand B), for K-major and MN-major operands alike — measured on GB300
// with one-hot A rows and position-encoding B values.
//   K-major:  element (mn, k) at (mn/8)*kSbo + (k/8)*kLbo + (mn%8)*16 + (k%8)*2
//   MN-major: element (k, mn) at (mn/8)*kSbo + (k/8)*kLbo + (k%8)*16 + (mn%8)*2
constexpr uint32_t kLbo = 128, kSbo = 512;

// Dense 16-bit operands that arrive by TMA use swizzled layouts instead: a
// box of 16-byte rows moves at about a quarter of the L2 -> shared memory
// rate of 128-byte rows (measured on GB300: 2.4 vs 7-9 TB/s).
//   MN-major, 128-byte swizzle: atoms of 8 reduction rows x 64 elements
//     (1024 B, rows 128 B apart, 16-byte chunk q of row r stored at chunk
//     q ^ (r & 7)); SBO = distance between 8-row groups along the reduction,
//     LBO = distance between 64-element atoms along M / N.
//   K-major, 64-byte swizzle: atoms of 8 rows x 32 reduction elements (512 B,
//     chunk q of row r at q ^ ((r >> 1) & 3)); SBO = distance between 8-row
//     groups, LBO unused; the second K=16 half starts 32 bytes in.
constexpr uint32_t kLayoutSw128 = 2, kLayoutSw64 = 4;
constexpr uint32_t kSw128Atom = 1024, kSw64Atom = 512;

// Instruction descriptor for kind::f16: D f32 (bits 4-5), A and B of the
// same 16-bit type (bits 7-9, 10-12: bf16 = 1, f16 = 0), A / B major (bits
// 15, 16: 0 = K-major, 1 = MN-major), N >> 3 (bits 17-22), M >> 4 (24-28).
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t ab_type, uint32_t a_mn, uint32_t b_mn, uint32_t n,
                                                 uint32_t m) {
  return (1u << 4) | (ab_type << 7) | (ab_type << 10) | (a_mn << 15) | (b_mn << 16) | ((n >> 3) << 17) |
         ((m >> 4) << 24);
}

// 8 bits of a word → 8 16-bit values 0 / one, packed little-endian.
__device__ __forceinline__ uint4 expand8(uint32_t byte, uint32_t one) {
  uint32_t w[4];
#pragma unroll
  for (int j = 0; j < 4; j++)
    w[j] = (((byte >> (2 * j)) & 1u) ? one : 0u) | ((((byte >> (2 * j + 1)) & 1u) ? one : 0u) << 16);
  return make_uint4(w[0], w[1], w[2], w[3]);
}

}  // namespace tc
}  // namespace bsp
