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

// 32 bits of a word → 32 16-bit values, 2.0 for a set bit and 0 otherwise,
// as four 16-byte chunks of 8 consecutive values (value i = bit i).  2.0 is
// 0x4000 in BF16 and FP16 alike: one set bit, so after the word is
// unshuffled (even bits to the low half, odd bits to the high half — the
// perfect-unshuffle of Hacker's Delight, section 7-2) the pair of values
// 2j, 2j+1 is one shift and one mask.  Products made with 2.0 are scaled by
// 0.5 when stored, which is exact in binary floating point (unless a sum
// exceeds half the FP32 range).
constexpr float kTwoScale = 0.5f;
__device__ __forceinline__ void expand32_two(uint32_t w, uint4 (&o)[4]) {
  uint32_t x = w, t;
  t = (x ^ (x >> 1)) & 0x22222222u;
  x ^= t ^ (t << 1);
  t = (x ^ (x >> 2)) & 0x0c0c0c0cu;
  x ^= t ^ (t << 2);
  t = (x ^ (x >> 4)) & 0x00f000f0u;
  x ^= t ^ (t << 4);
  t = (x ^ (x >> 8)) & 0x0000ff00u;
  x ^= t ^ (t << 8);
  // x: bit j = bit 2j of w, bit 16+j = bit 2j+1 of w (j < 16)
  uint32_t v[16];
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = (j <= 14 ? (x << (14 - j)) : (x >> (j - 14))) & 0x40004000u;
#pragma unroll
  for (int c = 0; c < 4; c++) o[c] = make_uint4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
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
