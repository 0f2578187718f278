// spmm_dev.cuh — device helpers shared by the SpMM kernels: vector loads of
// B, index streams over packed words / delta lists, FP32 accumulators.
#pragma once
#include "bsp_internal.cuh"
#include "spmm.cuh"

namespace bsp {
namespace {

constexpr int kCompThreshold = 4096;  // set bits above which rows use TwoSum

// ---- vector loads of B ----------------------------------------------------
template <typename BT> struct Vec;
template <> struct Vec<float> {
  static constexpr int COLS = 4;
  using Raw = float4;
  __device__ static Raw load(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
  __device__ static void cvt(const Raw& r, float* o) { o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = r.w; }
};
template <> struct Vec<__nv_bfloat16> {
  static constexpr int COLS = 8;
  using Raw = uint4;
  __device__ static Raw load(const __nv_bfloat16* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }
  __device__ static void cvt(const Raw& r, float* o) {
    const uint32_t u[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      o[2 * j] = __uint_as_float(u[j] << 16);
      o[2 * j + 1] = __uint_as_float(u[j] & 0xffff0000u);
    }
  }
};
template <> struct Vec<__half> {
  static constexpr int COLS = 8;
  using Raw = uint4;
  __device__ static Raw load(const __half* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }
  __device__ static void cvt(const Raw& r, float* o) {
    const uint32_t u[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      __half2 h = *reinterpret_cast<const __half2*>(&u[j]);
      float2 f = __half22float2(h);
      o[2 * j] = f.x;
      o[2 * j + 1] = f.y;
    }
  }
};

// ---- index streams --------------------------------------------------------
// next() returns a raw entry: column in bits 0..30, bit 31 = subtract (delta
// lists only); kEnd when exhausted.  All state is warp-uniform.
constexpr uint32_t kEnd = 0xffffffffu;

// Set-bit walker over words [w_begin, w_end) of one packed row: `my` is this
// lane's word of the current 32-word group, `pending` the lanes whose words
// still hold bits, `cur` the word being consumed; columns come out ascending.
struct BitWalker {
  const uint32_t* words;
  int w_end, g, curbase, lane;
  uint32_t my, pending, cur;
  __device__ void init(const uint32_t* w, int w_begin, int w_end_, int lane_) {
    words = w;
    w_end = w_end_;
    g = w_begin - 32;
    my = pending = cur = 0u;
    curbase = 0;
    lane = lane_;
  }
  __device__ __forceinline__ uint32_t next() {
    while (cur == 0u) {
      if (pending == 0u) {
        g += 32;
        if (g >= w_end) return kEnd;
        my = (g + lane < w_end) ? __ldg(words + g + lane) : 0u;
        pending = __ballot_sync(kFull, my != 0u);
        continue;
      }
      const int src = __ffs(pending) - 1;
      pending &= pending - 1;
      cur = __shfl_sync(kFull, my, src);
      curbase = (g + src) * 32;
    }
    const int b = __ffs(cur) - 1;
    cur &= cur - 1;
    return (uint32_t)(curbase + b);
  }
};

// Entries of a delta list, 32 loaded at a time and broadcast by shuffle.
struct ListWalker {
  const uint32_t* list;
  int pos, end, base, lane;
  uint32_t mine;
  __device__ void init(const uint32_t* l, int b, int e, int lane_) {
    list = l;
    pos = b;
    end = e;
    base = b - 32;
    lane = lane_;
    mine = 0u;
  }
  __device__ __forceinline__ uint32_t next() {
    if (pos >= end) return kEnd;
    if (pos >= base + 32) {
      base = pos;
      mine = (pos + lane < end) ? __ldg(list + pos + lane) : 0u;
    }
    const uint32_t e = __shfl_sync(kFull, mine, pos - base);
    pos++;
    return e;
  }
};

// A row's delta list from its 128-byte slot (words 2 and 3 = count and the
// list's start, words 4..31 = the first 28 entries, one per lane) and, past
// 28 entries, from the list: the same entries in the same order as a
// ListWalker over the whole list.
struct SlotWalker {
  static constexpr int kIn = 28;
  uint32_t slot;
  int n, j;
  ListWalker tail;
  __device__ void init(uint32_t slot_, const uint32_t* list, int lane) {
    slot = slot_;
    n = (int)__shfl_sync(kFull, slot_, 2);
    const int s = (int)__shfl_sync(kFull, slot_, 3);
    j = 0;
    tail.init(list, s + kIn, n > kIn ? s + n : s + kIn, lane);
  }
  __device__ __forceinline__ uint32_t next() {
    if (j < n && j < kIn) return __shfl_sync(kFull, slot, 4 + j++);
    return tail.next();
  }
};

template <int VPL, int COLS, bool COMP>
struct Acc {
  float s[VPL][COLS];
  float c[COMP ? VPL : 1][COMP ? COLS : 1];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int v = 0; v < VPL; v++)
#pragma unroll
      for (int j = 0; j < COLS; j++) {
        s[v][j] = 0.f;
        if (COMP) c[COMP ? v : 0][COMP ? j : 0] = 0.f;
      }
  }
  __device__ __forceinline__ void add(int v, int j, float x) {
    if (COMP) {  // TwoSum: s + x = t + e exactly; e accumulates separately
      const float t = s[v][j] + x;
      const float bp = t - s[v][j];
      const float e = (s[v][j] - (t - bp)) + (x - bp);
      s[v][j] = t;
      c[COMP ? v : 0][COMP ? j : 0] += e;
    } else {
      s[v][j] += x;
    }
  }
  __device__ __forceinline__ float result(int v, int j) const {
    return COMP ? s[v][j] + c[COMP ? v : 0][COMP ? j : 0] : s[v][j];
  }
};

// Gathers D rows of B at a time (this lane's VPL vectors of each) and adds
// them in stream order; entries with bit 31 set are subtracted.
template <typename BT, int VPL, int D, bool COMP, typename Walker, typename LD = int64_t>
__device__ __forceinline__ void accumulate_walk(Walker& wk, const BT* __restrict__ B, LD ldb,
                                                const int* col, const bool* cvalid,
                                                Acc<VPL, Vec<BT>::COLS, COMP>& acc) {
  using V = Vec<BT>;
  while (true) {
    uint32_t idx[D];
#pragma unroll
    for (int s = 0; s < D; s++) idx[s] = wk.next();
    if (idx[0] == kEnd) break;
    typename V::Raw raw[D][VPL];
#pragma unroll
    for (int s = 0; s < D; s++) {
      const BT* brow = B + (LD)(idx[s] & 0x7fffffffu) * ldb;
#pragma unroll
      for (int v = 0; v < VPL; v++)
        if (idx[s] != kEnd && cvalid[v]) raw[s][v] = V::load(brow + col[v]);
    }
#pragma unroll
    for (int s = 0; s < D; s++) {
      if (idx[s] == kEnd) continue;
      const bool neg = (idx[s] >> 31) != 0u;
#pragma unroll
      for (int v = 0; v < VPL; v++) {
        if (!cvalid[v]) continue;
        float f[V::COLS];
        V::cvt(raw[s][v], f);
#pragma unroll
        for (int j = 0; j < V::COLS; j++) acc.add(v, j, neg ? -f[j] : f[j]);
      }
    }
    if (idx[D - 1] == kEnd) break;
  }
}

__device__ __forceinline__ int row_popcount(const uint32_t* __restrict__ row, int Kw, int lane) {
  int c = 0;
  for (int w = lane; w < Kw; w += 32) c += __popc(__ldg(row + w));
#pragma unroll
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
  return c;
}

template <int VPL, int COLS, bool COMP>
__device__ __forceinline__ void store_vecs(float* __restrict__ crow, const int* col,
                                           const bool* cvalid, const Acc<VPL, COLS, COMP>& acc,
                                           const float* __restrict__ prow) {
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    if (!cvalid[v]) continue;
    float o[COLS];
#pragma unroll
    for (int j = 0; j < COLS; j++) o[j] = acc.result(v, j);
    if (prow) {
#pragma unroll
      for (int j = 0; j < COLS; j += 4) {
        const float4 p = *reinterpret_cast<const float4*>(prow + col[v] + j);
        o[j] += p.x; o[j + 1] += p.y; o[j + 2] += p.z; o[j + 3] += p.w;
      }
    }
#pragma unroll
    for (int j = 0; j < COLS; j += 4)
      *reinterpret_cast<float4*>(crow + col[v] + j) = make_float4(o[j], o[j + 1], o[j + 2], o[j + 3]);
  }
}

}  // namespace
}  // namespace bsp
