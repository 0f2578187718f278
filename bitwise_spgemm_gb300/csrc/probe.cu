// probe.cu — bsp_probe_gather: the L2 row-gather roof that bounds the
// clustered-row SpMM.
//
// The planned SpMM's traffic is random row slices of B, which stays in L2
// (16 MB for 8192x512 FP32), so its ceiling is how fast SMs can gather
// random slices out of L2, not HBM bandwidth.  This kernel measures that
// ceiling with the same access pattern and nothing else: every warp reads
// its `per_warp` row indices 32 at a time (one coalesced load, broadcast by
// shuffle) and, for each, loads one slice of `slice_bytes` bytes of that
// row with 16-byte vector loads, one slice in flight per warp, adding the
// values so the loads cannot be dropped; the sum is written to `sink` only
// if it equals an impossible value.  Measured on GB300: 512-byte slices at
// 64 warps per SM reach about 17.7 TB/s; 1 KB slices at 64 warps per SM
// about 13 TB/s (more bytes in flight raise the latency faster than the
// throughput).
#include "bsp_internal.cuh"

namespace bsp {
namespace {

template <int V4>  // float4 loads per lane per slice: slice = 512·V4 bytes
__global__ void __launch_bounds__(256) k_probe_gather(const float4* __restrict__ buf, int64_t rows,
                                                      int64_t row_f4, const uint32_t* __restrict__ idx,
                                                      int64_t per_warp, float* sink) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const uint32_t* my = idx + gw * per_warp;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t r0 = 0; r0 < per_warp; r0 += 32) {
    const uint32_t mine = r0 + lane < per_warp ? __ldg(my + r0 + lane) : 0u;
    const int n = (int)min((int64_t)32, per_warp - r0);
    for (int j = 0; j < n; j++) {
      const uint32_t k = __shfl_sync(kFull, mine, j);
      if (k >= rows) continue;  // an index past the buffer reads nothing
#pragma unroll
      for (int v = 0; v < V4; v++) {
        const float4 x = __ldg(buf + (int64_t)k * row_f4 + v * 32 + lane);
        acc.x += x.x;
        acc.y += x.y;
        acc.z += x.z;
        acc.w += x.w;
      }
    }
  }
  const float t = acc.x + acc.y + acc.z + acc.w;
  if (t == -1.2345e-37f) sink[gw] = t;
}

}  // namespace
}  // namespace bsp

extern "C" int bsp_probe_gather(const void* buf, int64_t rows, int64_t row_bytes, const uint32_t* row_idx,
                                int64_t n_warps, int64_t per_warp, int slice_bytes, float* sink,
                                bsp_stream_t stream) {
  using namespace bsp;
  if (!buf || !row_idx || !sink || rows <= 0 || n_warps <= 0 || per_warp <= 0) return BSP_ERR_INVALID_ARG;
  if (slice_bytes != 512 && slice_bytes != 1024 && slice_bytes != 2048) return BSP_ERR_INVALID_ARG;
  if (row_bytes < slice_bytes || row_bytes % 16 != 0 || !is_aligned(buf, 16)) return BSP_ERR_ALIGNMENT;
  if (n_warps % 8 != 0 || n_warps / 8 > 0x7fffffff) return BSP_ERR_INVALID_ARG;
  const cudaStream_t s = (cudaStream_t)stream;
  const unsigned grid = (unsigned)(n_warps / 8);
  const float4* b = static_cast<const float4*>(buf);
  const int64_t rf4 = row_bytes / 16;
  switch (slice_bytes) {
    case 512: k_probe_gather<1><<<grid, 256, 0, s>>>(b, rows, rf4, row_idx, per_warp, sink); break;
    case 1024: k_probe_gather<2><<<grid, 256, 0, s>>>(b, rows, rf4, row_idx, per_warp, sink); break;
    default: k_probe_gather<4><<<grid, 256, 0, s>>>(b, rows, rf4, row_idx, per_warp, sink); break;
  }
  BSP_LAUNCHED();
  return BSP_OK;
}
