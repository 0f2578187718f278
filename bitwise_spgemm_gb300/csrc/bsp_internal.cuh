// bsp_internal.cuh — helpers shared by the library's translation units.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsp.h"

namespace bsp {

// Records the cudaError_t of the most recent failure on this host thread.
int cuda_status(cudaError_t e);

#define BSP_TRY(x)                         \
  do {                                     \
    int bsp_s_ = (x);                      \
    if (bsp_s_ != BSP_OK) return bsp_s_;   \
  } while (0)

#define BSP_CUDA(x)                                          \
  do {                                                       \
    cudaError_t bsp_e_ = (x);                                \
    if (bsp_e_ != cudaSuccess) return ::bsp::cuda_status(bsp_e_); \
  } while (0)

#define BSP_LAUNCHED() BSP_CUDA(cudaPeekAtLastError())

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline bool is_aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }
inline int dtype_size(int dt) {
  switch (dt) {
    case BSP_F32: return 4;
    case BSP_F16:
    case BSP_BF16: return 2;
    case BSP_I8:
    case BSP_U8: return 1;
    default: return 0;
  }
}

// SM count of the current device (cached per device ordinal).
int num_sms();

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float to_f32(float x) { return x; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ float to_f32(__half x) { return __half2float(x); }
template <typename T> __device__ __forceinline__ T from_f32(float x);
template <> __device__ __forceinline__ float from_f32<float>(float x) { return x; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <> __device__ __forceinline__ __half from_f32<__half>(float x) { return __float2half_rn(x); }

// Exclusive scan of one int per thread over the block (≤ 32 warps);
// smem_warp holds 32 ints; *total = the block's sum.  Ends with a barrier,
// so smem_warp may be reused right after.
__device__ __forceinline__ int block_exclusive_scan(int v, int* smem_warp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int s = lane < (int)(blockDim.x >> 5) ? smem_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, s, o);
      if (lane >= o) s += y;
    }
    smem_warp[lane] = s;  // inclusive warp-sum prefix
  }
  __syncthreads();
  const int before = wid ? smem_warp[wid - 1] : 0;
  *total = smem_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

// Internal launchers (defined in the .cu files, called from capi.cu).
int launch_pack_rows(const void* dense, int dtype, int64_t M, int64_t K, int64_t ld,
                     uint32_t* words, int msb, cudaStream_t s);
int launch_pack_cols(const void* dense, int dtype, int64_t M, int64_t K, int64_t ld,
                     uint32_t* words_t, int msb, cudaStream_t s);
int launch_transpose_bits(const uint32_t* words, int64_t M, int64_t K, uint32_t* words_t,
                          cudaStream_t s);
int launch_unpack_rows(const uint32_t* words, int64_t M, int64_t K, void* dense, int dtype,
                       int64_t ld, int msb, cudaStream_t s);
// rows_layout: words[M][planes][Kw] (planes of a row side by side) instead
// of words[planes][M][Kw]
int launch_bitplanes(const uint8_t* v, int64_t M, int64_t K, int64_t ld, int planes,
                     uint32_t* words, int msb, cudaStream_t s, int rows_layout = 0);
int launch_stack_planes_b(const void* B, int bdt, int64_t ldb, int64_t K, int64_t N, int nplanes, int signed_top,
                          void* out, int64_t ldo, cudaStream_t s);
int launch_group_rows(const uint32_t* words, int64_t M, int64_t Kw, int tile_rows,
                      int max_groups, int32_t* group_id, uint32_t* group_mask,
                      int32_t* group_row, int32_t* spill_cnt, int32_t* spill_nnz,
                      int32_t* spill_rows, int64_t* grouped_nnz, cudaStream_t s);
int launch_group_to_dense(const float* gv, const int32_t* gid, const uint32_t* words,
                          int64_t M, int64_t K, int tile_rows, int max_groups, float* dense,
                          int64_t ldd, cudaStream_t s);

// Exclusive prefix sum of n int32 values into out[0..n] (out[n] = total).
// ws must hold scan_workspace_bytes(n) bytes.
size_t scan_workspace_bytes(int64_t n);
// formats.cu
size_t tiles8_workspace_bytes(int64_t M, int64_t K);
int launch_rows_to_tiles8(const uint32_t* words, int64_t M, int64_t K, uint64_t* bmp, int32_t* trow, int32_t* tcol,
                          int32_t* offset, int64_t* n_tiles, void* ws, cudaStream_t s);
int launch_tiles8_to_rows(const uint64_t* bmp, const int32_t* trow, const int32_t* tcol, int64_t n, int64_t M,
                          int64_t K, uint32_t* words, cudaStream_t s);
size_t csr_tiled_workspace_bytes(int64_t M, int64_t K, int64_t nnz, int tile_rows, int tile_cols);
int launch_csr_to_tiled(const int32_t* row_ptr, const int32_t* col, const void* val, int vbytes, int64_t M,
                        int64_t K, int64_t nnz, int tr, int tc, int32_t* acc, int32_t* toff, int32_t* tcol,
                        void* tval, void* ws, cudaStream_t s);
// output.cu
int launch_symbolic_rows(const uint32_t* A, int64_t M, int64_t K, const uint32_t* Bw, int64_t N, uint32_t* Cw,
                         cudaStream_t s);
// Through a prototype plan: per-cluster bit-sliced column counts in
// `planes` (symbolic_planes_bytes), then the rows from their deltas.
size_t symbolic_planes_bytes(int64_t n_proto, int64_t N);
int launch_symbolic_planned(const uint32_t* A, int64_t M, int64_t K, const uint32_t* Bw, int64_t N, uint32_t* Cw,
                            const int32_t* row_cluster, const int32_t* delta_ptr, const uint32_t* delta_idx,
                            const uint32_t* cons, int64_t n_proto, uint32_t* planes, cudaStream_t s);
int launch_bitplane_spmm(const uint32_t* planes, int nplanes, int signed_top, int64_t M, int64_t K,
                         const void* B, int bdt, int64_t ldb, int64_t N, float* C, int64_t ldc, bool vec,
                         cudaStream_t s);
int launch_scan_i32(const int32_t* in, int64_t n, int32_t* out, void* ws, cudaStream_t s);

}  // namespace bsp
