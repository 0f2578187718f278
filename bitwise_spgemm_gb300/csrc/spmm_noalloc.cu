// spmm_noalloc.cu — bsp_spmm_noalloc: the planned SpMM without a caller
// workspace, for callers that may not allocate device memory when they run
// the SpMM (plugin callbacks that are handed pointers only, hot loops that
// must not call the allocator, processes whose device memory belongs to
// another allocator).
//
// The scratch that bsp_spmm keeps in the caller's workspace lives here in a
// file-scope device array of fixed size: the prototype sums and, for 16-bit
// B on the tensor cores, the split-K partials and the tiled copy of B where
// they fit.  Its address is looked up once per device with
// cudaGetSymbolAddress (a host-side name of a __device__ array is not a
// device address), so the first call on a device must come before any
// stream capture; the call then runs the ordinary bsp_spmm path with the
// whole array as workspace, whatever the plan.  No allocation happens in
// this entry point.
#include <mutex>

#include "bsp_internal.cuh"
#include "plan.cuh"

namespace bsp {
namespace {

// 8 MiB: prototype sums of n_proto prototypes x ceil8(N) columns in FP32
// (plus 256 bytes of alignment slack) must fit.
constexpr size_t kNoAllocBytes = (size_t)8 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_scratch_mu;
void* g_scratch_addr[64] = {};

// Device address of g_noalloc_scratch on the current device (looked up on
// the first call for that device).
int scratch_address(void** out) {
  int dev = -1;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return BSP_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    BSP_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (!p) return BSP_ERR_INTERNAL;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return BSP_OK;
}

}  // namespace
}  // namespace bsp

extern "C" int bsp_spmm_noalloc(const uint32_t* A_words, int64_t M, int64_t K, const void* B,
                                int b_dtype, int64_t ldb, int64_t N, float* C, int64_t ldc,
                                const bsp_plan* plan, bsp_stream_t stream) {
  size_t need = 0;
  BSP_TRY(bsp_spmm_workspace(plan, N < 0 ? 0 : N, &need));
  if (need > bsp::kNoAllocBytes) return BSP_ERR_CAPACITY;
  void* scratch = nullptr;
  BSP_TRY(bsp::scratch_address(&scratch));
  return bsp_spmm(A_words, M, K, B, b_dtype, ldb, N, C, ldc, plan, scratch, bsp::kNoAllocBytes, stream);
}
