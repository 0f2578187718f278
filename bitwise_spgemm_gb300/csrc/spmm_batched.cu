// spmm_batched.cu — many independent bitmap SpMMs in one tensor-core launch.
//
// A batch (bsp_batch_create) holds, in device memory, one record per problem
// (B's tensor map, encoded once on the host, and A, C, sizes) and a work list
// with one item per (problem, 256-row block, 256-column block), sorted by
// reduction length, longest first, so the long items start in the first wave.
// bsp_batched_spmm runs the list with the tensor-core SpMM kernel
// (spmm_tc.cu, batch mode): one CTA per item, the item's problem read from
// the record, every K tile of its rows (a batch has no occupancy plan), B
// streamed by TMA through the problem's own tensor map.  One launch, no host
// synchronisation, no allocation.
#include <algorithm>
#include <new>
#include <cstring>
#include <vector>

#include "bsp_internal.cuh"
#include "spmm.cuh"

namespace bsp {

// Kept for bsp_device_status: the tensor-core kernel reports its own waits.
__device__ int g_batch_error;

int batched_device_error(int* out, bool clear) {
  BSP_CUDA(cudaMemcpyFromSymbol(out, g_batch_error, sizeof(int)));
  if (clear) {
    const int zero = 0;
    BSP_CUDA(cudaMemcpyToSymbol(g_batch_error, &zero, sizeof(int)));
  }
  return BSP_OK;
}

namespace {
constexpr int64_t kItemRows = 256, kItemCols = 256;  // the tensor-core kernel's CTA tile
}  // namespace

}  // namespace bsp

struct bsp_batch {
  int n = 0;
  int64_t N = 0;
  int bdt = BSP_BF16;
  int n_items = 0;
  int device = 0;
  void* dev = nullptr;  // BatchProblemTc[n] followed by int4 items[n_items]
  bsp::BatchProblemTc* probs = nullptr;
  int4* items = nullptr;
};

extern "C" {

int bsp_batch_create(const bsp_problem* problems, int n, int64_t N, int b_dtype, bsp_batch** batch,
                     bsp_stream_t stream) {
  using namespace bsp;
  if (!batch) return BSP_ERR_INVALID_ARG;
  *batch = nullptr;
  if (n < 0 || N < 0 || N > ((int64_t)1 << 30)) return BSP_ERR_INVALID_ARG;
  if (n > 0 && !problems) return BSP_ERR_INVALID_ARG;
  if (b_dtype != BSP_BF16 && b_dtype != BSP_F16) return BSP_ERR_UNSUPPORTED;
  if (N % 8 != 0) return BSP_ERR_ALIGNMENT;
  std::vector<BatchProblemTc> hp((size_t)n);
  std::vector<int4> items;
  for (int i = 0; i < n; i++) {
    const bsp_problem& p = problems[i];
    if (p.M < 0 || p.K < 0 || p.M > INT32_MAX || p.K > ((int64_t)1 << 30)) return BSP_ERR_INVALID_ARG;
    if (p.K > tc_max_reduction()) return BSP_ERR_CAPACITY;
    if (p.ldb < N || p.ldc < N) return BSP_ERR_INVALID_ARG;
    if ((p.M > 0 && p.K > 0 && !p.A_words) || (p.K > 0 && N > 0 && !p.B) || (p.M > 0 && N > 0 && !p.C))
      return BSP_ERR_INVALID_ARG;
    if (!is_aligned(p.A_words, 4) || !is_aligned(p.B, 16) || (p.ldb * 2) % 16 != 0 || !is_aligned(p.C, 16) ||
        p.ldc % 4 != 0)
      return BSP_ERR_ALIGNMENT;
    const int64_t Kw = ceil_div(p.K, 32);
    BatchProblemTc& r = hp[(size_t)i];
    std::memset(&r.map, 0, sizeof(r.map));
    if (p.K > 0 && N > 0) BSP_TRY(make_batch_map(&r.map, p.B, b_dtype, p.K, N, p.ldb));
    r.A = p.A_words;
    r.M = p.M;
    r.K = p.K;
    r.Kw = Kw;
    r.C = p.C;
    r.ldc = p.ldc;
    for (int64_t rb = 0; rb < ceil_div(p.M, kItemRows); rb++)
      for (int64_t nb = 0; nb < ceil_div(N, kItemCols); nb++) items.push_back(make_int4(i, (int)rb, (int)nb, (int)Kw));
  }
  if (items.size() > (size_t)INT32_MAX) return BSP_ERR_CAPACITY;
  // longest reduction first (LPT), ties by problem order: stable
  std::stable_sort(items.begin(), items.end(), [](const int4& x, const int4& y) { return x.w > y.w; });
  bsp_batch* b = new (std::nothrow) bsp_batch();
  if (!b) return BSP_ERR_ALLOC;
  b->n = n;
  b->N = N;
  b->bdt = b_dtype;
  b->n_items = (int)items.size();
  cudaGetDevice(&b->device);
  const size_t pbytes = sizeof(BatchProblemTc) * (size_t)std::max(n, 1);
  const size_t ibytes = sizeof(int4) * std::max<size_t>(items.size(), 1);
  const size_t poff = (pbytes + 255) & ~size_t(255);
  cudaError_t e = cudaMalloc(&b->dev, poff + ibytes);
  if (e != cudaSuccess) {
    cuda_status(e);
    delete b;
    return BSP_ERR_ALLOC;
  }
  b->probs = static_cast<BatchProblemTc*>(b->dev);
  b->items = reinterpret_cast<int4*>(static_cast<char*>(b->dev) + poff);
  const cudaStream_t s = (cudaStream_t)stream;
  int st = BSP_OK;
  if (n > 0 &&
      (e = cudaMemcpyAsync(b->probs, hp.data(), sizeof(BatchProblemTc) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    st = cuda_status(e);
  if (st == BSP_OK && !items.empty() &&
      (e = cudaMemcpyAsync(b->items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    st = cuda_status(e);
  if (st == BSP_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) st = cuda_status(e);
  if (st != BSP_OK) {
    cudaFree(b->dev);
    delete b;
    return st;
  }
  *batch = b;
  return BSP_OK;
}

int bsp_batch_destroy(bsp_batch* batch) {
  if (!batch) return BSP_OK;
  if (batch->dev) cudaFree(batch->dev);
  delete batch;
  return BSP_OK;
}

int bsp_batched_spmm(const bsp_batch* b, bsp_stream_t stream) {
  using namespace bsp;
  if (!b) return BSP_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) return BSP_ERR_INVALID_ARG;
  if (b->n_items == 0 || b->N == 0) return BSP_OK;
  return launch_batched_tc(b->probs, b->items, b->n_items, b->N, b->bdt, (cudaStream_t)stream);
}

}  // extern "C"
