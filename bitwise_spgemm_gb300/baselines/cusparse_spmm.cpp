// cusparse_spmm.cpp — the reference's library baseline for the SpMM:
// cuSPARSE's CSR SpMM, as the reference times it in
// timing_cusparse_spmm_csr (source/src/main.cu:1061-1131).  Timing and
// cross-checking only: it is built into its own libbsp_cusparse.so, so the
// bitmap library never links cuSPARSE and no bsp_* entry point calls it.
//
// Differences from the reference's timing, all stated by the caller's
// report: the reference times one cold call (bufferSize + cudaMalloc of the
// workspace + one SpMM, with the handle and descriptors made outside); here
// that cold call is timed the same way (*first_ms) and, in addition, `iters`
// warm calls after `warmup` untimed ones (*ms, the mean), all on the
// caller's stream.
#include <cuda_runtime.h>
#include <cusparse.h>
#include <stdint.h>

#include "bsp.h"

namespace {

int status_of(cusparseStatus_t s) {
  if (s == CUSPARSE_STATUS_SUCCESS) return BSP_OK;
  if (s == CUSPARSE_STATUS_NOT_SUPPORTED) return BSP_ERR_UNSUPPORTED;
  if (s == CUSPARSE_STATUS_INVALID_VALUE) return BSP_ERR_INVALID_ARG;
  if (s == CUSPARSE_STATUS_ALLOC_FAILED || s == CUSPARSE_STATUS_INSUFFICIENT_RESOURCES) return BSP_ERR_ALLOC;
  return BSP_ERR_CUDA;
}

// Every handle and buffer the run holds, released on every path.
struct Run {
  cusparseHandle_t h = nullptr;
  cusparseSpMatDescr_t a = nullptr;
  cusparseDnMatDescr_t b = nullptr, c = nullptr;
  void* buf = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~Run() {
    if (a) cusparseDestroySpMat(a);
    if (b) cusparseDestroyDnMat(b);
    if (c) cusparseDestroyDnMat(c);
    if (h) cusparseDestroy(h);
    if (buf) cudaFree(buf);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
};

}  // namespace

#define CK_SP(x)                          \
  do {                                    \
    const cusparseStatus_t s_ = (x);      \
    if (s_ != CUSPARSE_STATUS_SUCCESS) {  \
      return status_of(s_);               \
    }                                     \
  } while (0)
#define CK_RT(x)                                \
  do {                                          \
    if ((x) != cudaSuccess) return BSP_ERR_CUDA; \
  } while (0)

extern "C" {

// C[M][ldc] (FP32) = A·B for A in CSR (32-bit row offsets [M+1] and column
// indices [nnz], values [nnz] of `dtype`) and B row-major [K][ldb] of
// `dtype` (BSP_F32 or BSP_BF16; compute FP32).  `alg` is a
// cusparseSpMMAlg_t value (0 = CUSPARSE_SPMM_ALG_DEFAULT, as the reference).
// Returns BSP_OK, BSP_ERR_UNSUPPORTED when cuSPARSE does not offer the
// combination, or another negative status.
int bsp_cusparse_spmm_csr(int64_t M, int64_t K, int64_t N, int64_t nnz, const int32_t* offsets,
                          const int32_t* columns, const void* values, const void* B, int dtype, int64_t ldb,
                          float* C, int64_t ldc, int alg, int warmup, int iters, cudaStream_t stream, float* ms,
                          float* first_ms) {
  if (M <= 0 || K <= 0 || N <= 0 || nnz < 0 || !offsets || (nnz > 0 && (!columns || !values)) || !B || !C ||
      ldb < N || ldc < N || warmup < 0 || iters < 1 || !ms || !first_ms)
    return BSP_ERR_INVALID_ARG;
  if (dtype != BSP_F32 && dtype != BSP_BF16) return BSP_ERR_UNSUPPORTED;
  const cudaDataType vt = dtype == BSP_F32 ? CUDA_R_32F : CUDA_R_16BF;
  const cusparseSpMMAlg_t algo = static_cast<cusparseSpMMAlg_t>(alg);
  const float alpha = 1.0f, beta = 0.0f;
  Run r;
  CK_SP(cusparseCreate(&r.h));
  CK_SP(cusparseSetStream(r.h, stream));
  CK_SP(cusparseCreateCsr(&r.a, M, K, nnz, const_cast<int32_t*>(offsets), const_cast<int32_t*>(columns),
                          const_cast<void*>(values), CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                          CUSPARSE_INDEX_BASE_ZERO, vt));
  CK_SP(cusparseCreateDnMat(&r.b, K, N, ldb, const_cast<void*>(B), vt, CUSPARSE_ORDER_ROW));
  CK_SP(cusparseCreateDnMat(&r.c, M, N, ldc, C, CUDA_R_32F, CUSPARSE_ORDER_ROW));
  CK_RT(cudaEventCreate(&r.e0));
  CK_RT(cudaEventCreate(&r.e1));
  CK_RT(cudaStreamSynchronize(stream));
  // the reference's cold call: workspace query, allocation, one SpMM
  CK_RT(cudaEventRecord(r.e0, stream));
  size_t bytes = 0;
  CK_SP(cusparseSpMM_bufferSize(r.h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha,
                                r.a, r.b, &beta, r.c, CUDA_R_32F, algo, &bytes));
  CK_RT(cudaMalloc(&r.buf, bytes > 0 ? bytes : 1));
  CK_SP(cusparseSpMM(r.h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, r.a, r.b,
                     &beta, r.c, CUDA_R_32F, algo, r.buf));
  CK_RT(cudaEventRecord(r.e1, stream));
  CK_RT(cudaEventSynchronize(r.e1));
  CK_RT(cudaEventElapsedTime(first_ms, r.e0, r.e1));
  // warm calls
  for (int i = 0; i < warmup; i++)
    CK_SP(cusparseSpMM(r.h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, r.a, r.b,
                       &beta, r.c, CUDA_R_32F, algo, r.buf));
  CK_RT(cudaEventRecord(r.e0, stream));
  for (int i = 0; i < iters; i++)
    CK_SP(cusparseSpMM(r.h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, r.a, r.b,
                       &beta, r.c, CUDA_R_32F, algo, r.buf));
  CK_RT(cudaEventRecord(r.e1, stream));
  CK_RT(cudaEventSynchronize(r.e1));
  float total = 0.0f;
  CK_RT(cudaEventElapsedTime(&total, r.e0, r.e1));
  *ms = total / (float)iters;
  return BSP_OK;
}

}  // extern "C"
