// bsp_harness — the library's stand-in for the reference's main()
// (source/src/main.cu:1879-2388): it builds a bitmap operand from a dense
// 0/1 matrix, groups its rows, plans and runs the SpMM through the C ABI
// only (no torch, no Python), times the SpMM with CUDA events and checks C
// against an exact CPU sum.  Integer-valued B (as the reference's
// benchmarks used) makes the check exact: every partial sum is an integer
// below 2^24.
//
//   bsp_harness [M K N density seed] [--bf16]
//
// Prints one summary line and returns 0 when the check passes, 1 when it
// fails, 2 on a usage or library error.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bsp.h"

namespace {

#define H_CUDA(x)                                                              \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 2;                                                                \
    }                                                                          \
  } while (0)
#define H_BSP(x)                                                               \
  do {                                                                         \
    int s_ = (x);                                                              \
    if (s_ != BSP_OK) {                                                        \
      std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, bsp_status_string(s_)); \
      return 2;                                                                \
    }                                                                          \
  } while (0)

struct Rng {  // xorshift64*: a small, portable generator (same draws on x86 and Arm)
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 1) {}
  uint64_t next() {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return s * 0x2545F4914F6CDD1Dull;
  }
  double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
};

uint16_t f32_to_bf16(float f) {  // exact for the small integers used here
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

}  // namespace

int main(int argc, char** argv) {
  int64_t M = 2048, K = 2048, N = 256;
  double density = 0.05;
  uint64_t seed = 1;
  bool bf16 = false;
  int pos = 0;
  for (int i = 1; i < argc; i++) {
    if (std::strcmp(argv[i], "--bf16") == 0) {
      bf16 = true;
      continue;
    }
    switch (pos++) {
      case 0: M = std::atoll(argv[i]); break;
      case 1: K = std::atoll(argv[i]); break;
      case 2: N = std::atoll(argv[i]); break;
      case 3: density = std::atof(argv[i]); break;
      case 4: seed = std::strtoull(argv[i], nullptr, 10); break;
      default: std::fprintf(stderr, "usage: bsp_harness [M K N density seed] [--bf16]\n"); return 2;
    }
  }
  if (M <= 0 || K <= 0 || N <= 0 || density < 0 || density > 1 || M * K > ((int64_t)1 << 31)) {
    std::fprintf(stderr, "bad sizes\n");
    return 2;
  }
  const int64_t Kw = (K + 31) / 32;

  // host operands: dense 0/1 A (FP32, as dense2bitmask read it) and integer B
  Rng rng(seed);
  std::vector<float> A((size_t)(M * K));
  for (auto& a : A) a = rng.uniform() < density ? 1.f : 0.f;
  std::vector<float> B((size_t)(K * N));
  for (auto& b : B) b = (float)((int)(rng.next() % 17) - 8);
  std::vector<uint16_t> B16;
  if (bf16) {
    B16.resize(B.size());
    for (size_t i = 0; i < B.size(); i++) B16[i] = f32_to_bf16(B[i]);
  }

  cudaStream_t st;
  H_CUDA(cudaStreamCreate(&st));
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  uint32_t *dW = nullptr, *dGmask = nullptr;
  int32_t* dGid = nullptr;
  const int tile_rows = 512, groups = 2;
  const int64_t tiles = (M + tile_rows - 1) / tile_rows * Kw;
  H_CUDA(cudaMalloc(&dA, sizeof(float) * M * K));
  H_CUDA(cudaMalloc(&dB, bf16 ? 2 * K * N : sizeof(float) * K * N));
  H_CUDA(cudaMalloc(&dC, sizeof(float) * M * N));
  H_CUDA(cudaMalloc(&dW, sizeof(uint32_t) * M * Kw));
  H_CUDA(cudaMalloc(&dGid, sizeof(int32_t) * M * Kw));
  H_CUDA(cudaMalloc(&dGmask, sizeof(uint32_t) * tiles * groups));
  int64_t* dGnnz = nullptr;
  H_CUDA(cudaMalloc(&dGnnz, sizeof(int64_t)));
  H_CUDA(cudaMemcpyAsync(dA, A.data(), sizeof(float) * M * K, cudaMemcpyHostToDevice, st));
  if (bf16)
    H_CUDA(cudaMemcpyAsync(dB, B16.data(), 2 * K * N, cudaMemcpyHostToDevice, st));
  else
    H_CUDA(cudaMemcpyAsync(dB, B.data(), sizeof(float) * K * N, cudaMemcpyHostToDevice, st));

  // dense2bitmask (main.cu:591-628), generate_groups_large (main.cu:50-247)
  H_BSP(bsp_pack_rows(dA, BSP_F32, M, K, K, dW, BSP_LSB_FIRST, st));
  H_BSP(bsp_group_rows(dW, M, Kw, tile_rows, groups, dGid, dGmask, nullptr, nullptr, nullptr, nullptr, dGnnz, st));
  int64_t grouped = 0;
  H_CUDA(cudaMemcpyAsync(&grouped, dGnnz, sizeof(int64_t), cudaMemcpyDeviceToHost, st));

  // plan, workspace, SpMM
  bsp_plan* plan = nullptr;
  H_BSP(bsp_plan_create(dW, M, K, nullptr, &plan, st));
  bsp_plan_info info;
  H_BSP(bsp_plan_get_info(plan, &info));
  size_t ws_bytes = 0;
  H_BSP(bsp_spmm_workspace_preferred(plan, N, &ws_bytes));
  void* ws = nullptr;
  if (ws_bytes) H_CUDA(cudaMalloc(&ws, ws_bytes));
  const int dt = bf16 ? BSP_BF16 : BSP_F32;
  for (int i = 0; i < 3; i++) H_BSP(bsp_spmm(dW, M, K, dB, dt, N, N, dC, N, plan, ws, ws_bytes, st));
  cudaEvent_t e0, e1;
  H_CUDA(cudaEventCreate(&e0));
  H_CUDA(cudaEventCreate(&e1));
  const int iters = 20;
  H_CUDA(cudaEventRecord(e0, st));
  for (int i = 0; i < iters; i++) H_BSP(bsp_spmm(dW, M, K, dB, dt, N, N, dC, N, plan, ws, ws_bytes, st));
  H_CUDA(cudaEventRecord(e1, st));
  H_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  H_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  ms /= iters;
  int dev_status = 0;
  H_BSP(bsp_device_status(&dev_status, 1));
  std::vector<float> C((size_t)(M * N));
  H_CUDA(cudaMemcpy(C.data(), dC, sizeof(float) * M * N, cudaMemcpyDeviceToHost));

  // exact check: check()'s sum (backup/bit_wise_gemm.cu:13-32) over every row
  int64_t bad = 0;
  std::vector<double> row((size_t)N);
  for (int64_t i = 0; i < M; i++) {
    std::fill(row.begin(), row.end(), 0.0);
    for (int64_t k = 0; k < K; k++)
      if (A[(size_t)(i * K + k)] != 0.f)
        for (int64_t j = 0; j < N; j++) row[(size_t)j] += B[(size_t)(k * N + j)];
    for (int64_t j = 0; j < N; j++) bad += (double)C[(size_t)(i * N + j)] != row[(size_t)j];
  }
  const double bytes = 4.0 * M * Kw + (bf16 ? 2.0 : 4.0) * K * N + 4.0 * M * N;
  std::printf("bsp_harness M=%lld K=%lld N=%lld B=%s nnz=%lld grouped_nnz=%lld plan_mode=%d spmm_ms=%.4f "
              "GBps=%.1f device_status=%d mismatches=%lld check=%s\n",
              (long long)M, (long long)K, (long long)N, bf16 ? "bf16" : "f32", (long long)info.nnz,
              (long long)grouped, info.mode, ms, bytes / (ms * 1e-3) / 1e9, dev_status, (long long)bad,
              bad == 0 && dev_status == 0 ? "PASS" : "FAIL");

  bsp_plan_destroy(plan);
  cudaFree(ws);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dW);
  cudaFree(dGid);
  cudaFree(dGmask);
  cudaFree(dGnnz);
  cudaStreamDestroy(st);
  return bad == 0 && dev_status == 0 ? 0 : 1;
}
