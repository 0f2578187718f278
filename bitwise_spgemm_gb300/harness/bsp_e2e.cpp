// bsp_e2e — the end-to-end serving loop of the bitmap SpMM through the C ABI
// only (no torch, no Python): per step, A's packed words and B go up from
// pinned host memory, the plan is built (or an earlier plan reused), the
// SpMM runs and C comes back to pinned host memory.  Two steps are in
// flight, as a serving loop runs them: step i's C download (its own stream)
// overlaps step i+1's uploads and plan build, and B's upload (a second
// stream) waits only for the SpMM that last read its buffer.  Each per-step
// plan is released in stream order right after its SpMM.
//
//   bsp_e2e DIR M K N STEPS WARMUP MODE
//
// MODE 0: plan built every step; 1: plan reused; 2: the copies alone (the
// same uploads and downloads in the same pipeline, no plan and no SpMM) —
// the floor the host link sets for the other two.
//
// DIR holds words.bin (M x ceil(K/32) uint32, LSB-first) and B.bin (K x N
// float32).  Prints one JSON line: wall time per step over STEPS steps
// (after WARMUP), the bytes moved each way, and writes the last step's C to
// DIR/C.bin.  Returns 0 on success, 2 on a usage or library error.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bsp.h"

namespace {

#define E_CUDA(x)                                                              \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 2;                                                                \
    }                                                                          \
  } while (0)
#define E_BSP(x)                                                               \
  do {                                                                         \
    int s_ = (x);                                                              \
    if (s_ != BSP_OK) {                                                        \
      std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, bsp_status_string(s_)); \
      return 2;                                                                \
    }                                                                          \
  } while (0)

bool read_file(const std::string& path, void* dst, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  const size_t got = std::fread(dst, 1, bytes, f);
  std::fclose(f);
  return got == bytes;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: bsp_e2e DIR M K N STEPS WARMUP MODE\n");
    return 2;
  }
  const std::string dir = argv[1];
  const int64_t M = std::atoll(argv[2]), K = std::atoll(argv[3]), N = std::atoll(argv[4]);
  const int steps = std::atoi(argv[5]), warmup = std::atoi(argv[6]);
  const int mode = std::atoi(argv[7]);
  const bool reuse = mode != 0, copies_only = mode == 2;
  if (M <= 0 || K <= 0 || N <= 0 || steps <= 0 || warmup < 0) {
    std::fprintf(stderr, "bad sizes\n");
    return 2;
  }
  const int64_t Kw = (K + 31) / 32;
  const size_t wbytes = sizeof(uint32_t) * (size_t)(M * Kw), bbytes = sizeof(float) * (size_t)(K * N),
               cbytes = sizeof(float) * (size_t)(M * N);

  uint32_t* h_words = nullptr;
  float *h_B = nullptr, *h_C[2] = {nullptr, nullptr};
  E_CUDA(cudaMallocHost(&h_words, wbytes));
  E_CUDA(cudaMallocHost(&h_B, bbytes));
  for (auto& p : h_C) E_CUDA(cudaMallocHost(&p, cbytes));
  if (!read_file(dir + "/words.bin", h_words, wbytes) || !read_file(dir + "/B.bin", h_B, bbytes)) {
    std::fprintf(stderr, "cannot read %s/words.bin or B.bin\n", dir.c_str());
    return 2;
  }
  uint32_t* d_words[2];
  float *d_B[2], *d_C[2];
  for (int j = 0; j < 2; j++) {
    E_CUDA(cudaMalloc(&d_words[j], wbytes));
    E_CUDA(cudaMalloc(&d_B[j], bbytes));
    E_CUDA(cudaMalloc(&d_C[j], cbytes));
  }
  cudaStream_t main_s, side, d2h;
  E_CUDA(cudaStreamCreateWithFlags(&main_s, cudaStreamNonBlocking));
  E_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  E_CUDA(cudaStreamCreateWithFlags(&d2h, cudaStreamNonBlocking));
  cudaEvent_t downloaded[2], used[2], b_up[2];
  for (int j = 0; j < 2; j++) {
    E_CUDA(cudaEventCreateWithFlags(&downloaded[j], cudaEventDisableTiming));
    E_CUDA(cudaEventCreateWithFlags(&used[j], cudaEventDisableTiming));
    E_CUDA(cudaEventCreateWithFlags(&b_up[j], cudaEventDisableTiming));
    E_CUDA(cudaEventRecord(downloaded[j], d2h));
    E_CUDA(cudaEventRecord(used[j], main_s));
  }
  // a first plan (also the reused one) and a workspace sized for it
  E_CUDA(cudaMemcpyAsync(d_words[0], h_words, wbytes, cudaMemcpyHostToDevice, main_s));
  bsp_plan* plan0 = nullptr;
  E_BSP(bsp_plan_create(d_words[0], M, K, nullptr, &plan0, (bsp_stream_t)main_s));
  size_t ws_bytes = 0;
  E_BSP(bsp_spmm_workspace_preferred(plan0, N, &ws_bytes));
  void* ws = nullptr;
  if (ws_bytes) E_CUDA(cudaMalloc(&ws, ws_bytes));
  E_CUDA(cudaStreamSynchronize(main_s));

  auto step = [&](int i) -> int {
    const int j = i % 2;
    E_CUDA(cudaStreamWaitEvent(main_s, downloaded[j], 0));  // this set's previous C is on the host
    E_CUDA(cudaMemcpyAsync(d_words[j], h_words, wbytes, cudaMemcpyHostToDevice, main_s));
    E_CUDA(cudaStreamWaitEvent(side, used[j], 0));  // the SpMM that last read this B has run
    E_CUDA(cudaMemcpyAsync(d_B[j], h_B, bbytes, cudaMemcpyHostToDevice, side));
    E_CUDA(cudaEventRecord(b_up[j], side));
    bsp_plan* p = plan0;
    if (!reuse) E_BSP(bsp_plan_create(d_words[j], M, K, nullptr, &p, (bsp_stream_t)main_s));
    E_CUDA(cudaStreamWaitEvent(main_s, b_up[j], 0));
    if (!copies_only)
      E_BSP(bsp_spmm(d_words[j], M, K, d_B[j], BSP_F32, N, N, d_C[j], N, p, ws, ws_bytes, (bsp_stream_t)main_s));
    E_CUDA(cudaEventRecord(used[j], main_s));
    if (!reuse) E_BSP(bsp_plan_destroy_async(p, (bsp_stream_t)main_s));
    E_CUDA(cudaStreamWaitEvent(d2h, used[j], 0));
    E_CUDA(cudaMemcpyAsync(h_C[j], d_C[j], cbytes, cudaMemcpyDeviceToHost, d2h));
    E_CUDA(cudaEventRecord(downloaded[j], d2h));
    return 0;
  };
  for (int i = 0; i < warmup; i++)
    if (step(i)) return 2;
  E_CUDA(cudaDeviceSynchronize());
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < steps; i++)
    if (step(i)) return 2;
  E_CUDA(cudaDeviceSynchronize());
  const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  int dev_status = 0;
  E_BSP(bsp_device_status(&dev_status, 0));
  const int last = (steps - 1) % 2;
  FILE* f = std::fopen((dir + (copies_only ? "/C_copies.bin" : "/C.bin")).c_str(), "wb");
  if (!f || std::fwrite(h_C[last], 1, cbytes, f) != cbytes) {
    std::fprintf(stderr, "cannot write %s/C.bin\n", dir.c_str());
    if (f) std::fclose(f);
    return 2;
  }
  std::fclose(f);
  std::printf("{\"ms_per_step\": %.6f, \"steps\": %d, \"warmup\": %d, \"plan\": \"%s\", "
              "\"h2d_bytes_per_step\": %zu, \"d2h_bytes_per_step\": %zu, \"device_status\": %d}\n",
              s * 1e3 / steps, steps, warmup, copies_only ? "none (copies only)" : reuse ? "reused" : "built every step",
              wbytes + bbytes, cbytes,
              dev_status);
  bsp_plan_destroy(plan0);
  return 0;
}
