// spmm_stream.cu — prototype-mode SpMM, streaming form.
//
// 1. Prototype sums P = cons·B by streaming B (k_proto_stream): a CTA owns a
//    block of R consecutive rows of B and one column chunk; it stages those
//    R row slices in shared memory with one TMA bulk copy per row (all in
//    flight at once), then warp w adds every staged row k into the partial
//    sums of the prototypes c ≡ w (mod 8) that contain k, k ascending —
//    each (prototype, column) accumulator has one owner, so the result is
//    deterministic.  k_proto_reduce adds the per-block partials in block
//    order.  B is read exactly once.
// 2. Clustered rows (k_spmm_proto_stream): each warp owns a contiguous block
//    of rows and consumes one flat stream of items — "row start (cluster c)"
//    followed by the row's ± delta columns — in batches of D gathers that
//    run across row boundaries.  The stream's index windows are prefetched
//    one window ahead and P[c] is prefetched when a row starts, so no
//    dependent load sits between two batches of gathers.
// The three kernels are chained with programmatic dependent launch.
#include "ptx.cuh"
#include "spmm_dev.cuh"

namespace bsp {

__device__ int g_stream_error;

namespace {

constexpr uint32_t kSubtract = 0x80000000u;
constexpr uint32_t kRowStart = 0x40000000u;
constexpr uint32_t kIndexMask = 0x3fffffffu;

// ---------------------------------------------------------------------------
// prototype sums
constexpr int kPsWarps = 8;
constexpr int kPsProtos = 64;  // prototypes per CTA (grid.z groups)

template <typename BT>
struct PsShape {
  static constexpr int COLS = Vec<BT>::COLS;
  static constexpr int CW = 32 * COLS;  // columns per CTA
};

// smem: staged B rows [R][CW] of BT, partial sums [64][CW] floats, 1 mbarrier
template <typename BT>
__global__ void __launch_bounds__(kPsWarps * 32) k_proto_stream(SpmmArgs a, const uint32_t* __restrict__ consT,
                                                                int Pw, int rows_per_block,
                                                                float* __restrict__ partial) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = PsShape<BT>::CW;
  extern __shared__ __align__(128) uint8_t smem[];
  const int R = rows_per_block;
  BT* Bs = reinterpret_cast<BT*>(smem);
  float* Ps = reinterpret_cast<float*>(smem + (size_t)R * CW * sizeof(BT));
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + (size_t)R * CW * sizeof(BT) +
                                              (size_t)kPsProtos * CW * sizeof(float));
  ptx::griddep_launch_dependents();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k0 = min((int64_t)blockIdx.x * R, a.K);
  const int64_t k1 = min(a.K, k0 + R);
  const int n0 = (int)blockIdx.y * CW;
  const int ncols = min(CW, (int)(a.N - n0));
  const int c0 = (int)blockIdx.z * kPsProtos;
  const int nprot = min(kPsProtos, (int)(a.n_proto - c0));
  const uint32_t row_bytes = (uint32_t)ncols * sizeof(BT);
  const int nrows = (int)(k1 - k0);  // 0 ≤ nrows ≤ R ≤ kPsMaxRows (host guarantees nrows ≥ 1)
  if (threadIdx.x == 0) {
    ptx::mbar_init(bar, 1);
    ptx::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) ptx::mbar_arrive_expect_tx(bar, row_bytes * (uint32_t)nrows);
  __syncthreads();
  const BT* Bsrc = static_cast<const BT*>(a.B) + n0;
  for (int r = threadIdx.x; r < nrows; r += blockDim.x)
    ptx::bulk_g2s(Bs + (size_t)r * CW, Bsrc + (k0 + r) * a.ldb, row_bytes, bar);
  // zero the owned partial rows while the copies fly
  for (int c = warp; c < kPsProtos; c += kPsWarps)
#pragma unroll
    for (int j = 0; j < COLS; j++) Ps[c * CW + lane * COLS + j] = 0.f;
  const bool ok = ptx::mbar_wait(bar, 0);
  if (!ok) {
    if (lane == 0) atomicCAS(&g_stream_error, 0, 2);
    return;
  }
  const bool cvalid = lane * COLS < ncols;
  // owned prototypes: c_local ≡ warp (mod 8) among the first nprot
  uint64_t own = 0;
  for (int c = warp; c < nprot; c += kPsWarps) own |= 1ull << c;
  const int wlo = (c0 >> 5), whi = wlo + 1;
  for (int kb = 0; kb < nrows; kb += 32) {
    const int64_t k = k0 + kb + lane;
    uint64_t m = 0;
    if (kb + lane < nrows) {
      const uint32_t lo = __ldg(consT + k * Pw + wlo);
      const uint32_t hi = whi < Pw ? __ldg(consT + k * Pw + whi) : 0u;
      m = ((uint64_t)lo | ((uint64_t)hi << 32)) & own;
    }
    const int lim = min(32, nrows - kb);
    for (int j = 0; j < lim; j++) {
      uint64_t mj = __shfl_sync(kFull, m, j);
      if (!mj) continue;
      float f[COLS];
      if (cvalid) {
        const typename V::Raw raw =
            *reinterpret_cast<const typename V::Raw*>(Bs + (size_t)(kb + j) * CW + lane * COLS);
        V::cvt(raw, f);
      }
      while (mj) {
        const int c = __ffsll((long long)mj) - 1;
        mj &= mj - 1;
        if (cvalid) {
          float* p = Ps + c * CW + lane * COLS;
#pragma unroll
          for (int q = 0; q < COLS; q++) p[q] += f[q];
        }
      }
    }
  }
  __syncwarp();
  // write the owned partial rows: partial[block][c][n]
  float* out = partial + ((int64_t)blockIdx.x * a.n_proto + c0) * a.ldp + n0;
  for (int c = warp; c < nprot; c += kPsWarps)
    if (cvalid)
#pragma unroll
      for (int q = 0; q < COLS; q += 4)
        *reinterpret_cast<float4*>(out + (int64_t)c * a.ldp + lane * COLS + q) =
            *reinterpret_cast<const float4*>(Ps + c * CW + lane * COLS + q);
}

// P[c][n] = Σ_g partial[g][c][n], g ascending.
__global__ void __launch_bounds__(256) k_proto_reduce(SpmmArgs a, int G, const float* __restrict__ partial) {
  ptx::griddep_launch_dependents();
  ptx::griddep_wait();
  const int64_t total = a.n_proto * a.ldp;
  const int64_t stride = a.n_proto * a.ldp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int g = 0; g < G; g++) s += partial[g * stride + i];
    a.P[i] = s;
  }
}

// ---------------------------------------------------------------------------
// clustered rows
template <typename BT, int VPL, int D, int MINB>
__global__ void __launch_bounds__(256, MINB) k_spmm_proto_stream(SpmmArgs a) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = 32 * VPL * COLS;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t rpw = (a.M + nwarps - 1) / nwarps;
  int64_t row = gw * rpw;
  const int64_t r_end = min(a.M, row + rpw);
  const int n0 = (int)blockIdx.y * CW;
  const BT* __restrict__ B = static_cast<const BT*>(a.B) + n0;
  const float* __restrict__ P = a.P + n0;
  float* __restrict__ C = a.C + n0;
  const int n_delta = (int)a.n_delta;
  int col[VPL];
  bool cvalid[VPL];
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    col[v] = (v * 32 + lane) * COLS;
    cvalid[v] = n0 + col[v] < a.N;
  }
  if (row >= r_end) {
    ptx::griddep_wait();
    return;
  }
  // row window (pointers, clusters) and entry windows
  int64_t pbase = row;
  int win_p = 0, win_c = -1, nextp = 0;
  auto load_rows = [&]() {
    win_p = (pbase + lane <= a.M) ? __ldg(a.delta_ptr + pbase + lane) : 0;
    win_c = (pbase + lane < a.M) ? __ldg(a.row_cluster + pbase + lane) : -1;
    nextp = __ldg(a.delta_ptr + min(pbase + 32, a.M));
  };
  load_rows();
  auto ptr_of = [&](int64_t r) -> int {
    const int off = (int)(r - pbase);
    const int v = __shfl_sync(kFull, win_p, off & 31);
    return off < 32 ? v : nextp;
  };
  int e = ptr_of(row);
  int wbase = e;
  uint32_t win_e = (wbase + lane < n_delta) ? __ldg(a.delta_idx + wbase + lane) : 0u;
  uint32_t win_n = (wbase + 32 + lane < n_delta) ? __ldg(a.delta_idx + wbase + 32 + lane) : 0u;
  bool started = false;
  ptx::griddep_wait();  // P is complete from here on

  float acc[VPL][COLS], pcur[VPL][COLS];
  int acc_row = -1;
  auto store = [&]() {
    float* crow = C + (int64_t)acc_row * a.ldc;
#pragma unroll
    for (int v = 0; v < VPL; v++) {
      if (!cvalid[v]) continue;
#pragma unroll
      for (int j = 0; j < COLS; j += 4)
        *reinterpret_cast<float4*>(crow + col[v] + j) =
            make_float4(acc[v][j] + pcur[v][j], acc[v][j + 1] + pcur[v][j + 1],
                        acc[v][j + 2] + pcur[v][j + 2], acc[v][j + 3] + pcur[v][j + 3]);
    }
  };

  while (true) {
    // produce up to D items: lane s holds item s
    int n = 0;
    int my_row = -1;
    uint32_t my_e = 0;
    while (n < D && row < r_end) {
      if (row >= pbase + 32) {
        pbase = row;
        load_rows();
      }
      const int c = __shfl_sync(kFull, win_c, (int)(row - pbase));
      if (c < 0) {
        row++;
        continue;
      }
      if (!started) {
        if (lane == n) {
          my_row = (int)row;
          my_e = kRowStart | (uint32_t)c;
        }
        n++;
        started = true;
        continue;
      }
      const int re = ptr_of(row + 1);
      if (e < re) {
        if (e >= wbase + 32) {
          wbase += 32;
          win_e = win_n;
          win_n = (wbase + 32 + lane < n_delta) ? __ldg(a.delta_idx + wbase + 32 + lane) : 0u;
        }
        const int take = min(min(D - n, re - e), wbase + 32 - e);
        const uint32_t v = __shfl_sync(kFull, win_e, (lane - n + (e - wbase)) & 31);
        if (lane >= n && lane < n + take) {
          my_row = (int)row;
          my_e = v;
        }
        n += take;
        e += take;
      }
      if (e >= re) {
        row++;
        started = false;
      }
    }
    if (n == 0) break;
    uint32_t it[D];
    typename V::Raw raw[D][VPL];
#pragma unroll
    for (int s = 0; s < D; s++) {
      it[s] = __shfl_sync(kFull, my_e, s);
      if (s < n && !(it[s] & kRowStart)) {
        const BT* brow = B + (int64_t)(it[s] & kIndexMask) * a.ldb;
#pragma unroll
        for (int v = 0; v < VPL; v++)
          if (cvalid[v]) raw[s][v] = V::load(brow + col[v]);
      }
    }
#pragma unroll
    for (int s = 0; s < D; s++) {
      if (s >= n) break;
      if (it[s] & kRowStart) {
        if (acc_row >= 0) store();
        acc_row = __shfl_sync(kFull, my_row, s);
        const float* prow = P + (int64_t)(it[s] & kIndexMask) * a.ldp;
#pragma unroll
        for (int v = 0; v < VPL; v++) {
#pragma unroll
          for (int j = 0; j < COLS; j++) acc[v][j] = 0.f;
          if (cvalid[v]) {
#pragma unroll
            for (int j = 0; j < COLS; j += 4) {
              const float4 p = __ldg(reinterpret_cast<const float4*>(prow + col[v] + j));
              pcur[v][j] = p.x; pcur[v][j + 1] = p.y; pcur[v][j + 2] = p.z; pcur[v][j + 3] = p.w;
            }
          }
        }
      } else {
        const bool neg = (it[s] & kSubtract) != 0u;
#pragma unroll
        for (int v = 0; v < VPL; v++) {
          if (!cvalid[v]) continue;
          float f[COLS];
          V::cvt(raw[s][v], f);
#pragma unroll
          for (int j = 0; j < COLS; j++) acc[v][j] += neg ? -f[j] : f[j];
        }
      }
    }
  }
  if (acc_row >= 0) store();
}

cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <typename BT>
int launch_proto_stream_t(const SpmmArgs& a, const uint32_t* consT, int Pw, float* partial,
                          int rows_per_block, int G, cudaStream_t s) {
  constexpr int CW = PsShape<BT>::CW;
  const size_t smem = (size_t)rows_per_block * CW * sizeof(BT) + (size_t)kPsProtos * CW * sizeof(float) + 16;
  static bool configured[64] = {false};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(k_proto_stream<BT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448));
    configured[dev] = true;
  }
  const dim3 grid((unsigned)G, (unsigned)ceil_div(a.N, CW), (unsigned)ceil_div(a.n_proto, kPsProtos));
  k_proto_stream<BT><<<grid, kPsWarps * 32, smem, s>>>(a, consT, Pw, rows_per_block, partial);
  BSP_LAUNCHED();
  cudaLaunchAttribute attr[1];
  const int64_t total = a.n_proto * a.ldp;
  int rb = (int)ceil_div(total, 256);
  if (rb > num_sms() * 8) rb = num_sms() * 8;
  cudaLaunchConfig_t cfg = pdl_config(dim3((unsigned)rb), dim3(256), 0, s, attr);
  BSP_CUDA(cudaLaunchKernelEx(&cfg, k_proto_reduce, a, G, (const float*)partial));
  return BSP_OK;
}

template <typename BT, int VPL, int D, int MINB>
int launch_rows_stream_t(const SpmmArgs& a, cudaStream_t s) {
  constexpr int CW = 32 * VPL * Vec<BT>::COLS;
  const int64_t chunks = ceil_div(a.N, CW);
  int occ = 0;
  BSP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_spmm_proto_stream<BT, VPL, D, MINB>, 256, 0));
  if (occ < 1) occ = 1;
  int64_t gx = ceil_div((int64_t)num_sms() * occ, chunks);
  const int64_t max_gx = ceil_div(a.M, 8);
  if (gx > max_gx) gx = max_gx;
  if (gx < 1) gx = 1;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pdl_config(dim3((unsigned)gx, (unsigned)chunks), dim3(256), 0, s, attr);
  BSP_CUDA(cudaLaunchKernelEx(&cfg, k_spmm_proto_stream<BT, VPL, D, MINB>, a));
  return BSP_OK;
}

template <typename BT>
int launch_rows_stream_v(const SpmmArgs& a, int variant, cudaStream_t s) {
  constexpr bool F32 = Vec<BT>::COLS == 4;
  if (a.N <= 32 * Vec<BT>::COLS) return launch_rows_stream_t<BT, 1, 8, 4>(a, s);
  switch (variant) {
    case 1: return launch_rows_stream_t<BT, 1, 8, 4>(a, s);
    case 2: return launch_rows_stream_t<BT, 2, 3, 4>(a, s);
    case 3: return launch_rows_stream_t<BT, 1, 6, 4>(a, s);
    case 4: return launch_rows_stream_t<BT, (F32 ? 4 : 2), 2, 3>(a, s);
    case 5: return launch_rows_stream_t<BT, 2, 4, 2>(a, s);
    case 6: return launch_rows_stream_t<BT, (F32 ? 4 : 2), 4, 2>(a, s);
    case 7: return launch_rows_stream_t<BT, 1, 8, 3>(a, s);
    default: return launch_rows_stream_t<BT, 2, 4, 3>(a, s);
  }
}

}  // namespace

// Blocks of the prototype-sum stream: R rows of B per CTA, R ≤ kPsMaxRows
// (shared memory: R*512 B staged rows + 64*CW*4 B partial sums), and about
// one CTA per SM.  G = ceil(K/R), so every CTA gets 1..R rows — the byte
// count each CTA announces to its mbarrier is R*512 ≤ 160 KB, inside the
// 2^20-1 limit of mbarrier.expect_tx.
size_t proto_stream_partial_bytes(int64_t K, int64_t n_proto, int64_t ldp, int* G, int* rows_per_block) {
  constexpr int64_t kPsMaxRows = 320;
  int64_t g = ceil_div(K, kPsMaxRows);
  if (g < num_sms()) g = num_sms();
  if (g > K) g = K;
  if (g < 1) g = 1;
  const int64_t R = ceil_div(K, g);
  g = ceil_div(K, R);
  *G = (int)g;
  *rows_per_block = (int)R;
  return sizeof(float) * (size_t)g * (size_t)n_proto * (size_t)ldp;
}

int launch_proto_sums_stream(const SpmmArgs& a, const uint32_t* consT, int Pw, float* partial,
                             cudaStream_t s) {
  if (a.n_proto == 0 || a.N == 0) return BSP_OK;
  int G = 0, R = 0;
  proto_stream_partial_bytes(a.K, a.n_proto, a.ldp, &G, &R);
  switch (a.bdt) {
    case BSP_F32: return launch_proto_stream_t<float>(a, consT, Pw, partial, R, G, s);
    case BSP_BF16: return launch_proto_stream_t<__nv_bfloat16>(a, consT, Pw, partial, R, G, s);
    case BSP_F16: return launch_proto_stream_t<__half>(a, consT, Pw, partial, R, G, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

int launch_spmm_proto_stream(const SpmmArgs& a, int variant, cudaStream_t s) {
  if (a.M == 0 || a.N == 0) return BSP_OK;
  switch (a.bdt) {
    case BSP_F32: return launch_rows_stream_v<float>(a, variant, s);
    case BSP_BF16: return launch_rows_stream_v<__nv_bfloat16>(a, variant, s);
    case BSP_F16: return launch_rows_stream_v<__half>(a, variant, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

int stream_device_error(int* out, bool clear) {
  BSP_CUDA(cudaMemcpyFromSymbol(out, g_stream_error, sizeof(int)));
  if (clear) {
    const int zero = 0;
    BSP_CUDA(cudaMemcpyToSymbol(g_stream_error, &zero, sizeof(int)));
  }
  return BSP_OK;
}

}  // namespace bsp
