// spmm.cu — CUDA-core bitmap SpMM kernels: C[M×N] = A·B, A packed LSB-first.
//
// "Multiply by one replaced by adds": row i of C is the sum of the rows k of
// B at A's set bits (reference backup/layout_trans.cu:158-171 did one global
// atomicAdd per set bit and column).  Here one warp owns a row and a chunk of
// columns, walks the row's set bits with __ffs in ascending column order,
// gathers D rows of B at a time with 16-byte vector loads (D gathers in
// flight per warp) and accumulates in FP32 registers in walk order.  Rows
// with more than 4096 set bits use a compensated two-term (TwoSum)
// accumulator.  Every output element is written once, without atomics, so
// results are deterministic run to run.
//
// Prototype mode (plans from plan.cu): a row i in cluster c is
//   C[i] = P[c] + Σ_{k ∈ A_i \ cons_c} B[k] − Σ_{k ∈ cons_c \ A_i} B[k],
// where P[c] = Σ_{k ∈ cons_c} B[k] is computed once per cluster by
// k_proto_sums (K split across the warps of a CTA, fixed-order reduction).
#include <cooperative_groups.h>

#include "ptx.cuh"
#include "spmm_dev.cuh"

namespace cg = cooperative_groups;

namespace bsp {
namespace {

// One warp per (row, column chunk of 32*VPL*COLS).  In PROTO launches, rows
// with a cluster walk their delta list and add P[c]; every other row walks
// A's words.  Rows with more than kCompThreshold set bits are summed with
// TwoSum one column vector at a time, which keeps the wide path's register
// budget unchanged.
template <typename BT, int VPL, int D, bool PROTO>
__global__ void __launch_bounds__(256) k_spmm_rows(SpmmArgs a) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = 32 * VPL * COLS;
  const int lane = threadIdx.x & 31;
  int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (a.row_list) {
    if (row >= a.n_list) return;
    row = __ldg(a.row_list + row);
  } else if (row >= a.M) {
    return;
  }
  const int n0 = (int)blockIdx.y * CW;
  const BT* __restrict__ B = static_cast<const BT*>(a.B);
  int col[VPL];
  bool cvalid[VPL];
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    col[v] = n0 + (v * 32 + lane) * COLS;
    cvalid[v] = col[v] < a.N;
  }
  float* crow = a.C + row * a.ldc;
  if (PROTO) {
    const int cl = __ldg(a.row_cluster + row);
    if (cl >= 0) {
      ListWalker wk;
      wk.init(a.delta_idx, __ldg(a.delta_ptr + row), __ldg(a.delta_ptr + row + 1), lane);
      Acc<VPL, COLS, false> acc;
      acc.zero();
      accumulate_walk<BT, VPL, D, false>(wk, B, a.ldb, col, cvalid, acc);
      store_vecs<VPL, COLS, false>(crow, col, cvalid, acc, a.P + (int64_t)cl * a.ldp);
      return;
    }
  }
  const uint32_t* arow = a.A + row * a.Kw;
  const int nnz = row_popcount(arow, (int)a.Kw, lane);
  if (nnz <= kCompThreshold) {
    BitWalker wk;
    wk.init(arow, 0, (int)a.Kw, lane);
    Acc<VPL, COLS, false> acc;
    acc.zero();
    accumulate_walk<BT, VPL, D, false>(wk, B, a.ldb, col, cvalid, acc);
    store_vecs<VPL, COLS, false>(crow, col, cvalid, acc, nullptr);
  } else {
    for (int v = 0; v < VPL; v++) {
      BitWalker wk;
      wk.init(arow, 0, (int)a.Kw, lane);
      Acc<1, COLS, true> acc;
      acc.zero();
      int c1[1] = {col[v]};
      bool ok[1] = {cvalid[v]};
      accumulate_walk<BT, 1, 4, true>(wk, B, a.ldb, c1, ok, acc);
      store_vecs<1, COLS, true>(crow, c1, ok, acc, nullptr);
    }
  }
}

// Prototype rows, register path: one warp per (clustered row, column chunk).
// The delta gathers are issued first; P[c] is read after griddep_wait(), so
// with programmatic dependent launch the whole gather phase overlaps the
// prototype-sum kernel.  MINB caps registers (occupancy sweep).  OFF32 = B's
// element offsets fit in 32 bits (K·ldb < 2^31) and FULL = every column
// chunk is whole (N a multiple of the chunk width); with 32-bit row
// arithmetic (M < 2^31, checked on the host) they keep the 8-blocks-per-SM
// shape within its 32 registers without spilling (a 12-byte spill cost the
// clustered 8192²×512 step 3 µs).
template <typename BT, int VPL, int D, int MINB, bool OFF32, bool FULL, bool SLOT>
__global__ void __launch_bounds__(256, MINB) k_spmm_proto_regs(SpmmArgs a) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = 32 * VPL * COLS;
  const int lane = threadIdx.x & 31;
  int row, cl;
  uint32_t slot = 0u;
  if (SLOT) {
    // warp p takes the p-th row slot (rows by descending delta count): row,
    // cluster and list in one load whose address depends on p alone
    const int p = (int)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (p < (int)a.n_slot) slot = __ldg(a.delta_pad + (int64_t)p * 32 + lane);
    row = (int)__shfl_sync(kFull, slot, 0);
    cl = p < (int)a.n_slot ? (int)__shfl_sync(kFull, slot, 1) : -1;
  } else {
    row = (int)blockIdx.x * 8 + (threadIdx.x >> 5);
    cl = row < (int)a.M ? __ldg(a.row_cluster + row) : -1;
  }
  if (cl >= 0) {
    const int n0 = (int)blockIdx.y * CW;
    const BT* __restrict__ B = static_cast<const BT*>(a.B);
    int col[VPL];
    bool cvalid[VPL];
#pragma unroll
    for (int v = 0; v < VPL; v++) {
      col[v] = n0 + (v * 32 + lane) * COLS;
      cvalid[v] = FULL || col[v] < (int)a.N;
    }
    Acc<VPL, COLS, false> acc;
    acc.zero();
    if (SLOT) {
      SlotWalker wk;
      wk.init(slot, a.delta_idx, lane);
      if (OFF32) accumulate_walk<BT, VPL, D, false>(wk, B, (uint32_t)a.ldb, col, cvalid, acc);
      else accumulate_walk<BT, VPL, D, false>(wk, B, a.ldb, col, cvalid, acc);
    } else {
      ListWalker wk;
      wk.init(a.delta_idx, __ldg(a.delta_ptr + row), __ldg(a.delta_ptr + row + 1), lane);
      if (OFF32) accumulate_walk<BT, VPL, D, false>(wk, B, (uint32_t)a.ldb, col, cvalid, acc);
      else accumulate_walk<BT, VPL, D, false>(wk, B, a.ldb, col, cvalid, acc);
    }
    ptx::griddep_wait();
    store_vecs<VPL, COLS, false>(a.C + (int64_t)row * a.ldc, col, cvalid, acc, a.P + (int64_t)cl * a.ldp);
  } else {
    ptx::griddep_wait();
  }
}

// Scalar fallback for unaligned or ragged layouts: lane = column.
template <typename BT>
__global__ void __launch_bounds__(256) k_spmm_rows_scalar(SpmmArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= a.M) return;
  const BT* __restrict__ B = static_cast<const BT*>(a.B);
  const uint32_t* arow = a.A + row * a.Kw;
  const int nnz = row_popcount(arow, (int)a.Kw, lane);
  const bool comp = nnz > kCompThreshold;
  for (int64_t n0 = (int64_t)blockIdx.y * 32; n0 < a.N; n0 += (int64_t)gridDim.y * 32) {
    const int64_t j = n0 + lane;
    float s = 0.f, c = 0.f;
    BitWalker wk;
    wk.init(arow, 0, (int)a.Kw, lane);
    for (uint32_t k = wk.next(); k != kEnd; k = wk.next()) {
      const float x = j < a.N ? to_f32(B[(int64_t)k * a.ldb + j]) : 0.f;
      if (comp) {
        const float t = s + x, bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
      } else {
        s += x;
      }
    }
    if (j < a.N) a.C[row * a.ldc + j] = comp ? s + c : s;
  }
}

// P[c][n0 .. n0+32*COLS) for one prototype per CTA row: warp w walks the
// prototype's words [w*Kw/W, (w+1)*Kw/W), partial sums meet in shared memory
// and are added in warp order.  COMP (the densest prototype has more than
// 4096 set bits): each warp keeps a TwoSum pair (sum, error) and the pairs
// are added with TwoSum too; P = sum + error.
template <typename BT, int D, bool COMP, bool OFF32>
__global__ void __launch_bounds__(512) k_proto_sums(SpmmArgs a) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = 32 * COLS;
  extern __shared__ float part[];  // [W][CW] sums, then (COMP) [W][CW] errors
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, W = blockDim.x >> 5;
  const int64_t c = blockIdx.x;
  const int64_t n0 = (int64_t)blockIdx.y * CW;
  const BT* __restrict__ B = static_cast<const BT*>(a.B);
  int col[1] = {(int)n0 + lane * COLS};
  bool cvalid[1] = {col[0] < a.N};
  ptx::griddep_launch_dependents();
  const uint32_t* cw = a.cons + c * a.Kw;
  const int w0 = (int)(a.Kw * wid / W), w1 = (int)(a.Kw * (wid + 1) / W);
  BitWalker wk;
  wk.init(cw, w0, w1, lane);
  Acc<1, COLS, COMP> acc;
  acc.zero();
  if (OFF32) accumulate_walk<BT, 1, D, COMP>(wk, B, (uint32_t)a.ldb, col, cvalid, acc);
  else accumulate_walk<BT, 1, D, COMP>(wk, B, a.ldb, col, cvalid, acc);
#pragma unroll
  for (int j = 0; j < COLS; j++) {
    part[wid * CW + lane * COLS + j] = acc.s[0][j];
    if (COMP) part[(W + wid) * CW + lane * COLS + j] = acc.c[0][COMP ? j : 0];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < CW; j += blockDim.x) {
    float s = 0.f, e = 0.f;
    for (int w = 0; w < W; w++) {
      const float x = part[w * CW + j];
      if (COMP) {
        const float t = s + x, bp = t - s;
        e += ((s - (t - bp)) + (x - bp)) + part[(W + w) * CW + j];
        s = t;
      } else {
        s += x;
      }
    }
    if (n0 + j < a.N) a.P[c * a.ldp + n0 + j] = COMP ? s + e : s;
  }
}

// P[c] over one chunk of CW = 32·VPL·COLS columns from the prototype's
// column list, by a cluster of 8 CTAs × 8 warps: warp p = rank·8 + w sums
// list entries [len·p/64, len·(p+1)/64) with one B slice in flight.  With 64
// short chains instead of 16 long ones the sums finish sooner (each gather
// waits out the L2 latency of a loaded GPU), and 256-thread CTAs at 32
// registers leave the SMs to the row kernel that runs beside them under
// programmatic dependent launch.  Each CTA adds its warps' partials in warp
// order; rank 0 adds the 8 CTA partials in rank order through distributed
// shared memory (all loads issued first), so P is the same on every run.
constexpr int kSumCluster = 8;
template <typename BT, int VPL, bool OFF32>
__global__ void __cluster_dims__(kSumCluster, 1, 1) __launch_bounds__(256) k_proto_sums_list(SpmmArgs a) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int CW = 32 * VPL * COLS;
  constexpr int PARTS = kSumCluster * 8;
  __shared__ float4 wp[8][CW / 4];
  __shared__ float4 cp[CW / 4];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int n0 = (int)(blockIdx.x / kSumCluster) * CW;
  const int64_t c = blockIdx.y;
  ptx::griddep_launch_dependents();
  int col[VPL];
  bool cvalid[VPL];
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    col[v] = n0 + (v * 32 + lane) * COLS;
    cvalid[v] = col[v] < (int)a.N;
  }
  const int s0 = __ldg(a.cons_ptr + c), len = __ldg(a.cons_ptr + c + 1) - s0;
  const int p = rank * 8 + wid;
  ListWalker wk;
  wk.init(a.cons_idx, s0 + (int)((int64_t)len * p / PARTS), s0 + (int)((int64_t)len * (p + 1) / PARTS), lane);
  Acc<VPL, COLS, false> acc;
  acc.zero();
  const BT* __restrict__ B = static_cast<const BT*>(a.B);
  if (OFF32) accumulate_walk<BT, VPL, 1, false>(wk, B, (uint32_t)a.ldb, col, cvalid, acc);
  else accumulate_walk<BT, VPL, 1, false>(wk, B, a.ldb, col, cvalid, acc);
  float* w = reinterpret_cast<float*>(&wp[wid][0]);
#pragma unroll
  for (int v = 0; v < VPL; v++)
#pragma unroll
    for (int j = 0; j < COLS; j++) w[(v * 32 + lane) * COLS + j] = acc.result(v, j);
  __syncthreads();
  if (threadIdx.x < CW / 4) {
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const float4 x = wp[u][threadIdx.x];
      t.x += x.x;
      t.y += x.y;
      t.z += x.z;
      t.w += x.w;
    }
    cp[threadIdx.x] = t;
  }
  cluster.sync();
  if (rank == 0 && threadIdx.x < CW / 4) {
    float4 x[kSumCluster];
#pragma unroll
    for (int r = 0; r < kSumCluster; r++) x[r] = cluster.map_shared_rank(cp, r)[threadIdx.x];
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int r = 0; r < kSumCluster; r++) {
      t.x += x[r].x;
      t.y += x[r].y;
      t.z += x[r].z;
      t.w += x[r].w;
    }
    // P rows are ldp = ceil8(N) floats: a float4 starting below N stays in the row
    if (n0 + 4 * (int)threadIdx.x < (int)a.N) reinterpret_cast<float4*>(a.P + c * a.ldp + n0)[threadIdx.x] = t;
  }
  cluster.sync();
}

template <typename BT>
int launch_rows_t(const SpmmArgs& a, bool proto, bool vec, cudaStream_t s) {
  constexpr int COLS = Vec<BT>::COLS;
  const unsigned gx = (unsigned)ceil_div(a.row_list ? a.n_list : a.M, 8);
  if (gx == 0) return BSP_OK;
  if (!vec) {
    if (proto) return BSP_ERR_INTERNAL;
    const int64_t gy = ceil_div(a.N, 32) < 65535 ? ceil_div(a.N, 32) : 65535;
    k_spmm_rows_scalar<BT><<<dim3(gx, (unsigned)gy), 256, 0, s>>>(a);
    BSP_LAUNCHED();
    return BSP_OK;
  }
  // columns per warp: up to 4 vectors per lane for FP32, 2 for 16-bit B
  constexpr int VPL_MAX = COLS == 4 ? 4 : 2;
  const int64_t per1 = 32 * COLS;
  if (a.N <= per1) {
    const dim3 g(gx, (unsigned)ceil_div(a.N, per1));
    if (proto) k_spmm_rows<BT, 1, 16, true><<<g, 256, 0, s>>>(a);
    else k_spmm_rows<BT, 1, 16, false><<<g, 256, 0, s>>>(a);
  } else if (a.N <= 2 * per1 || VPL_MAX == 2) {
    const dim3 g(gx, (unsigned)ceil_div(a.N, 2 * per1));
    if (proto) k_spmm_rows<BT, 2, 8, true><<<g, 256, 0, s>>>(a);
    else k_spmm_rows<BT, 2, 8, false><<<g, 256, 0, s>>>(a);
  } else {
    const dim3 g(gx, (unsigned)ceil_div(a.N, 4 * per1));
    if (proto) k_spmm_rows<BT, 4, 4, true><<<g, 256, 0, s>>>(a);
    else k_spmm_rows<BT, 4, 4, false><<<g, 256, 0, s>>>(a);
  }
  BSP_LAUNCHED();
  return BSP_OK;
}

// BSP_SLOT_LISTS=0: rows in index order, each list read through its bounds
// (for comparisons).
bool slot_lists_enabled() {
  static const bool on = [] {
    const char* e = getenv("BSP_SLOT_LISTS");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <typename BT, int VPL, int D, int MINB>
int launch_proto_regs_t(const SpmmArgs& a, cudaStream_t s) {
  constexpr int CW = 32 * VPL * Vec<BT>::COLS;
  cudaLaunchConfig_t cfg = {};
  const bool off32 = a.K * a.ldb < ((int64_t)1 << 31), full = a.N % CW == 0;
  const bool slot = off32 && a.delta_pad && a.n_slot > 0 && slot_lists_enabled();
  cfg.gridDim = dim3((unsigned)ceil_div(slot ? a.n_slot : a.M, 8), (unsigned)ceil_div(a.N, CW));
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (slot && full)
    BSP_CUDA(cudaLaunchKernelEx(&cfg, k_spmm_proto_regs<BT, VPL, D, MINB, true, true, true>, a));
  else if (slot)
    BSP_CUDA(cudaLaunchKernelEx(&cfg, k_spmm_proto_regs<BT, VPL, D, MINB, true, false, true>, a));
  else if (off32 && full)
    BSP_CUDA(cudaLaunchKernelEx(&cfg, k_spmm_proto_regs<BT, VPL, D, MINB, true, true, false>, a));
  else if (off32)
    BSP_CUDA(cudaLaunchKernelEx(&cfg, k_spmm_proto_regs<BT, VPL, D, MINB, true, false, false>, a));
  else
    BSP_CUDA(cudaLaunchKernelEx(&cfg, k_spmm_proto_regs<BT, VPL, D, MINB, false, false, false>, a));
  return BSP_OK;
}

template <typename BT>
int launch_proto_regs_v(const SpmmArgs& a, int variant, cudaStream_t s) {
  constexpr bool F32 = Vec<BT>::COLS == 4;
  // variants: columns per warp (VPL vectors per lane), gathers in flight (D), min blocks/SM
  if (a.N <= 32 * Vec<BT>::COLS) return launch_proto_regs_t<BT, 1, 16, 3>(a, s);
  switch (variant) {
    case 1: return launch_proto_regs_t<BT, 2, 4, 4>(a, s);
    case 2: return launch_proto_regs_t<BT, (F32 ? 4 : 2), 1, 5>(a, s);
    case 3: return launch_proto_regs_t<BT, 2, 2, 6>(a, s);
    case 4: return launch_proto_regs_t<BT, 2, 1, 8>(a, s);
    case 5: return launch_proto_regs_t<BT, 1, 4, 8>(a, s);
    case 6: return launch_proto_regs_t<BT, 2, 2, 5>(a, s);
    case 7: return launch_proto_regs_t<BT, (F32 ? 4 : 2), 1, 6>(a, s);
    case 8: return launch_proto_regs_t<BT, (F32 ? 4 : 2), 3, 3>(a, s);
    default: return launch_proto_regs_t<BT, (F32 ? 4 : 2), 2, 4>(a, s);
  }
}

template <typename BT>
int launch_proto_t(const SpmmArgs& a, cudaStream_t s) {
  constexpr int VPL = Vec<BT>::COLS == 4 ? 2 : 1;
  constexpr int CWL = 32 * VPL * Vec<BT>::COLS;
  const bool comp = a.proto_max_nnz > kCompThreshold;
  // From the column lists, B slices staged by bulk copies when B's rows are
  // 16-byte aligned (BSP_SUMS_BULK = -1 selects the cluster form below, n >=
  // 0 a staging shape; defaults measured at 8192x8192x512: FP32 23.4 -> 22.8
  // us a step, BF16 20.1 -> 16.9 us)
  static const int sv = getenv("BSP_SUMS_BULK") ? atoi(getenv("BSP_SUMS_BULK")) : (sizeof(BT) == 4 ? 1 : 8);
  const int esz = (int)sizeof(BT);
  if (sv >= 0 && a.cons_idx && !comp && a.n_proto <= 65535 && reinterpret_cast<uintptr_t>(a.B) % 16 == 0 &&
      (a.ldb * esz) % 16 == 0 && (a.N * esz) % 16 == 0) {
    const int rc = launch_proto_sums_bulk(a, sv, s);
    if (rc != BSP_ERR_UNSUPPORTED) return rc;  // a shape too large for this B type: the cluster form
  }
  if (a.cons_idx && !comp && a.n_proto <= 65535 && ceil_div(a.N, CWL) * kSumCluster <= 0x7fffffff) {
    const dim3 g((unsigned)(ceil_div(a.N, CWL) * kSumCluster), (unsigned)a.n_proto);
    if (a.K * a.ldb < ((int64_t)1 << 31)) k_proto_sums_list<BT, VPL, true><<<g, 256, 0, s>>>(a);
    else k_proto_sums_list<BT, VPL, false><<<g, 256, 0, s>>>(a);
    BSP_LAUNCHED();
    return BSP_OK;
  }
  constexpr int CW = 32 * Vec<BT>::COLS;
  const int threads = 512;
  const size_t smem = (size_t)(threads / 32) * CW * sizeof(float) * (comp ? 2 : 1);
  const dim3 g((unsigned)a.n_proto, (unsigned)ceil_div(a.N, CW));
  const bool off32 = a.K * a.ldb < ((int64_t)1 << 31);
  if (comp && off32) k_proto_sums<BT, 8, true, true><<<g, threads, smem, s>>>(a);
  else if (comp) k_proto_sums<BT, 8, true, false><<<g, threads, smem, s>>>(a);
  else if (off32) k_proto_sums<BT, 8, false, true><<<g, threads, smem, s>>>(a);
  else k_proto_sums<BT, 8, false, false><<<g, threads, smem, s>>>(a);
  BSP_LAUNCHED();
  return BSP_OK;
}

// SDDMM on CUDA cores: warp per row i of A; the row of dA is zeroed, then for
// every set bit k (ascending) the lanes stride over N accumulating
// G[i][j]·X[k][j] in FP32 and a warp reduction writes dA[i][k].
template <typename T>
__global__ void __launch_bounds__(256) k_sddmm_rows(const uint32_t* __restrict__ A, int64_t M, int64_t K,
                                                    int64_t Kw, const T* __restrict__ G, int64_t ldg,
                                                    const T* __restrict__ X, int64_t ldx, int64_t N,
                                                    float* __restrict__ dA, int64_t ldda) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= M) return;
  float* out = dA + row * ldda;
  for (int64_t k = lane; k < K; k += 32) out[k] = 0.f;
  __syncwarp();
  const T* g = G + row * ldg;
  BitWalker wk;
  wk.init(A + row * Kw, 0, (int)Kw, lane);
  for (uint32_t k = wk.next(); k != kEnd; k = wk.next()) {
    const T* x = X + (int64_t)k * ldx;
    float s = 0.f;
    for (int64_t j = lane; j < N; j += 32) s = fmaf(to_f32(g[j]), to_f32(x[j]), s);
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    if (lane == 0) out[k] = s;
  }
}

}  // namespace

int launch_sddmm_rows(const uint32_t* A, int64_t M, int64_t K, const void* G, int64_t ldg, const void* X,
                      int64_t ldx, int dt, int64_t N, float* dA, int64_t ldda, cudaStream_t s) {
  if (M == 0 || K == 0) return BSP_OK;
  const unsigned grid = (unsigned)ceil_div(M, 8);
  const int64_t Kw = ceil_div(K, 32);
  switch (dt) {
    case BSP_F32: k_sddmm_rows<float><<<grid, 256, 0, s>>>(A, M, K, Kw, (const float*)G, ldg, (const float*)X, ldx, N, dA, ldda); break;
    case BSP_BF16: k_sddmm_rows<__nv_bfloat16><<<grid, 256, 0, s>>>(A, M, K, Kw, (const __nv_bfloat16*)G, ldg, (const __nv_bfloat16*)X, ldx, N, dA, ldda); break;
    case BSP_F16: k_sddmm_rows<__half><<<grid, 256, 0, s>>>(A, M, K, Kw, (const __half*)G, ldg, (const __half*)X, ldx, N, dA, ldda); break;
    default: return BSP_ERR_UNSUPPORTED;
  }
  BSP_LAUNCHED();
  return BSP_OK;
}

int launch_spmm_rows(const SpmmArgs& a, bool proto, bool vec, cudaStream_t s) {
  if (a.M == 0 || a.N == 0) return BSP_OK;
  switch (a.bdt) {
    case BSP_F32: return launch_rows_t<float>(a, proto, vec, s);
    case BSP_BF16: return launch_rows_t<__nv_bfloat16>(a, proto, vec, s);
    case BSP_F16: return launch_rows_t<__half>(a, proto, vec, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

int launch_spmm_proto_regs(const SpmmArgs& a, int variant, cudaStream_t s) {
  if (a.M == 0 || a.N == 0) return BSP_OK;
  switch (a.bdt) {
    case BSP_F32: return launch_proto_regs_v<float>(a, variant, s);
    case BSP_BF16: return launch_proto_regs_v<__nv_bfloat16>(a, variant, s);
    case BSP_F16: return launch_proto_regs_v<__half>(a, variant, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

int launch_proto_sums(const SpmmArgs& a, cudaStream_t s) {
  if (a.n_proto == 0 || a.N == 0) return BSP_OK;
  switch (a.bdt) {
    case BSP_F32: return launch_proto_t<float>(a, s);
    case BSP_BF16: return launch_proto_t<__nv_bfloat16>(a, s);
    case BSP_F16: return launch_proto_t<__half>(a, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

}  // namespace bsp
