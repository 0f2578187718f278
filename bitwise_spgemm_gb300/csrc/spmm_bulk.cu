// spmm_bulk.cu — prototype-mode SpMM with B rows staged in shared memory by
// TMA bulk copies (cp.async.bulk + mbarrier), the GB300 form of "add the B
// row of every set bit" (reference backup/layout_trans.cu:158-171).
//
// Each warp owns a contiguous block of rows.  Its work is one stream of
// 2 KB column slices: for every clustered row, first the slice of the
// prototype sum P[c], then the slices of B at the row's delta columns.  The
// warp keeps S stages of SLOTS slices in flight: one lane per slot issues a
// bulk copy into the stage buffer, the stage's mbarrier counts the bytes,
// and the warp adds a completed stage from shared memory (16-byte LDS,
// conflict-free) while the other stages are still in flight.  A slot tagged
// as a P slice starts a new row (the previous row is stored).  The bytes in
// flight per SM (up to S*SLOTS*2 KB per warp) no longer depend on register
// count or occupancy, and the index stream is prefetched one 32-entry window
// ahead, so the kernel runs at the L2→SM gather rate.
//
// Every mbarrier wait is bounded; on timeout the kernel records error 1 in
// g_bulk_error, waits (bounded) for its other stages and returns.
#include "ptx.cuh"
#include "spmm_dev.cuh"

namespace bsp {

__device__ int g_bulk_error;

namespace {

constexpr uint32_t kSubtract = 0x80000000u;
constexpr uint32_t kProtoTag = 0x40000000u;
constexpr uint32_t kIndexMask = 0x3fffffffu;
constexpr int kSlotBytes = 2048;
constexpr int kChunkCols = 512;  // columns per slice; FP32 P slice = 2 KB

template <int WARPS, int S, int SLOTS>
struct BulkLayout {
  static constexpr size_t kBuf = (size_t)WARPS * S * SLOTS * kSlotBytes;
  static constexpr size_t kBars = (size_t)WARPS * S * sizeof(uint64_t);
  static constexpr size_t kMeta = (size_t)WARPS * S * SLOTS * sizeof(int2);
  static constexpr size_t kCnt = (size_t)WARPS * S * sizeof(int);
  static constexpr size_t kTotal = kBuf + kBars + kMeta + kCnt;
};

template <typename BT, int WARPS, int S, int SLOTS>
__global__ void __launch_bounds__(WARPS * 32, 1) k_spmm_proto_bulk(SpmmArgs a, int n_delta) {
  using V = Vec<BT>;
  constexpr int COLS = V::COLS;
  constexpr int VPL = kChunkCols / (32 * COLS);
  using L = BulkLayout<WARPS, S, SLOTS>;
  static_assert(SLOTS <= 32, "one lane per slot");
  static_assert(L::kTotal <= 232448, "shared memory");
  extern __shared__ __align__(1024) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t* buf = smem + (size_t)warp * S * SLOTS * kSlotBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::kBuf) + warp * S;
  int2* meta = reinterpret_cast<int2*>(smem + L::kBuf + L::kBars) + warp * S * SLOTS;
  int* cnt = reinterpret_cast<int*>(smem + L::kBuf + L::kBars + L::kMeta) + warp * S;

  // rows of this warp: one contiguous block
  const int64_t nwarps = (int64_t)gridDim.x * WARPS;
  const int64_t gw = (int64_t)blockIdx.x * WARPS + warp;
  const int64_t rpw = (a.M + nwarps - 1) / nwarps;
  int64_t row = gw * rpw;
  const int64_t r_end = min(a.M, row + rpw);
  if (row >= r_end) return;

  if (lane == 0)
    for (int s = 0; s < S; s++) ptx::mbar_init(&bars[s], 1);
  ptx::fence_mbar_init();
  __syncwarp();

  const int n0 = (int)blockIdx.y * kChunkCols;
  const int ncols = min(kChunkCols, (int)(a.N - n0));
  const uint32_t b_bytes = (uint32_t)ncols * (uint32_t)sizeof(BT);
  const uint32_t p_bytes = (uint32_t)ncols * 4u;
  const BT* Bn = static_cast<const BT*>(a.B) + n0;
  const float* Pn = a.P + n0;
  int col[VPL];
  bool cvalid[VPL];
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    col[v] = (v * 32 + lane) * COLS;
    cvalid[v] = col[v] < ncols;
  }

  // row window: pointers and clusters of rows pbase .. pbase+31
  int64_t pbase = row;
  int win_p = 0, win_c = -1, nextp = 0;
  auto load_rows = [&]() {
    win_p = (pbase + lane <= a.M) ? __ldg(a.delta_ptr + pbase + lane) : 0;
    win_c = (pbase + lane < a.M) ? __ldg(a.row_cluster + pbase + lane) : -1;
    nextp = __ldg(a.delta_ptr + min(pbase + 32, a.M));
  };
  load_rows();
  auto ptr_of = [&](int64_t r) -> int {  // r in [pbase, pbase+32]
    const int off = (int)(r - pbase);
    const int v = __shfl_sync(kFull, win_p, off & 31);
    return off < 32 ? v : nextp;
  };
  // entry windows: [wbase, wbase+32) current, next 32 prefetched
  int e = ptr_of(row);
  int wbase = e;
  uint32_t win_e = (wbase + lane < n_delta) ? __ldg(a.delta_idx + wbase + lane) : 0u;
  uint32_t win_n = (wbase + 32 + lane < n_delta) ? __ldg(a.delta_idx + wbase + 32 + lane) : 0u;
  bool p_done = false;

  auto fill = [&](int s) {
    int n = 0;
    int my_row = -1;
    uint32_t my_e = 0;
    while (n < SLOTS && row < r_end) {
      if (row >= pbase + 32) {
        pbase = row;
        load_rows();
      }
      const int c = __shfl_sync(kFull, win_c, (int)(row - pbase));
      if (c < 0) {  // walked by the direct kernel; it has no delta entries
        row++;
        continue;
      }
      if (!p_done) {
        if (lane == n) {
          my_row = (int)row;
          my_e = kProtoTag | (uint32_t)c;
        }
        n++;
        p_done = true;
        continue;
      }
      const int re = ptr_of(row + 1);
      if (e < re) {
        if (e >= wbase + 32) {  // advance the window, prefetch the next one
          wbase += 32;
          win_e = win_n;
          win_n = (wbase + 32 + lane < n_delta) ? __ldg(a.delta_idx + wbase + 32 + lane) : 0u;
        }
        const int take = min(min(SLOTS - n, re - e), wbase + 32 - e);
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
        p_done = false;
      }
    }
    const bool mine = lane < n;
    const bool is_p = (my_e & kProtoTag) != 0u;
    const uint32_t my_bytes = mine ? (is_p ? p_bytes : b_bytes) : 0u;
    const uint32_t total = __reduce_add_sync(kFull, my_bytes);
    if (mine) meta[s * SLOTS + lane] = make_int2(my_row, (int)my_e);
    if (lane == 0) {
      cnt[s] = n;
      if (n > 0) ptx::mbar_arrive_expect_tx(&bars[s], total);
    }
    __syncwarp();
    if (mine) {
      const void* src = is_p ? static_cast<const void*>(Pn + (int64_t)(my_e & kIndexMask) * a.ldp)
                             : static_cast<const void*>(Bn + (int64_t)(my_e & kIndexMask) * a.ldb);
      ptx::bulk_g2s(buf + (size_t)(s * SLOTS + lane) * kSlotBytes, src, my_bytes, &bars[s]);
    }
  };

  float acc[VPL][COLS];
  int acc_row = -1;
  auto store = [&]() {
    float* crow = a.C + (int64_t)acc_row * a.ldc + n0;
#pragma unroll
    for (int v = 0; v < VPL; v++) {
      if (!cvalid[v]) continue;
#pragma unroll
      for (int j = 0; j < COLS; j += 4)
        *reinterpret_cast<float4*>(crow + col[v] + j) =
            make_float4(acc[v][j], acc[v][j + 1], acc[v][j + 2], acc[v][j + 3]);
    }
  };

  uint32_t phases = 0;
#pragma unroll
  for (int s = 0; s < S; s++) fill(s);
  int s = 0;
  while (true) {
    __syncwarp();
    const int n = cnt[s];
    if (n == 0) break;
    if (!ptx::mbar_wait(&bars[s], (phases >> s) & 1u)) {
      if (lane == 0) atomicCAS(&g_bulk_error, 0, 1);
      for (int t = 0; t < S; t++)
        if (t != s && cnt[t] > 0) ptx::mbar_wait(&bars[t], (phases >> t) & 1u);
      return;
    }
    phases ^= 1u << s;
    for (int j = 0; j < n; j++) {
      const int2 m = meta[s * SLOTS + j];
      const uint32_t ent = (uint32_t)m.y;
      const uint8_t* slot = buf + (size_t)(s * SLOTS + j) * kSlotBytes;
      if (ent & kProtoTag) {
        if (acc_row >= 0) store();
        acc_row = m.x;
#pragma unroll
        for (int v = 0; v < VPL; v++) {
          if (!cvalid[v]) continue;
#pragma unroll
          for (int q = 0; q < COLS; q += 4) {
            const float4 p = *reinterpret_cast<const float4*>(slot + (size_t)(col[v] + q) * 4);
            acc[v][q] = p.x; acc[v][q + 1] = p.y; acc[v][q + 2] = p.z; acc[v][q + 3] = p.w;
          }
        }
      } else {
        const bool neg = (ent & kSubtract) != 0u;
#pragma unroll
        for (int v = 0; v < VPL; v++) {
          if (!cvalid[v]) continue;
          const typename V::Raw r =
              *reinterpret_cast<const typename V::Raw*>(slot + (size_t)col[v] * sizeof(BT));
          float f[COLS];
          V::cvt(r, f);
#pragma unroll
          for (int q = 0; q < COLS; q++) acc[v][q] += neg ? -f[q] : f[q];
        }
      }
    }
    __syncwarp();
    ptx::fence_proxy_async_smem();
    fill(s);
    s = (s + 1 == S) ? 0 : s + 1;
  }
  if (acc_row >= 0) store();
}

// Prototype sums P[c] over one chunk of CW = 32·VPL·COLS columns by one CTA
// of WARPS warps: warp w walks entries [len·w/WARPS, len·(w+1)/WARPS) of the
// prototype's column list, keeping S stages of SLOTS B slices in flight as
// bulk copies (the bytes in flight cost shared memory, not registers), and
// adds them in list order; the warps' partials are added in warp order, so P
// is the same on every run.  Few warps with deep copy queues finish the sums
// in a few L2 round trips while leaving most warp slots and registers of the
// SM to the row kernel under programmatic dependent launch.  A wait that
// runs out records error 2 in g_bulk_error; the warp waits (bounded) for its
// other stages and the CTA writes nothing.
template <typename BT, int VPL, int WARPS, int S, int SLOTS>
struct SumsBulkLayout {
  static constexpr int kCW = 32 * VPL * Vec<BT>::COLS;
  static constexpr int kSlot = kCW * (int)sizeof(BT);
  static constexpr size_t kBuf = (size_t)WARPS * S * SLOTS * kSlot;
  static constexpr size_t kTotal = kBuf + (size_t)WARPS * S * sizeof(uint64_t);
};

template <typename BT, int VPL, int WARPS, int S, int SLOTS>
__global__ void __launch_bounds__(WARPS * 32, 1) k_proto_sums_bulk(SpmmArgs a) {
  using V = Vec<BT>;
  using L = SumsBulkLayout<BT, VPL, WARPS, S, SLOTS>;
  constexpr int COLS = V::COLS;
  constexpr int CW = L::kCW;
  static_assert(SLOTS <= 32, "one lane per slot");
  static_assert(CW / 4 <= WARPS * 32, "one thread per float4 of the chunk");
  static_assert(L::kTotal + WARPS * CW * 4 <= 232448, "shared memory");
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ float4 wp[WARPS][CW / 4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t* buf = smem + (size_t)warp * S * SLOTS * L::kSlot;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::kBuf) + warp * S;
  ptx::griddep_launch_dependents();

  const int n0 = (int)blockIdx.x * CW;
  const int64_t c = blockIdx.y;
  const int ncols = min(CW, (int)(a.N - n0));
  const uint32_t bytes = (uint32_t)ncols * (uint32_t)sizeof(BT);
  const BT* Bn = static_cast<const BT*>(a.B) + n0;
  const int s0 = __ldg(a.cons_ptr + c), len = __ldg(a.cons_ptr + c + 1) - s0;
  int e = s0 + (int)((int64_t)len * warp / WARPS);
  const int e_end = s0 + (int)((int64_t)len * (warp + 1) / WARPS);
  int col[VPL];
  bool cvalid[VPL];
#pragma unroll
  for (int v = 0; v < VPL; v++) {
    col[v] = (v * 32 + lane) * COLS;
    cvalid[v] = col[v] < ncols;
  }
  if (lane == 0)
    for (int s = 0; s < S; s++) ptx::mbar_init(&bars[s], 1);
  ptx::fence_mbar_init();
  __syncwarp();

  auto fill = [&](int s) -> int {
    const int n = min(SLOTS, e_end - e);
    if (n <= 0) return 0;
    if (lane == 0) ptx::mbar_arrive_expect_tx(&bars[s], (uint32_t)n * bytes);
    __syncwarp();
    if (lane < n) {
      const uint32_t k = __ldg(a.cons_idx + e + lane);
      ptx::bulk_g2s(buf + (size_t)(s * SLOTS + lane) * L::kSlot, Bn + (int64_t)k * a.ldb, bytes, &bars[s]);
    }
    e += n;
    return n;
  };

  Acc<VPL, COLS, false> acc;
  acc.zero();
  int ns[S];
#pragma unroll
  for (int s = 0; s < S; s++) ns[s] = fill(s);
  uint32_t phases = 0;
  bool ok = true;
  for (bool any = true; any && ok;) {
    any = false;
#pragma unroll
    for (int s = 0; s < S; s++) {
      const int n = ns[s];
      if (n == 0 || !ok) continue;
      any = true;
      if (!ptx::mbar_wait(&bars[s], (phases >> s) & 1u)) {
        if (lane == 0) atomicCAS(&g_bulk_error, 0, 2);
#pragma unroll
        for (int t = 0; t < S; t++)
          if (t != s && ns[t] > 0) ptx::mbar_wait(&bars[t], (phases >> t) & 1u);
        ok = false;
        continue;
      }
      phases ^= 1u << s;
      for (int j = 0; j < n; j++) {
        const uint8_t* slot = buf + (size_t)(s * SLOTS + j) * L::kSlot;
#pragma unroll
        for (int v = 0; v < VPL; v++) {
          if (!cvalid[v]) continue;
          const typename V::Raw r = *reinterpret_cast<const typename V::Raw*>(slot + (size_t)col[v] * sizeof(BT));
          float f[COLS];
          V::cvt(r, f);
#pragma unroll
          for (int q = 0; q < COLS; q++) acc.add(v, q, f[q]);
        }
      }
      __syncwarp();
      ptx::fence_proxy_async_smem();
      ns[s] = fill(s);
    }
  }
  float* w = reinterpret_cast<float*>(&wp[warp][0]);
#pragma unroll
  for (int v = 0; v < VPL; v++)
#pragma unroll
    for (int j = 0; j < COLS; j++) w[(v * 32 + lane) * COLS + j] = acc.result(v, j);
  const int good = __syncthreads_and(ok ? 1 : 0);
  if (good && threadIdx.x < CW / 4 && 4 * (int)threadIdx.x < ncols) {
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < WARPS; u++) {
      const float4 x = wp[u][threadIdx.x];
      t.x += x.x;
      t.y += x.y;
      t.z += x.z;
      t.w += x.w;
    }
    reinterpret_cast<float4*>(a.P + c * a.ldp + n0)[threadIdx.x] = t;
  }
}

template <typename BT, int VPL, int WARPS, int S, int SLOTS>
int launch_sums_bulk_t(const SpmmArgs& a, cudaStream_t st) {
  using L = SumsBulkLayout<BT, VPL, WARPS, S, SLOTS>;
  static bool configured[64] = {false};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  auto kern = k_proto_sums_bulk<BT, VPL, WARPS, S, SLOTS>;
  if (dev < 64 && !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kTotal));
    configured[dev] = true;
  }
  const int64_t chunks = ceil_div(a.N, L::kCW);
  if (chunks > 0x7fffffff || a.n_proto > 65535) return BSP_ERR_CAPACITY;
  kern<<<dim3((unsigned)chunks, (unsigned)a.n_proto), WARPS * 32, L::kTotal, st>>>(a);
  BSP_LAUNCHED();
  return BSP_OK;
}

template <typename BT, int VPL, int WARPS, int S, int SLOTS>
int launch_sums_bulk_fit(const SpmmArgs& a, cudaStream_t st) {
  using L = SumsBulkLayout<BT, VPL, WARPS, S, SLOTS>;
  if constexpr (L::kTotal + (size_t)WARPS * L::kCW * 4 <= 232448) return launch_sums_bulk_t<BT, VPL, WARPS, S, SLOTS>(a, st);
  else return BSP_ERR_UNSUPPORTED;
}

template <typename BT>
int launch_sums_bulk_v(const SpmmArgs& a, int variant, cudaStream_t st) {
  constexpr int VPL = Vec<BT>::COLS == 4 ? 2 : 1;
  switch (variant) {
    case 1: return launch_sums_bulk_fit<BT, VPL, 8, 2, 12>(a, st);
    case 2: return launch_sums_bulk_fit<BT, VPL, 12, 2, 8>(a, st);
    case 3: return launch_sums_bulk_fit<BT, VPL, 16, 2, 6>(a, st);
    case 4: return launch_sums_bulk_fit<BT, VPL, 16, 3, 4>(a, st);
    case 5: return launch_sums_bulk_fit<BT, VPL, 6, 2, 16>(a, st);
    case 6: return launch_sums_bulk_fit<BT, VPL, 8, 3, 16>(a, st);
    case 7: return launch_sums_bulk_fit<BT, VPL, 16, 2, 12>(a, st);
    case 8: return launch_sums_bulk_fit<BT, VPL, 12, 2, 16>(a, st);
    default: return launch_sums_bulk_fit<BT, VPL, 8, 3, 8>(a, st);
  }
}

template <typename BT, int WARPS, int S, int SLOTS>
int launch_bulk_t(const SpmmArgs& a, int n_delta, cudaStream_t st) {
  using L = BulkLayout<WARPS, S, SLOTS>;
  static bool configured[64] = {false};
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  auto kern = k_spmm_proto_bulk<BT, WARPS, S, SLOTS>;
  if (dev < 64 && !configured[dev]) {
    BSP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kTotal));
    configured[dev] = true;
  }
  const int64_t chunks = ceil_div(a.N, kChunkCols);
  int64_t gx = num_sms() / chunks;
  if (gx < 1) gx = 1;
  if (gx > a.M) gx = a.M;
  if (chunks > 65535) return BSP_ERR_CAPACITY;
  kern<<<dim3((unsigned)gx, (unsigned)chunks), WARPS * 32, L::kTotal, st>>>(a, n_delta);
  BSP_LAUNCHED();
  return BSP_OK;
}

template <typename BT>
int launch_bulk_variant(const SpmmArgs& a, int n_delta, int variant, cudaStream_t st) {
  switch (variant) {
    case 1: return launch_bulk_t<BT, 6, 2, 8>(a, n_delta, st);
    case 2: return launch_bulk_t<BT, 4, 3, 9>(a, n_delta, st);
    case 3: return launch_bulk_t<BT, 8, 2, 6>(a, n_delta, st);
    case 4: return launch_bulk_t<BT, 6, 4, 4>(a, n_delta, st);
    case 5: return launch_bulk_t<BT, 16, 2, 3>(a, n_delta, st);
    case 6: return launch_bulk_t<BT, 12, 2, 4>(a, n_delta, st);
    case 7: return launch_bulk_t<BT, 10, 2, 5>(a, n_delta, st);
    default: return launch_bulk_t<BT, 6, 3, 6>(a, n_delta, st);
  }
}

}  // namespace

int launch_spmm_proto_bulk(const SpmmArgs& a, int variant, cudaStream_t s) {
  if (a.M == 0 || a.N == 0) return BSP_OK;
  const int n_delta = (int)a.n_delta;
  switch (a.bdt) {
    case BSP_F32: return launch_bulk_variant<float>(a, n_delta, variant, s);
    case BSP_BF16: return launch_bulk_variant<__nv_bfloat16>(a, n_delta, variant, s);
    case BSP_F16: return launch_bulk_variant<__half>(a, n_delta, variant, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

int launch_proto_sums_bulk(const SpmmArgs& a, int variant, cudaStream_t s) {
  if (a.n_proto == 0 || a.N == 0) return BSP_OK;
  switch (a.bdt) {
    case BSP_F32: return launch_sums_bulk_v<float>(a, variant, s);
    case BSP_BF16: return launch_sums_bulk_v<__nv_bfloat16>(a, variant, s);
    case BSP_F16: return launch_sums_bulk_v<__half>(a, variant, s);
    default: return BSP_ERR_UNSUPPORTED;
  }
}

int bulk_device_error(int* out, bool clear) {
  BSP_CUDA(cudaMemcpyFromSymbol(out, g_bulk_error, sizeof(int)));
  if (clear) {
    const int zero = 0;
    BSP_CUDA(cudaMemcpyToSymbol(g_bulk_error, &zero, sizeof(int)));
  }
  return BSP_OK;
}

}  // namespace bsp
