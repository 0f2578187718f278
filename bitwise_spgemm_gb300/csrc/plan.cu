// plan.cu — similarity row grouping that schedules the SpMM.
//
// Rows of A that are near-copies of one another (the clustered workload: 64
// prototype masks, every row a prototype with ~0.2 % of its bits flipped)
// share most of their set bits.  The plan finds such clusters and stores, per
// clustered row, only the bits where it differs from its cluster's majority
// mask ("consensus"), so the SpMM adds ~16 rows of B per row instead of ~420.
//
// Steps (all on the GPU, on the caller's stream; the host reads back the
// cluster count and the plan's counters to size buffers):
//  1. signatures: H MinHash values per row — h_j(row) = min over the row's
//     set columns k of mix(k, j) — plus the row's popcount (warp per row,
//     __popc + warp min-reduction);
//  2. bucketing: rows with equal band key (h_0, h_1, h_2) meet in an
//     open-addressing hash table (atomicCAS insert, atomicAdd size,
//     atomicMin leader = lowest row).  Two unrelated rows share one MinHash
//     value with probability equal to their Jaccard similarity (≈2.5 % for
//     two random 5 %-dense masks), so a single-hash key would merge clusters;
//     the three-value band makes that ≈J³;
//  3. buckets with ≥ min_cluster_rows rows become clusters, numbered by an
//     exclusive scan over "row is a bucket leader" flags (stable: ascending
//     leader row), so numbering is deterministic;
//  4. consensus: per-cluster per-column counts (atomicAdd), majority bit;
//  5. every row also looks up, for each pair band (h_2b, h_2b+1), the
//     cluster whose consensus has the same pair, and keeps the nearest
//     candidate (Hamming distance, ties → lower cluster id) — this rescues
//     rows whose band key in step 2 was disturbed by their own flips;
//  6. every row keeps its cluster only if |row XOR consensus| < popcount(row);
//     delta lists (ascending column, bit 31 = column present in the consensus
//     but not in the row → subtract) are laid out by an exclusive scan.
// Every step is order-independent or ordered by row index, so the plan is a
// deterministic function of A.  The tensor-core structures (occupancy bitmaps,
// A's words by column) depend on A alone and are built on a side stream
// meanwhile.
#include <climits>
#include <mutex>
#include <cstdlib>
#include <new>

#include "bsp_internal.cuh"
#include "plan.cuh"
#include "spmm.cuh"

namespace bsp {
namespace {

constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kMaxHashes = 8;

__device__ __forceinline__ uint32_t mix32(uint32_t k, uint32_t j, uint32_t seed) {
  // murmur3 finaliser of a per-function offset key
  uint32_t h = k * 0x9e3779b1u + (j + 1u) * 0x85ebca77u + seed;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

constexpr int kBand = 3;  // MinHash values in the bucket key

__device__ __forceinline__ uint32_t band_key(const uint32_t* __restrict__ sig, int H) {
  uint32_t k = 0x811c9dc5u;
  for (int j = 0; j < kBand && j < H; j++) {
    if (sig[j] == kEmpty) return kEmpty;
    k = (k ^ sig[j]) * 0x01000193u;
    k ^= k >> 15;
  }
  return k == kEmpty ? kEmpty - 1 : k;
}

__device__ __forceinline__ uint32_t slot_of(uint32_t key, uint32_t mask) {
  return (key * 0x9e3779b1u) & mask;
}

// Position of the n-th (0-based) set bit of x; n < popcount(x).
__device__ __forceinline__ int nth_set_bit(uint32_t x, int n) {
  int pos = 0;
#pragma unroll
  for (int width = 16; width; width >>= 1) {
    const uint32_t low = x & ((1u << width) - 1u);
    const int c = __popc(low);
    if (n >= c) {
      n -= c;
      x >>= width;
      pos += width;
    } else {
      x = low;
    }
  }
  return pos;
}

// Warp per row: H MinHash values and the popcount.  The row's words are taken
// 32 at a time (one per lane) and their set bits are dealt out evenly: lane l
// takes bits l, l+32, ... of the group in column order (its source word found
// by a binary search over the lanes' inclusive bit counts), so every lane
// hashes about the same number of columns however the bits fall.
__global__ void __launch_bounds__(256) k_signatures(const uint32_t* __restrict__ words, int64_t M,
                                                    int Kw, int H, uint32_t seed,
                                                    uint32_t* __restrict__ sig,
                                                    int32_t* __restrict__ nnz) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= M) return;
  uint32_t mn[kMaxHashes];
#pragma unroll
  for (int j = 0; j < kMaxHashes; j++) mn[j] = kEmpty;
  int cnt = 0;
  const uint32_t* r = words + row * Kw;
  for (int g = 0; g < Kw; g += 32) {
    const uint32_t x = (g + lane < Kw) ? __ldg(r + g + lane) : 0u;
    const int c = __popc(x);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int excl = incl - c;
    const int total = __shfl_sync(kFull, incl, 31);
    cnt += total;
    for (int b0 = 0; b0 < total; b0 += 32) {
      const int gi = b0 + lane;  // this lane's bit of the group, in column order
      int src = 0;               // lanes whose words end before bit gi
#pragma unroll
      for (int step = 16; step; step >>= 1) {
        const int v = __shfl_sync(kFull, incl, src + step - 1);
        if (v <= gi) src += step;
      }
      const uint32_t wx = __shfl_sync(kFull, x, src);
      const int ex = __shfl_sync(kFull, excl, src);
      if (gi < total) {
        const uint32_t k = (uint32_t)((g + src) * 32 + nth_set_bit(wx, gi - ex));
#pragma unroll
        for (int j = 0; j < kMaxHashes; j++)
          if (j < H) mn[j] = min(mn[j], mix32(k, (uint32_t)j, seed));
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kMaxHashes; j++) {
    if (j >= H) break;
    const uint32_t m = __reduce_min_sync(kFull, mn[j]);
    if (lane == j) sig[row * H + j] = m;
  }
  if (lane == 0) nnz[row] = cnt;
}

// Thread per row: insert the row's band key into the bucket table.
__global__ void k_bucket_insert(const uint32_t* __restrict__ sig, const int32_t* __restrict__ nnz,
                                int64_t M, int H, uint32_t* keys, int32_t* count, int32_t* leader,
                                uint32_t tmask, int32_t* __restrict__ row_slot) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= M) return;
  const uint32_t key = band_key(sig + row * H, H);
  int32_t found = -1;
  if (nnz[row] > 0 && key != kEmpty) {
    uint32_t s = slot_of(key, tmask);
    for (uint32_t probe = 0; probe <= tmask; probe++) {
      const uint32_t prev = atomicCAS(keys + s, kEmpty, key);
      if (prev == kEmpty || prev == key) {
        atomicAdd(count + s, 1);
        atomicMin(leader + s, (int32_t)row);
        found = (int32_t)s;
        break;
      }
      s = (s + 1) & tmask;
    }
  }
  row_slot[row] = found;
}

__global__ void k_leader_flags(const int32_t* __restrict__ row_slot, const int32_t* __restrict__ count,
                               const int32_t* __restrict__ leader, int64_t M, int min_rows,
                               int32_t* __restrict__ flag) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= M) return;
  const int32_t s = row_slot[row];
  flag[row] = (s >= 0 && count[s] >= min_rows && leader[s] == (int32_t)row) ? 1 : 0;
}

__global__ void k_assign(const int32_t* __restrict__ row_slot, const int32_t* __restrict__ count,
                         const int32_t* __restrict__ leader, const int32_t* __restrict__ cid_of_row,
                         int64_t M, int min_rows, int32_t* __restrict__ cluster,
                         int32_t* __restrict__ csize) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= M) return;
  const int32_t s = row_slot[row];
  int32_t c = -1;
  if (s >= 0 && count[s] >= min_rows) {
    c = cid_of_row[leader[s]];
    if (leader[s] == (int32_t)row) csize[c] = count[s];
  }
  cluster[row] = c;
}

// Thread per (row, word) of clustered rows: per-column bit counts.
__global__ void k_count_bits(const uint32_t* __restrict__ words, int64_t M, int Kw, int64_t K,
                             const int32_t* __restrict__ cluster, int32_t* __restrict__ counts) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= M * Kw) return;
  const int64_t row = t / Kw;
  const int w = (int)(t - row * Kw);
  const int32_t c = cluster[row];
  if (c < 0) return;
  uint32_t x = words[t];
  while (x) {
    const int b = __ffs(x) - 1;
    x &= x - 1;
    atomicAdd(counts + (int64_t)c * K + w * 32 + b, 1);
  }
}

// Thread per (cluster, word): majority vote.
__global__ void k_majority(const int32_t* __restrict__ counts, const int32_t* __restrict__ csize,
                           int64_t n_clusters, int Kw, int64_t K, uint32_t* __restrict__ cons) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n_clusters * Kw) return;
  const int64_t c = t / Kw;
  const int w = (int)(t - c * Kw);
  const int32_t sz = csize[c];
  uint32_t m = 0;
  for (int b = 0; b < 32; b++) {
    const int64_t k = (int64_t)w * 32 + b;
    if (k < K && 2 * counts[c * K + k] > sz) m |= 1u << b;
  }
  cons[t] = m;
}

__device__ __forceinline__ uint32_t pair_key(uint32_t a, uint32_t b) {
  if (a == kEmpty || b == kEmpty) return kEmpty;
  uint32_t k = (a * 0x9e3779b1u) ^ (b + 0x7f4a7c15u + (a << 6) + (a >> 2));
  k ^= k >> 16;
  k *= 0x85ebca6bu;
  k ^= k >> 13;
  return k == kEmpty ? kEmpty - 1 : k;
}

// Tables j = 0..H/2-1: pair band (h_2j, h_2j+1) of consensus c → lowest c.
__global__ void k_alt_insert(const uint32_t* __restrict__ csig, int64_t n_clusters, int H,
                             uint32_t* keys, int32_t* vals, uint32_t tmask) {
  const int NB = H / 2;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n_clusters * NB) return;
  const int64_t c = t / NB;
  const int j = (int)(t - c * NB);
  const uint32_t key = pair_key(csig[c * H + 2 * j], csig[c * H + 2 * j + 1]);
  if (key == kEmpty) return;
  uint32_t* K = keys + (int64_t)j * (tmask + 1);
  int32_t* V = vals + (int64_t)j * (tmask + 1);
  uint32_t s = slot_of(key, tmask);
  for (uint32_t probe = 0; probe <= tmask; probe++) {
    const uint32_t prev = atomicCAS(K + s, kEmpty, key);
    if (prev == kEmpty || prev == key) {
      atomicMin(V + s, (int32_t)c);
      return;
    }
    s = (s + 1) & tmask;
  }
}

__device__ int alt_lookup(const uint32_t* __restrict__ keys, const int32_t* __restrict__ vals,
                          uint32_t tmask, uint32_t key) {
  uint32_t s = slot_of(key, tmask);
  for (uint32_t probe = 0; probe <= tmask; probe++) {
    const uint32_t k = keys[s];
    if (k == key) return vals[s];
    if (k == kEmpty) return -1;
    s = (s + 1) & tmask;
  }
  return -1;
}

__device__ __forceinline__ int xor_popcount(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                                            int Kw, int lane) {
  int d = 0;
  for (int w = lane; w < Kw; w += 32) d += __popc(__ldg(a + w) ^ __ldg(b + w));
  return (int)__reduce_add_sync(kFull, (unsigned)d);
}

// Warp per row: the row's bucket cluster and the clusters sharing one of its
// pair bands compete on Hamming distance; the row keeps the winner only if
// the delta is smaller than its popcount.
__global__ void __launch_bounds__(256) k_finalize_rows(
    const uint32_t* __restrict__ words, int64_t M, int Kw, int H, const uint32_t* __restrict__ sig,
    const int32_t* __restrict__ nnz, const uint32_t* __restrict__ cons, int64_t n_clusters,
    const uint32_t* __restrict__ akeys, const int32_t* __restrict__ avals, uint32_t amask,
    int32_t* __restrict__ cluster, int32_t* __restrict__ delta_cnt,
    unsigned long long* __restrict__ stats) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= M) return;
  const uint32_t* r = words + row * Kw;
  const int n = nnz[row];
  int c = cluster[row];
  int d = INT_MAX;
  if (c >= 0) d = xor_popcount(r, cons + (int64_t)c * Kw, Kw, lane);
  if (n > 0 && n_clusters > 0) {
    for (int j = 0; j < H / 2; j++) {
      const uint32_t key = pair_key(sig[row * H + 2 * j], sig[row * H + 2 * j + 1]);
      if (key == kEmpty) continue;
      const int cand = alt_lookup(akeys + (int64_t)j * (amask + 1),
                                  avals + (int64_t)j * (amask + 1), amask, key);
      if (cand < 0 || cand == c) continue;
      const int dc = xor_popcount(r, cons + (int64_t)cand * Kw, Kw, lane);
      if (dc < d || (dc == d && cand < c)) {
        d = dc;
        c = cand;
      }
    }
  }
  if (c >= 0 && d >= n) c = -1;
  if (lane == 0) {
    cluster[row] = c;
    delta_cnt[row] = c >= 0 ? d : 0;
    atomicAdd(stats + 0, (unsigned long long)n);                  // nnz
    if (c >= 0) atomicAdd(stats + 1, (unsigned long long)d);      // delta entries
    else {
      atomicAdd(stats + 2, 1ull);                                 // direct rows
      atomicAdd(stats + 3, (unsigned long long)n);                // direct nnz
    }
  }
}

__global__ void k_cons_popc(const uint32_t* __restrict__ cons, int64_t n, unsigned long long* stats) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int c = t < n ? __popc(cons[t]) : 0;
  const unsigned s = __reduce_add_sync(kFull, (unsigned)c);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(stats + 4, (unsigned long long)s);
}

// Warp per clustered row: delta entries in ascending column order.
__global__ void __launch_bounds__(256) k_delta_fill(const uint32_t* __restrict__ words, int64_t M,
                                                    int Kw, const uint32_t* __restrict__ cons,
                                                    const int32_t* __restrict__ cluster,
                                                    const int32_t* __restrict__ dptr,
                                                    uint32_t* __restrict__ didx) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= M) return;
  const int c = cluster[row];
  if (c < 0) return;
  const uint32_t* r = words + row * Kw;
  const uint32_t* p = cons + (int64_t)c * Kw;
  int base = dptr[row];
  for (int w0 = 0; w0 < Kw; w0 += 32) {
    const int w = w0 + lane;
    const uint32_t a = w < Kw ? r[w] : 0u;
    const uint32_t q = w < Kw ? p[w] : 0u;
    uint32_t x = a ^ q;
    const int cnt = __popc(x);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    int pos = base + incl - cnt;
    while (x) {
      const int b = __ffs(x) - 1;
      x &= x - 1;
      didx[pos++] = (uint32_t)(w * 32 + b) | (((q >> b) & 1u) ? 0x80000000u : 0u);
    }
    base += __shfl_sync(kFull, incl, 31);
  }
}

__global__ void k_direct_flags(const int32_t* __restrict__ cluster, int64_t M, int32_t* __restrict__ flag) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < M) flag[r] = cluster[r] < 0 ? 1 : 0;
}

__global__ void k_direct_scatter(const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                                 int64_t M, int32_t* __restrict__ list) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < M && flag[r]) list[pos[r]] = (int32_t)r;
}

uint32_t pow2_at_least(int64_t n) {
  uint32_t p = 1024;
  while ((int64_t)p < n && p < 0x80000000u) p <<= 1;
  return p;
}

// Plan-build temporaries come from a library-owned, stream-ordered memory
// pool per device that keeps its memory between builds (release threshold
// = unlimited): no device-wide synchronisation on free, no remapping on the
// next build.  Held until the process exits; bounded by the largest build.
cudaMemPool_t temp_pool() {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[dev] = pool;
  }
  return pools[dev];
}

struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  bool pooled = false;
  ~DevBuf() {
    if (!p) return;
    if (pooled) cudaFreeAsync(p, s);
    else cudaFree(p);
  }
  int alloc(size_t bytes, cudaStream_t st) {
    s = st;
    cudaMemPool_t pool = temp_pool();
    cudaError_t e;
    if (pool) {
      e = cudaMallocFromPoolAsync(&p, bytes ? bytes : 16, pool, st);
      pooled = e == cudaSuccess;
    } else {
      e = cudaMalloc(&p, bytes ? bytes : 16);
    }
    if (e != cudaSuccess) {
      p = nullptr;
      cuda_status(e);
      return BSP_ERR_ALLOC;
    }
    return BSP_OK;
  }
};

inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// The plan's own storage, from the same pool (the plan is synchronised with
// its stream before it is returned, so any stream may use it afterwards).
// *pooled tells the destroy calls whether the block goes back with
// cudaFree (waits for the device) or may go back in stream order.
cudaError_t plan_alloc(void** p, size_t bytes, cudaStream_t s, bool* pooled) {
  cudaMemPool_t pool = temp_pool();
  *pooled = pool && cudaMallocFromPoolAsync(p, bytes, pool, s) == cudaSuccess;
  if (*pooled) return cudaSuccess;
  return cudaMalloc(p, bytes);
}

// A non-blocking stream per device for plan-build work that the grouping does
// not wait on (the tensor-core structures); created once, kept until exit.
cudaStream_t side_stream() {
  static std::mutex mu;
  static cudaStream_t streams[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!streams[dev] && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess)
    streams[dev] = nullptr;
  return streams[dev];
}

// Work forked from stream `s` onto the side stream: join() makes `s` wait for
// it; the destructor joins too (and frees the events), so temporaries that
// are freed on `s` afterwards outlive the side work on every return path.
struct SideFork {
  cudaStream_t s = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  bool joined = true;
  int start(cudaStream_t main) {
    s = main;
    side = side_stream();
    if (!side) return BSP_OK;  // no side stream: the work runs on `s`
    BSP_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    BSP_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    BSP_CUDA(cudaEventRecord(fork, s));
    BSP_CUDA(cudaStreamWaitEvent(side, fork, 0));
    joined = false;
    return BSP_OK;
  }
  cudaStream_t stream() const { return side ? side : s; }
  int join() {
    if (joined) return BSP_OK;
    joined = true;
    BSP_CUDA(cudaEventRecord(done, side));
    BSP_CUDA(cudaStreamWaitEvent(s, done, 0));
    return BSP_OK;
  }
  ~SideFork() {
    join();
    if (fork) cudaEventDestroy(fork);
    if (done) cudaEventDestroy(done);
  }
};

}  // namespace

int plan_build(const uint32_t* words, int64_t M, int64_t K, const bsp_plan_params* prm,
               bsp_plan* plan, cudaStream_t s) {
  const int Kw = (int)ceil_div(K, 32);
  const int H = prm->signature_hashes;
  const int min_rows = prm->min_cluster_rows;
  plan->M = M;
  plan->K = K;
  plan->Kw = Kw;

  // ---- temporaries -------------------------------------------------------
  const uint32_t tsize = pow2_at_least(2 * M);
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off += al256(bytes); return o; };
  const size_t o_sig = take(sizeof(uint32_t) * M * H);
  const size_t o_nnz = take(sizeof(int32_t) * M);
  const size_t o_keys = take(sizeof(uint32_t) * tsize);
  const size_t o_cnt = take(sizeof(int32_t) * tsize);
  const size_t o_lead = take(sizeof(int32_t) * tsize);
  const size_t o_slot = take(sizeof(int32_t) * M);
  const size_t o_flag = take(sizeof(int32_t) * M);
  const size_t o_cid = take(sizeof(int32_t) * (M + 1));
  const size_t o_scan = take(scan_workspace_bytes(M + 1));
  const size_t o_stats = take(sizeof(unsigned long long) * 8);
  const size_t o_dcnt = take(sizeof(int32_t) * M);
  DevBuf tmp;
  BSP_TRY(tmp.alloc(off, s));
  char* T = static_cast<char*>(tmp.p);
  uint32_t* sig = (uint32_t*)(T + o_sig);
  int32_t* nnz = (int32_t*)(T + o_nnz);
  uint32_t* keys = (uint32_t*)(T + o_keys);
  int32_t* cnt = (int32_t*)(T + o_cnt);
  int32_t* lead = (int32_t*)(T + o_lead);
  int32_t* slot = (int32_t*)(T + o_slot);
  int32_t* flag = (int32_t*)(T + o_flag);
  int32_t* cid = (int32_t*)(T + o_cid);
  void* scanws = T + o_scan;
  unsigned long long* stats = (unsigned long long*)(T + o_stats);
  int32_t* dcnt = (int32_t*)(T + o_dcnt);

  BSP_CUDA(cudaMemsetAsync(keys, 0xff, sizeof(uint32_t) * tsize, s));
  BSP_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * tsize, s));
  BSP_CUDA(cudaMemsetAsync(lead, 0x7f, sizeof(int32_t) * tsize, s));
  BSP_CUDA(cudaMemsetAsync(stats, 0, sizeof(unsigned long long) * 8, s));

  // ---- tensor-core structures: occupancy bitmaps and A's words by column
  // (the producers then load the words of 32 consecutive rows or columns as
  // one 128-byte run).  They depend on A only, so they are built on a side
  // stream while the grouping below runs; their tile counts land in stats[5],
  // stats[6] before the stats are read.
  size_t qoff = 0;
  auto qtake = [&](size_t bytes) { const size_t o = qoff; qoff += al256(bytes); return o; };
  const size_t p_occ = qtake(sizeof(uint32_t) * ceil_div(M, 128) * tc_occupancy_words(K));
  const size_t p_occT = qtake(sizeof(uint32_t) * ceil_div(K, 128) * tc_occupancy_t_words(M));
  const bool with_wt = (double)M * (double)Kw * 4.0 <= (double)(1ull << 32) && ceil_div(M, 32) <= 65535;
  const size_t p_wt = qtake(with_wt ? sizeof(uint32_t) * (size_t)Kw * (size_t)M : 0);
  BSP_CUDA(plan_alloc(&plan->tc_arena, qoff, s, &plan->tc_pooled));
  char* Qa = static_cast<char*>(plan->tc_arena);
  plan->occ = (uint32_t*)(Qa + p_occ);
  plan->occT = (uint32_t*)(Qa + p_occT);
  plan->wordsT = with_wt ? (uint32_t*)(Qa + p_wt) : nullptr;
  SideFork tc;
  BSP_TRY(tc.start(s));
  BSP_TRY(launch_occupancy(words, M, K, plan->occ, plan->occT, stats + 5, stats + 6, tc.stream()));
  if (with_wt) BSP_TRY(launch_transpose_words(words, M, Kw, plan->wordsT, tc.stream()));

  const unsigned wgrid = (unsigned)ceil_div(M, 8);    // warp-per-row kernels, 256 threads
  const unsigned tgrid = (unsigned)ceil_div(M, 256);  // thread-per-row kernels
  k_signatures<<<wgrid, 256, 0, s>>>(words, M, Kw, H, prm->seed, sig, nnz);
  k_bucket_insert<<<tgrid, 256, 0, s>>>(sig, nnz, M, H, keys, cnt, lead, tsize - 1, slot);
  k_leader_flags<<<tgrid, 256, 0, s>>>(slot, cnt, lead, M, min_rows, flag);
  BSP_LAUNCHED();
  BSP_TRY(launch_scan_i32(flag, M, cid, scanws, s));
  int32_t n_clusters = 0;
  BSP_CUDA(cudaMemcpyAsync(&n_clusters, cid + M, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  BSP_CUDA(cudaStreamSynchronize(s));

  // Per-column counts need n_clusters*K ints; beyond 1 GiB the plan stays direct.
  const bool can_cluster = n_clusters > 0 &&
                           (double)n_clusters * (double)K * 4.0 <= (double)(1ull << 30) &&
                           prm->mode != BSP_PLAN_DIRECT;
  const int64_t ncl = can_cluster ? n_clusters : 0;

  // ---- plan storage (cluster map, delta pointers, consensus) -------------
  size_t poff = 0;
  auto ptake = [&](size_t bytes) { const size_t o = poff; poff += al256(bytes); return o; };
  const size_t p_cl = ptake(sizeof(int32_t) * M);
  const size_t p_dp = ptake(sizeof(int32_t) * (M + 1));
  const size_t p_cons = ptake(sizeof(uint32_t) * ncl * Kw);
  const size_t p_dl = ptake(sizeof(int32_t) * M);
  void* parena = nullptr;
  BSP_CUDA(plan_alloc(&parena, poff ? poff : 16, s, &plan->arena_pooled));
  plan->arena = parena;
  char* Pa = static_cast<char*>(parena);
  plan->row_cluster = (int32_t*)(Pa + p_cl);
  plan->delta_ptr = (int32_t*)(Pa + p_dp);
  plan->cons = (uint32_t*)(Pa + p_cons);
  plan->direct_list = (int32_t*)(Pa + p_dl);
  plan->n_proto = ncl;

  if (ncl > 0) {
    const uint32_t asize = pow2_at_least(2 * ncl);
    size_t off2 = 0;
    auto take2 = [&](size_t bytes) { const size_t o = off2; off2 += al256(bytes); return o; };
    const size_t q_counts = take2(sizeof(int32_t) * ncl * K);
    const size_t q_csize = take2(sizeof(int32_t) * ncl);
    const size_t q_csig = take2(sizeof(uint32_t) * ncl * H);
    const size_t q_cnnz = take2(sizeof(int32_t) * ncl);
    const size_t q_akeys = take2(sizeof(uint32_t) * asize * H);
    const size_t q_avals = take2(sizeof(int32_t) * asize * H);
    DevBuf t2;
    BSP_TRY(t2.alloc(off2, s));
    char* T2 = static_cast<char*>(t2.p);
    int32_t* counts = (int32_t*)(T2 + q_counts);
    int32_t* csize = (int32_t*)(T2 + q_csize);
    uint32_t* csig = (uint32_t*)(T2 + q_csig);
    int32_t* cnnz = (int32_t*)(T2 + q_cnnz);
    uint32_t* akeys = (uint32_t*)(T2 + q_akeys);
    int32_t* avals = (int32_t*)(T2 + q_avals);
    BSP_CUDA(cudaMemsetAsync(counts, 0, sizeof(int32_t) * ncl * K, s));
    BSP_CUDA(cudaMemsetAsync(akeys, 0xff, sizeof(uint32_t) * asize * H, s));
    BSP_CUDA(cudaMemsetAsync(avals, 0x7f, sizeof(int32_t) * asize * H, s));
    k_assign<<<tgrid, 256, 0, s>>>(slot, cnt, lead, cid, M, min_rows, plan->row_cluster, csize);
    k_count_bits<<<(unsigned)ceil_div(M * Kw, 256), 256, 0, s>>>(words, M, Kw, K, plan->row_cluster,
                                                                 counts);
    k_majority<<<(unsigned)ceil_div(ncl * Kw, 256), 256, 0, s>>>(counts, csize, ncl, Kw, K,
                                                                 plan->cons);
    k_signatures<<<(unsigned)ceil_div(ncl, 8), 256, 0, s>>>(plan->cons, ncl, Kw, H, prm->seed,
                                                            csig, cnnz);
    if (H >= 2)
      k_alt_insert<<<(unsigned)ceil_div(ncl * (H / 2), 256), 256, 0, s>>>(csig, ncl, H, akeys,
                                                                        avals, asize - 1);
    k_finalize_rows<<<wgrid, 256, 0, s>>>(words, M, Kw, H, sig, nnz, plan->cons, ncl, akeys, avals,
                                          asize - 1, plan->row_cluster, dcnt, stats);
    k_cons_popc<<<(unsigned)ceil_div(ncl * Kw, 256), 256, 0, s>>>(plan->cons, ncl * Kw, stats);
    BSP_LAUNCHED();
  } else {
    BSP_CUDA(cudaMemsetAsync(plan->row_cluster, 0xff, sizeof(int32_t) * M, s));
    BSP_CUDA(cudaMemsetAsync(dcnt, 0, sizeof(int32_t) * M, s));
    k_finalize_rows<<<wgrid, 256, 0, s>>>(words, M, Kw, H, sig, nnz, plan->cons, 0, nullptr,
                                          nullptr, 0, plan->row_cluster, dcnt, stats);
    BSP_LAUNCHED();
  }
  BSP_TRY(launch_scan_i32(dcnt, M, plan->delta_ptr, scanws, s));
  unsigned long long st[8];
  BSP_TRY(tc.join());
  BSP_CUDA(cudaMemcpyAsync(st, stats, sizeof(st), cudaMemcpyDeviceToHost, s));
  BSP_CUDA(cudaStreamSynchronize(s));
  plan->nnz = (int64_t)st[0];
  plan->delta_nnz = (int64_t)st[1];
  plan->direct_rows = (int64_t)st[2];
  plan->direct_nnz = (int64_t)st[3];
  plan->proto_nnz = (int64_t)st[4];
  plan->occ_tiles = (int64_t)st[5];
  plan->occT_tiles = (int64_t)st[6];
  if (plan->delta_nnz >= INT_MAX) return BSP_ERR_CAPACITY;

  // Cost model in gathered rows of B: direct = nnz; proto = prototype bits +
  // delta entries + direct rows' bits + one prototype-row read per row.
  const double direct_cost = (double)plan->nnz;
  const double proto_cost = (double)plan->proto_nnz + (double)plan->delta_nnz +
                            (double)plan->direct_nnz + (double)(M - plan->direct_rows);
  int mode = prm->mode;
  if (mode == BSP_PLAN_AUTO) mode = (ncl > 0 && proto_cost < 0.6 * direct_cost) ? BSP_PLAN_PROTO : BSP_PLAN_DIRECT;
  if (ncl == 0) mode = BSP_PLAN_DIRECT;
  plan->mode = mode;
  if (mode == BSP_PLAN_PROTO && plan->direct_rows > 0) {
    k_direct_flags<<<tgrid, 256, 0, s>>>(plan->row_cluster, M, flag);
    BSP_TRY(launch_scan_i32(flag, M, cid, scanws, s));
    k_direct_scatter<<<tgrid, 256, 0, s>>>(flag, cid, M, plan->direct_list);
    BSP_LAUNCHED();
  }
  if (mode == BSP_PLAN_PROTO && plan->delta_nnz > 0) {
    BSP_CUDA(plan_alloc(&plan->delta_arena, sizeof(uint32_t) * plan->delta_nnz, s, &plan->delta_pooled));
    plan->delta_idx = (uint32_t*)plan->delta_arena;
    k_delta_fill<<<wgrid, 256, 0, s>>>(words, M, Kw, plan->cons, plan->row_cluster,
                                       plan->delta_ptr, plan->delta_idx);
    BSP_LAUNCHED();
  }
  BSP_CUDA(cudaStreamSynchronize(s));
  return BSP_OK;
}

void plan_free(bsp_plan* plan) {
  if (plan->arena) cudaFree(plan->arena);
  if (plan->delta_arena) cudaFree(plan->delta_arena);
  if (plan->tc_arena) cudaFree(plan->tc_arena);
  plan->arena = plan->delta_arena = plan->tc_arena = nullptr;
}

int plan_free_async(bsp_plan* plan, cudaStream_t s) {
  void** blocks[3] = {&plan->arena, &plan->delta_arena, &plan->tc_arena};
  const bool pooled[3] = {plan->arena_pooled, plan->delta_pooled, plan->tc_pooled};
  int st = BSP_OK;
  for (int i = 0; i < 3; i++) {
    if (!*blocks[i]) continue;
    const cudaError_t e = pooled[i] ? cudaFreeAsync(*blocks[i], s) : cudaFree(*blocks[i]);
    if (e != cudaSuccess && st == BSP_OK) st = cuda_status(e);
    *blocks[i] = nullptr;
  }
  return st;
}

}  // namespace bsp
