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
//  4. consensus: the rows are listed by cluster, and a CTA per cluster
//     counts each column's bits (bit-sliced counters) and keeps the majority;
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
#include <algorithm>
#include <climits>
#include <mutex>
#include <cstdlib>
#include <new>
#include <vector>

#include "bsp_internal.cuh"
#include "plan.cuh"
#include "spmm.cuh"

namespace bsp {
namespace {

constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kMaxHashes = 8;

__host__ __device__ __forceinline__ uint32_t mix32(uint32_t k, uint32_t j, uint32_t seed) {
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

// Warp per row: H MinHash values and the popcount.
//
// With `perm` (perm[j*K + t] = the column with the t-th smallest mix(., j);
// mix is a bijection of the column for fixed j, so the order is strict), the
// minimum over the row's columns of mix(k, j) is mix of the first column in
// that order that the row holds: lanes test 32 positions of the order at a
// time against the row's words and a ballot finds the first hit.  A row of
// density d needs about 1/d probes per function instead of hashing every
// set bit H times.  Rows sparser than 1/64, and functions without a hit in
// kPermRounds rounds, take the direct path: the row's words 32 at a time
// (one per lane), their set bits dealt out evenly — lane l takes bits l,
// l+32, ... of the group in column order, its source word found by a binary
// search over the lanes' inclusive bit counts — and hashed.  Both give the
// same minimum.
// Then lane 0 inserts the row's band key into the bucket table (open
// addressing: atomicCAS insert, atomicAdd size, atomicMin leader = lowest
// row) and records the row's slot (-1: empty row or no key).
constexpr int kPermRounds = 8;
__global__ void __launch_bounds__(256) k_signatures(const uint32_t* __restrict__ words, int64_t M,
                                                    int Kw, int64_t K, int H, uint32_t seed,
                                                    const uint32_t* __restrict__ perm,
                                                    uint32_t* __restrict__ sig,
                                                    int32_t* __restrict__ nnz, uint32_t* keys,
                                                    int32_t* count, int32_t* leader, uint32_t tmask,
                                                    int32_t* __restrict__ row_slot) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= M) return;
  uint32_t mn[kMaxHashes];
#pragma unroll
  for (int j = 0; j < kMaxHashes; j++) mn[j] = kEmpty;
  const uint32_t* r = words + row * Kw;
  int cnt = 0;
  for (int w = lane; w < Kw; w += 32) cnt += __popc(__ldg(r + w));
  cnt = (int)__reduce_add_sync(kFull, (unsigned)cnt);
  uint32_t miss = (1u << H) - 1u;  // functions still to compute directly
  if (perm && (int64_t)cnt * 64 >= K) {
#pragma unroll
    for (int j = 0; j < kMaxHashes; j++) {
      if (j >= H) break;
      const uint32_t* pj = perm + (int64_t)j * K;
      for (int rd = 0; rd < kPermRounds; rd++) {
        const int64_t t = (int64_t)rd * 32 + lane;
        uint32_t k = 0u;
        bool hit = false;
        if (t < K) {
          k = __ldg(pj + t);
          hit = (__ldg(r + (k >> 5)) >> (k & 31)) & 1u;
        }
        const uint32_t b = __ballot_sync(kFull, hit);
        if (b) {
          mn[j] = mix32(__shfl_sync(kFull, k, __ffs(b) - 1), (uint32_t)j, seed);
          miss &= ~(1u << j);
          break;
        }
        if ((int64_t)(rd + 1) * 32 >= K) break;
      }
    }
  }
  if (miss) {
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
          if ((miss >> j) & 1u) mn[j] = min(mn[j], mix32(k, (uint32_t)j, seed));
      }
    }
  }
  }
#pragma unroll
  for (int j = 0; j < kMaxHashes; j++) {
    mn[j] = j < H ? __reduce_min_sync(kFull, mn[j]) : kEmpty;
    if (j < H && lane == j) sig[row * H + j] = mn[j];
  }
  if (lane == 0) {
    nnz[row] = cnt;
    const uint32_t key = band_key(mn, H);
    int32_t found = -1;
    if (cnt > 0 && key != kEmpty) {
      uint32_t sl = slot_of(key, tmask);
      for (uint32_t probe = 0; probe <= tmask; probe++) {
        const uint32_t prev = atomicCAS(keys + sl, kEmpty, key);
        if (prev == kEmpty || prev == key) {
          atomicAdd(count + sl, 1);
          atomicMin(leader + sl, (int32_t)row);
          found = (int32_t)sl;
          break;
        }
        sl = (sl + 1) & tmask;
      }
    }
    row_slot[row] = found;
  }
}


__device__ __forceinline__ int leader_flag(const int32_t* __restrict__ row_slot, const int32_t* __restrict__ count,
                                           const int32_t* __restrict__ leader, int64_t row, int min_rows) {
  const int32_t s = row_slot[row];
  return (s >= 0 && count[s] >= min_rows && leader[s] == (int32_t)row) ? 1 : 0;
}

// Up to kLeaderScanMax rows, in one CTA (tiles in row order): the leader
// flags and their exclusive scan (cluster numbers, total in cid[M]), and the
// exclusive scan of the cluster sizes at leader rows (where each cluster's
// rows start in the by-cluster row list, total in coff[M]).
constexpr int kLeaderScanThreads = 1024;
constexpr int64_t kLeaderScanMax = 32768;
__global__ void __launch_bounds__(kLeaderScanThreads) k_leader_scan(const int32_t* __restrict__ row_slot,
                                                                    const int32_t* __restrict__ count,
                                                                    const int32_t* __restrict__ leader, int64_t M,
                                                                    int min_rows, int32_t* __restrict__ cid,
                                                                    int32_t* __restrict__ coff) {
  __shared__ int sw[32];
  constexpr int ITEMS = 4, TILE = kLeaderScanThreads * ITEMS;
  int carry = 0, carry_sz = 0;
  for (int64_t base = 0; base < M; base += TILE) {
    int v[ITEMS], z[ITEMS];
    int sum = 0, sum_sz = 0;
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
      const int64_t i = base + (int64_t)threadIdx.x * ITEMS + j;
      v[j] = i < M ? leader_flag(row_slot, count, leader, i, min_rows) : 0;
      z[j] = v[j] ? count[row_slot[i]] : 0;
      sum += v[j];
      sum_sz += z[j];
    }
    int total, total_sz;
    int run = block_exclusive_scan(sum, sw, &total) + carry;
    int run_sz = block_exclusive_scan(sum_sz, sw, &total_sz) + carry_sz;
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
      const int64_t i = base + (int64_t)threadIdx.x * ITEMS + j;
      if (i < M) {
        cid[i] = run;
        coff[i] = run_sz;
      }
      run += v[j];
      run_sz += z[j];
    }
    carry += total;
    carry_sz += total_sz;
  }
  if (threadIdx.x == 0) {
    cid[M] = carry;
    coff[M] = carry_sz;
  }
}

__global__ void k_leader_sizes(const int32_t* __restrict__ row_slot, const int32_t* __restrict__ count,
                               const int32_t* __restrict__ leader, int64_t M, int min_rows,
                               int32_t* __restrict__ size) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= M) return;
  size[row] = leader_flag(row_slot, count, leader, row, min_rows) ? count[row_slot[row]] : 0;
}

__global__ void k_leader_flags(const int32_t* __restrict__ row_slot, const int32_t* __restrict__ count,
                               const int32_t* __restrict__ leader, int64_t M, int min_rows,
                               int32_t* __restrict__ flag) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= M) return;
  flag[row] = leader_flag(row_slot, count, leader, row, min_rows);
}

// Thread per row: the row's cluster (its bucket's number, if the bucket
// became a cluster) and its place in the by-cluster row list (the order
// within a cluster follows atomicAdd and does not matter: the list is only
// counted); the leader row records the cluster's size and list start.
__global__ void k_cluster_rows(const int32_t* __restrict__ row_slot, const int32_t* __restrict__ count,
                               const int32_t* __restrict__ leader, const int32_t* __restrict__ cid_of_row,
                               const int32_t* __restrict__ coff_of_row, int64_t M, int min_rows,
                               int32_t* __restrict__ cluster, int32_t* __restrict__ csize,
                               int32_t* __restrict__ cstart, int32_t* cursor, int32_t* __restrict__ rows) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= M) return;
  const int32_t sl = row_slot[row];
  int32_t c = -1;
  if (sl >= 0 && count[sl] >= min_rows) {
    const int32_t L = leader[sl];
    c = cid_of_row[L];
    const int32_t base = coff_of_row[L];
    rows[base + atomicAdd(cursor + c, 1)] = (int32_t)row;
    if (L == (int32_t)row) {
      csize[c] = count[sl];
      cstart[c] = base;
    }
  }
  cluster[row] = c;
}

__device__ __forceinline__ uint32_t pair_key(uint32_t a, uint32_t b) {
  if (a == kEmpty || b == kEmpty) return kEmpty;
  uint32_t k = (a * 0x9e3779b1u) ^ (b + 0x7f4a7c15u + (a << 6) + (a >> 2));
  k ^= k >> 16;
  k *= 0x85ebca6bu;
  k ^= k >> 13;
  return k == kEmpty ? kEmpty - 1 : k;
}

// Block per cluster: the consensus words (majority of the cluster's rows per
// column), their popcount (stats[4]) and MinHash values (as k_signatures
// computes them for a row), and the consensus's pair bands (h_2j, h_2j+1)
// inserted into tables j = 0..H/2-1 (key → lowest cluster id).  For each
// block of 256 words, thread (g, w) counts word w's bits over rows g, g+4,
// ... of the cluster with bit-sliced counters (plane p holds bit p of the 32
// columns' counts; adding a row's word is a ripple carry over the planes),
// turns them into per-column counts and adds those into shared memory; then
// the group-0 thread of word w keeps the columns with 2·count > size.
constexpr int kConsWords = 256;
constexpr int kConsGroups = 4;
constexpr int kConsThreads = kConsWords * kConsGroups;
constexpr int kConsRowChunk = 1024;  // row indices staged in shared memory at a time
constexpr int kConsInFlight = 8;     // word loads in flight per thread
constexpr int kConsPlanes = 9;       // a group counts ≤ kConsRowChunk / kConsGroups = 256 rows per chunk
__global__ void __launch_bounds__(kConsThreads) k_consensus(const uint32_t* __restrict__ words, int Kw,
                                                            const int32_t* __restrict__ rows,
                                                            const int32_t* __restrict__ cstart,
                                                            const int32_t* __restrict__ csize,
                                                            int H, uint32_t seed, uint32_t* __restrict__ cons,
                                                            uint32_t* akeys, int32_t* avals, uint32_t tmask,
                                                            unsigned long long* stats, int32_t* cons_cnt) {
  static_assert(kConsRowChunk / kConsGroups < (1 << kConsPlanes), "planes");
  __shared__ uint32_t wmin[kMaxHashes][kConsThreads / 32];
  __shared__ unsigned wpop[kConsThreads / 32];
  __shared__ int32_t srow[kConsRowChunk];
  __shared__ int32_t colcnt[32 * kConsWords];  // [bit][word]
  const int64_t c = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int g = threadIdx.x / kConsWords, wl = threadIdx.x % kConsWords;
  const int32_t sz = csize[c];
  const int32_t* crow = rows + cstart[c];
  uint32_t mn[kMaxHashes];
#pragma unroll
  for (int j = 0; j < kMaxHashes; j++) mn[j] = kEmpty;
  unsigned pop = 0;
  for (int wb = 0; wb < Kw; wb += kConsWords) {  // uniform: every thread runs the same blocks and chunks
    const int w = wb + wl;
    const bool wv = w < Kw;
    for (int i = threadIdx.x; i < 32 * kConsWords; i += kConsThreads) colcnt[i] = 0;
    for (int r0 = 0; r0 < sz; r0 += kConsRowChunk) {
      const int nr = min(kConsRowChunk, sz - r0);
      __syncthreads();
      for (int i = threadIdx.x; i < nr; i += kConsThreads) srow[i] = crow[r0 + i];
      __syncthreads();
      uint32_t plane[kConsPlanes];
#pragma unroll
      for (int p = 0; p < kConsPlanes; p++) plane[p] = 0u;
      for (int i0 = g; i0 < nr; i0 += kConsGroups * kConsInFlight) {
        uint32_t xs[kConsInFlight];
#pragma unroll
        for (int u = 0; u < kConsInFlight; u++) {
          const int i = i0 + u * kConsGroups;
          xs[u] = (wv && i < nr) ? __ldg(words + (int64_t)srow[i] * Kw + w) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kConsInFlight; u++) {
          uint32_t x = xs[u];
#pragma unroll
          for (int p = 0; p < kConsPlanes; p++) {
            const uint32_t carry = plane[p] & x;
            plane[p] ^= x;
            x = carry;
            if (!x) break;
          }
        }
      }
      if (wv) {
#pragma unroll 4
        for (int b = 0; b < 32; b++) {
          int cnt = 0;
#pragma unroll
          for (int p = 0; p < kConsPlanes; p++) cnt |= (int)((plane[p] >> b) & 1u) << p;
          if (cnt) atomicAdd(&colcnt[b * kConsWords + wl], cnt);
        }
      }
    }
    __syncthreads();
    if (g == 0 && wv) {
      uint32_t m = 0u;
      for (int b = 0; b < 32; b++)
        if (2 * colcnt[b * kConsWords + wl] > sz) m |= 1u << b;
      cons[c * Kw + w] = m;
      pop += __popc(m);
      while (m) {
        const int b = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t k = (uint32_t)(w * 32 + b);
#pragma unroll
        for (int j = 0; j < kMaxHashes; j++)
          if (j < H) mn[j] = min(mn[j], mix32(k, (uint32_t)j, seed));
      }
    }
    __syncthreads();  // colcnt is cleared for the next block of words
  }
#pragma unroll
  for (int j = 0; j < kMaxHashes; j++) {
    const uint32_t v = __reduce_min_sync(kFull, mn[j]);
    if (lane == 0) wmin[j][wid] = v;
  }
  pop = __reduce_add_sync(kFull, pop);
  if (lane == 0) wpop[wid] = pop;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long total = 0;
    for (int i = 0; i < kConsThreads / 32; i++) total += wpop[i];
    cons_cnt[c] = (int32_t)total;
    if (total) {
      atomicAdd(stats + 4, total);
      atomicMax(stats + 7, total);
    }
  }
  const int j = threadIdx.x;
  if (j < H / 2) {
    uint32_t a = kEmpty, b = kEmpty;
    for (int i = 0; i < kConsThreads / 32; i++) {
      a = min(a, wmin[2 * j][i]);
      b = min(b, wmin[2 * j + 1][i]);
    }
    const uint32_t key = pair_key(a, b);
    if (key == kEmpty) return;
    uint32_t* Kt = akeys + (int64_t)j * (tmask + 1);
    int32_t* Vt = avals + (int64_t)j * (tmask + 1);
    uint32_t sl = slot_of(key, tmask);
    for (uint32_t probe = 0; probe <= tmask; probe++) {
      const uint32_t prev = atomicCAS(Kt + sl, kEmpty, key);
      if (prev == kEmpty || prev == key) {
        atomicMin(Vt + sl, (int32_t)c);
        return;
      }
      sl = (sl + 1) & tmask;
    }
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
constexpr int kOrderBuckets = 256;  // row-slot order: clustered rows counted by min(delta count, 255)

__global__ void __launch_bounds__(256) k_finalize_rows(
    const uint32_t* __restrict__ words, int64_t M, int Kw, int H, const uint32_t* __restrict__ sig,
    const int32_t* __restrict__ nnz, const uint32_t* __restrict__ cons, int64_t n_clusters,
    const uint32_t* __restrict__ akeys, const int32_t* __restrict__ avals, uint32_t amask,
    int32_t* __restrict__ cluster, int32_t* __restrict__ delta_cnt,
    unsigned long long* __restrict__ stats, int32_t* __restrict__ order_hist) {
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
    if (c >= 0) {
      atomicAdd(stats + 1, (unsigned long long)d);                // delta entries
      atomicAdd(order_hist + (d < kOrderBuckets - 1 ? d : kOrderBuckets - 1), 1);
    } else {
      atomicAdd(stats + 2, 1ull);                                 // direct rows
      atomicAdd(stats + 3, (unsigned long long)n);                // direct nnz
    }
  }
}


// ---- row slots: clustered rows by descending delta count -----------------
// The SpMM's warps take clustered rows in slot order, and the GPU starts CTAs
// in index order, so the longest lists start first and the last CTAs to
// start carry the shortest ones (a shorter tail).  A counting sort on
// b = min(count, 255): k_finalize_rows counts the rows of each b, and
// k_delta_fill's blocks each scan those 256 counts (descending b) before
// every clustered row takes the next position of its b.  Rows with equal b
// land in any order: the plan's layout depends on it, the SpMM's results do
// not (each row's sum is formed the same way wherever it sits).  A row's
// slot holds the row, its cluster, its delta count, the list's start and the
// first 28 entries, so the SpMM reads a row's whole description with one
// load whose address depends on the position alone.

// Warp per prototype: its set columns in ascending order into
// cons_idx[cons_ptr[c] ..] (the list the prototype-sum kernel walks).
__global__ void __launch_bounds__(256) k_cons_fill(const uint32_t* __restrict__ cons, int64_t n_proto, int Kw,
                                                   const int32_t* __restrict__ cons_ptr, uint32_t* __restrict__ idx) {
  const int lane = threadIdx.x & 31;
  const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (c >= n_proto) return;
  const uint32_t* p = cons + c * Kw;
  int base = cons_ptr[c];
  for (int w0 = 0; w0 < Kw; w0 += 32) {
    const int w = w0 + lane;
    uint32_t x = w < Kw ? p[w] : 0u;
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
      idx[pos++] = (uint32_t)(w * 32 + b);
    }
    base += __shfl_sync(kFull, incl, 31);
  }
}

// Warp per clustered row: delta entries in ascending column order, and with
// `pad` the row's slot (position from the bucket counts `hist`, the next
// free one of its bucket by `cursor`).
__global__ void __launch_bounds__(256) k_delta_fill(const uint32_t* __restrict__ words, int64_t M,
                                                    int Kw, const uint32_t* __restrict__ cons,
                                                    const int32_t* __restrict__ cluster,
                                                    const int32_t* __restrict__ dptr,
                                                    uint32_t* __restrict__ didx, const int32_t* __restrict__ hist,
                                                    int32_t* __restrict__ cursor, uint32_t* __restrict__ pad) {
  __shared__ int bucket_base[kOrderBuckets];
  __shared__ int wsum[8];
  const int lane = threadIdx.x & 31;
  if (pad) {  // bucket_base[b] = clustered rows with a larger bucket (scan over t = 255 - b)
    const int h = hist[kOrderBuckets - 1 - threadIdx.x];
    int v = h;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(kFull, v, o);
      if (lane >= o) v += u;
    }
    if (lane == 31) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    for (int u = 0; u < (int)(threadIdx.x >> 5); u++) v += wsum[u];
    bucket_base[kOrderBuckets - 1 - threadIdx.x] = v - h;
    __syncthreads();
  }
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= M) return;
  const int c = cluster[row];
  if (c < 0) return;
  const uint32_t* r = words + row * Kw;
  const uint32_t* p = cons + (int64_t)c * Kw;
  const int s0 = dptr[row];
  uint32_t* slot = nullptr;
  if (pad) {
    const int n = dptr[row + 1] - s0;
    const int b = n < kOrderBuckets - 1 ? n : kOrderBuckets - 1;
    int at = 0;
    if (lane == 0) at = bucket_base[b] + atomicAdd(&cursor[b], 1);
    slot = pad + (int64_t)__shfl_sync(kFull, at, 0) * 32;
    if (lane < 4) slot[lane] = lane == 0 ? (uint32_t)row : lane == 1 ? (uint32_t)c : lane == 2 ? (uint32_t)n : (uint32_t)s0;
    else if (lane - 4 >= n) slot[lane] = 0u;
  }
  int base = s0;
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
      const uint32_t e = (uint32_t)(w * 32 + b) | (((q >> b) & 1u) ? 0x80000000u : 0u);
      didx[pos] = e;
      if (slot && pos - s0 < 28) slot[4 + pos - s0] = e;
      pos++;
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

// Column orders of the MinHash functions (perm of k_signatures) per device
// and (K, H, seed): sorted on the host at first use, kept until exit (at most
// 16 orders, K ≤ kPermMaxK; otherwise the signatures are computed directly).
constexpr int64_t kPermMaxK = (int64_t)1 << 18;
const uint32_t* minhash_order(int64_t K, int H, uint32_t seed) {
  struct Entry {
    int dev;
    int64_t K;
    int H;
    uint32_t seed;
    uint32_t* d;
  };
  static std::mutex mu;
  static std::vector<Entry> cache;
  if (K < 1 || K > kPermMaxK || H < 1 || H > kMaxHashes) return nullptr;
  const char* e = getenv("BSP_MINHASH_DIRECT");  // comparisons: hash every set bit
  if (e && e[0] == '1') return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  for (const Entry& e : cache)
    if (e.dev == dev && e.K == K && e.H == H && e.seed == seed) return e.d;
  if (cache.size() >= 16) return nullptr;
  std::vector<uint64_t> key((size_t)K);
  std::vector<uint32_t> host((size_t)H * (size_t)K);
  for (int j = 0; j < H; j++) {
    for (int64_t k = 0; k < K; k++) key[k] = ((uint64_t)mix32((uint32_t)k, (uint32_t)j, seed) << 32) | (uint64_t)k;
    std::sort(key.begin(), key.end());
    for (int64_t t = 0; t < K; t++) host[(size_t)j * K + t] = (uint32_t)key[t];
  }
  uint32_t* d = nullptr;
  const size_t bytes = host.size() * sizeof(uint32_t);
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  cache.push_back(Entry{dev, K, H, seed, d});
  return d;
}

// Timing-free events for plan builds, reused across builds (per device).
std::mutex g_event_mu;
std::vector<cudaEvent_t> g_events[64];
int event_acquire(cudaEvent_t* e) {
  int dev = 0;
  BSP_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lk(g_event_mu);
    if (!g_events[dev].empty()) {
      *e = g_events[dev].back();
      g_events[dev].pop_back();
      return BSP_OK;
    }
  }
  BSP_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  return BSP_OK;
}
void event_release(cudaEvent_t e) {
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lk(g_event_mu);
    if (g_events[dev].size() < 64) {
      g_events[dev].push_back(e);
      return;
    }
  }
  cudaEventDestroy(e);
}

// Up to four arrays of 32-bit words filled with a value each, in one launch.
struct Fill {
  uint32_t* p;
  int64_t n;
  uint32_t v;
};
__global__ void k_fill4(Fill a, Fill b, Fill c, Fill d) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;; i += stride) {
    bool any = false;
    if (i < a.n) { a.p[i] = a.v; any = true; }
    if (i < b.n) { b.p[i] = b.v; any = true; }
    if (i < c.n) { c.p[i] = c.v; any = true; }
    if (i < d.n) { d.p[i] = d.v; any = true; }
    if (!any) break;
  }
}
int launch_fill4(Fill a, Fill b, Fill c, Fill d, cudaStream_t s) {
  const int64_t n = std::max(std::max(a.n, b.n), std::max(c.n, d.n));
  if (n <= 0) return BSP_OK;
  const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), (int64_t)num_sms() * 8);
  k_fill4<<<(unsigned)blocks, 256, 0, s>>>(a, b, c, d);
  BSP_LAUNCHED();
  return BSP_OK;
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
    BSP_TRY(event_acquire(&fork));
    BSP_TRY(event_acquire(&done));
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
    if (fork) event_release(fork);
    if (done) event_release(done);
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
  const size_t o_coff = take(sizeof(int32_t) * (M + 1));
  const size_t o_scan = take(scan_workspace_bytes(M + 1));
  // stats[8], then the row-slot order's bucket counts and cursors
  const size_t o_stats = take(sizeof(unsigned long long) * 8 + sizeof(int32_t) * 2 * kOrderBuckets);
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
  int32_t* coff = (int32_t*)(T + o_coff);
  void* scanws = T + o_scan;
  unsigned long long* stats = (unsigned long long*)(T + o_stats);
  int32_t* order_hist = (int32_t*)(stats + 8);
  int32_t* dcnt = (int32_t*)(T + o_dcnt);

  BSP_TRY(launch_fill4(Fill{keys, tsize, kEmpty}, Fill{(uint32_t*)cnt, tsize, 0u},
                       Fill{(uint32_t*)lead, tsize, 0x7f7f7f7fu}, Fill{(uint32_t*)stats, 16 + 2 * kOrderBuckets, 0u}, s));

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
  k_signatures<<<wgrid, 256, 0, s>>>(words, M, Kw, K, H, prm->seed, minhash_order(K, H, prm->seed), sig, nnz, keys,
                                     cnt, lead, tsize - 1, slot);
  if (M <= kLeaderScanMax) {
    k_leader_scan<<<1, kLeaderScanThreads, 0, s>>>(slot, cnt, lead, M, min_rows, cid, coff);
  } else {
    k_leader_flags<<<tgrid, 256, 0, s>>>(slot, cnt, lead, M, min_rows, flag);
    BSP_LAUNCHED();
    BSP_TRY(launch_scan_i32(flag, M, cid, scanws, s));
    k_leader_sizes<<<tgrid, 256, 0, s>>>(slot, cnt, lead, M, min_rows, flag);
    BSP_LAUNCHED();
    BSP_TRY(launch_scan_i32(flag, M, coff, scanws, s));
  }
  BSP_LAUNCHED();
  int32_t n_clusters = 0;
  BSP_CUDA(cudaMemcpyAsync(&n_clusters, cid + M, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  BSP_CUDA(cudaStreamSynchronize(s));

  const bool can_cluster = n_clusters > 0 && prm->mode != BSP_PLAN_DIRECT;
  const int64_t ncl = can_cluster ? n_clusters : 0;

  // ---- plan storage (cluster map, delta pointers, consensus) -------------
  size_t poff = 0;
  auto ptake = [&](size_t bytes) { const size_t o = poff; poff += al256(bytes); return o; };
  const size_t p_cl = ptake(sizeof(int32_t) * M);
  const size_t p_dp = ptake(sizeof(int32_t) * (M + 1));
  const size_t p_cons = ptake(sizeof(uint32_t) * ncl * Kw);
  const size_t p_cptr = ptake(sizeof(int32_t) * (ncl + 1));
  const size_t p_dl = ptake(sizeof(int32_t) * M);
  void* parena = nullptr;
  BSP_CUDA(plan_alloc(&parena, poff ? poff : 16, s, &plan->arena_pooled));
  plan->arena = parena;
  char* Pa = static_cast<char*>(parena);
  plan->row_cluster = (int32_t*)(Pa + p_cl);
  plan->delta_ptr = (int32_t*)(Pa + p_dp);
  plan->cons = (uint32_t*)(Pa + p_cons);
  plan->cons_ptr = (int32_t*)(Pa + p_cptr);
  plan->direct_list = (int32_t*)(Pa + p_dl);
  plan->n_proto = ncl;

  if (ncl > 0) {
    const uint32_t asize = pow2_at_least(2 * ncl);
    size_t off2 = 0;
    auto take2 = [&](size_t bytes) { const size_t o = off2; off2 += al256(bytes); return o; };
    const size_t q_csize = take2(sizeof(int32_t) * ncl);
    const size_t q_cstart = take2(sizeof(int32_t) * ncl);
    const size_t q_cursor = take2(sizeof(int32_t) * ncl);
    const size_t q_ccnt = take2(sizeof(int32_t) * ncl);
    const size_t q_rows = take2(sizeof(int32_t) * M);
    const size_t q_akeys = take2(sizeof(uint32_t) * asize * H);
    const size_t q_avals = take2(sizeof(int32_t) * asize * H);
    DevBuf t2;
    BSP_TRY(t2.alloc(off2, s));
    char* T2 = static_cast<char*>(t2.p);
    int32_t* csize = (int32_t*)(T2 + q_csize);
    int32_t* cstart = (int32_t*)(T2 + q_cstart);
    int32_t* cursor = (int32_t*)(T2 + q_cursor);
    int32_t* ccnt = (int32_t*)(T2 + q_ccnt);
    int32_t* crows = (int32_t*)(T2 + q_rows);
    uint32_t* akeys = (uint32_t*)(T2 + q_akeys);
    int32_t* avals = (int32_t*)(T2 + q_avals);
    BSP_TRY(launch_fill4(Fill{(uint32_t*)cursor, ncl, 0u}, Fill{akeys, (int64_t)asize * H, kEmpty},
                         Fill{(uint32_t*)avals, (int64_t)asize * H, 0x7f7f7f7fu}, Fill{nullptr, 0, 0u}, s));
    k_cluster_rows<<<tgrid, 256, 0, s>>>(slot, cnt, lead, cid, coff, M, min_rows, plan->row_cluster, csize, cstart,
                                         cursor, crows);
    k_consensus<<<(unsigned)ncl, kConsThreads, 0, s>>>(words, Kw, crows, cstart, csize, H, prm->seed, plan->cons,
                                                      akeys, avals, asize - 1, stats, ccnt);
    BSP_LAUNCHED();
    BSP_TRY(launch_scan_i32(ccnt, ncl, plan->cons_ptr, scanws, s));
    k_finalize_rows<<<wgrid, 256, 0, s>>>(words, M, Kw, H, sig, nnz, plan->cons, ncl, akeys, avals,
                                          asize - 1, plan->row_cluster, dcnt, stats, order_hist);
    BSP_LAUNCHED();
  } else {
    BSP_CUDA(cudaMemsetAsync(plan->row_cluster, 0xff, sizeof(int32_t) * M, s));
    BSP_CUDA(cudaMemsetAsync(dcnt, 0, sizeof(int32_t) * M, s));
    k_finalize_rows<<<wgrid, 256, 0, s>>>(words, M, Kw, H, sig, nnz, plan->cons, 0, nullptr,
                                          nullptr, 0, plan->row_cluster, dcnt, stats, order_hist);
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
  plan->proto_max_nnz = (int64_t)st[7];
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
  // the prototypes' column lists (int32 offsets: kept only below 2^31 entries)
  const int64_t n_list = plan->proto_nnz < INT_MAX ? plan->proto_nnz : 0;
  // a 128-byte slot per clustered row (up to 1 GiB of slots)
  const int64_t n_slot = M - plan->direct_rows;
  const int64_t n_pad = n_slot > 0 && n_slot * 128 <= ((int64_t)1 << 30) ? n_slot * 32 : 0;
  if (mode == BSP_PLAN_PROTO && plan->delta_nnz + n_list > 0) {
    // one block: the row slots, the delta lists, then the prototypes' column lists
    BSP_CUDA(plan_alloc(&plan->delta_arena, sizeof(uint32_t) * (n_pad + plan->delta_nnz + n_list), s,
                        &plan->delta_pooled));
    plan->delta_pad = n_pad > 0 ? (uint32_t*)plan->delta_arena : nullptr;
    plan->delta_idx = (uint32_t*)plan->delta_arena + n_pad;
    plan->cons_idx = n_list > 0 ? plan->delta_idx + plan->delta_nnz : nullptr;
    if (plan->delta_nnz > 0 || n_pad > 0)
      k_delta_fill<<<wgrid, 256, 0, s>>>(words, M, Kw, plan->cons, plan->row_cluster, plan->delta_ptr,
                                         plan->delta_idx, order_hist, order_hist + kOrderBuckets,
                                         plan->delta_pad);
    plan->n_slot = n_pad > 0 ? n_slot : 0;
    if (n_list > 0)
      k_cons_fill<<<(unsigned)ceil_div(ncl, 8), 256, 0, s>>>(plan->cons, ncl, Kw, plan->cons_ptr, plan->cons_idx);
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
