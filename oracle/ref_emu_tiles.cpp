/*
 * ref_emu_tiles.cpp — runs the reference's COO -> 8x8 bitmap-tile
 * conversion on the CPU and exports it with a C ABI for the oracle-pinning
 * tests.  TEST INFRASTRUCTURE ONLY.
 *
 * The code is not in this repository: build_ref.py extracts from the
 * reference checkout into oracle/_ref/*.inc
 *   coo2bmp_noTuple_d   source/src/main.cu:692-779
 *   find_tile_index     source/src/mm.h:83-104
 *   absolute2relative   source/src/mm.h:106-121
 *   bmp_popcount_d      source/src/mm.h:134-144
 * The reference runs them through Thrust on the GPU; here the same Thrust
 * calls run on Thrust's sequential C++ back end (the CUDA toolkit's own
 * Thrust headers, THRUST_DEVICE_SYSTEM_CPP), so the sorts, reductions and
 * scans are Thrust's own algorithms and the functors are the reference's.
 *
 * Two stand-ins make the 2019-era code compile against the toolkit's
 * Thrust, neither of which changes what it computes:
 *  - cusp::coo_matrix (the vendored cusp does not build against CUDA 13's
 *    Thrust): a struct with the members the function uses — num_rows,
 *    num_cols, num_entries, row_indices, column_indices, values, resize().
 *  - the functors take thrust::tuple<...&> and call its member get<N>(),
 *    which the old Thrust tuple had and CUDA 13's does not: inside the
 *    functors' namespace, thrust::tuple names a tuple of references derived
 *    from the toolkit's tuple that adds that member.
 * thrust::cuda::par, the reference's execution policy, names the
 * sequential policy here.
 */
#define THRUST_DEVICE_SYSTEM THRUST_DEVICE_SYSTEM_CPP
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/for_each.h>
#include <thrust/functional.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/transform.h>
#include <thrust/tuple.h>

#include <stdint.h>
#include <string.h>

namespace thrust {
namespace cuda {
static const auto par = thrust::cpp::par;
}
}  // namespace thrust

namespace cusp {
struct device_memory {};
struct host_memory {};
template <typename I, typename V, typename Mem>
struct coo_matrix {
  size_t num_rows = 0, num_cols = 0, num_entries = 0;
  thrust::device_vector<I> row_indices, column_indices;
  thrust::device_vector<V> values;
  coo_matrix() = default;
  coo_matrix(const coo_matrix&) = default;
  void resize(size_t r, size_t c, size_t n) {
    num_rows = r;
    num_cols = c;
    num_entries = n;
    row_indices.resize(n);
    column_indices.resize(n);
    values.resize(n);
  }
};
}  // namespace cusp

namespace refmm {
namespace thrust {
template <typename... T>
struct tuple : ::cuda::std::tuple<T...> {
  tuple(const ::cuda::std::tuple<T...>& t) : ::cuda::std::tuple<T...>(t) {}
  template <size_t I>
  auto& get() { return ::cuda::std::get<I>(*this); }
};
}  // namespace thrust
#define __host__
#define __device__
#define BMP_DIM 8U
static inline uint32_t __popcll(uint64_t x) { return (uint32_t)__builtin_popcountll(x); }
#include "ref_find_tile_index.inc"
#include "ref_absolute2relative.inc"
#include "ref_bmp_popcount_d.inc"
}  // namespace refmm

using refmm::find_tile_index;
using refmm::absolute2relative;
using refmm::bmp_popcount_d;
#include "ref_coo2bmp.inc"
#undef __host__
#undef __device__

extern "C" {

/* coo2bmp_noTuple_d<float> on an M×K COO matrix given in any entry order.
 * Outputs (capacity n_cap >= nnz): tiles bmp [n], tile rows and columns
 * [n], popcount offsets idx [n] (the exclusive scan, no total), values
 * regrouped by tile elems [nnz].  Returns n, or -1 when n_cap is short.  */
int64_t ref_coo2bmp(const int* row, const int* col, const float* val, int64_t nnz, int M,
                    int K, int64_t n_cap, uint64_t* bmp, int* tile_row, int* tile_col,
                    uint32_t* idx, float* elems) {
  cusp::coo_matrix<int, float, cusp::device_memory> in;
  in.resize(M, K, nnz);
  ::thrust::copy(row, row + nnz, in.row_indices.begin());
  ::thrust::copy(col, col + nnz, in.column_indices.begin());
  ::thrust::copy(val, val + nnz, in.values.begin());
  cusp::coo_matrix<int, uint64_t, cusp::device_memory> out;
  ::thrust::device_vector<float> el;
  ::thrust::device_vector<uint32_t> ix;
  coo2bmp_noTuple_d<float>(in, out, el, ix);
  int64_t n = (int64_t)out.num_entries;
  if (n > n_cap) return -1;
  ::thrust::copy(out.values.begin(), out.values.end(), bmp);
  ::thrust::copy(out.row_indices.begin(), out.row_indices.end(), tile_row);
  ::thrust::copy(out.column_indices.begin(), out.column_indices.end(), tile_col);
  ::thrust::copy(ix.begin(), ix.end(), idx);
  ::thrust::copy(el.begin(), el.end(), elems);
  return n;
}

}  // extern "C"
