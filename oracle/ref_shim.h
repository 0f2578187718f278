/*
 * ref_shim.h — host emulation of the CUDA built-ins that a handful of the
 * reference's kernels use, so that those kernels (compiled from the
 * reference's own source by build_ref.py into oracle/_ref/) run on the CPU
 * and pin the oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * Execution model: one block at a time; inside a block every CUDA thread is
 * a ucontext fiber.  Fibers run one after another in ascending threadIdx.x
 * order, each until it reaches __syncthreads() or returns; the block resumes
 * after every fiber has arrived.  Atomics are therefore plain read-modify-
 * write operations and every race of the original kernel is resolved in
 * ascending thread order — the canonical serialisation the oracle restates.
 *
 * `__shared__` arrays become function-local statics aligned to 4 KiB, each
 * in a slot of its own, so that the out-of-bounds shared-memory writes of
 * generate_groups_large (row_group[MAX_GROUP_NUM] at source/src/main.cu:131
 * and group_ele_row_idx[MAX_GROUP_NUM][i] at :188 on its spill path) land in
 * padding instead of another array.
 */
#ifndef BSP_REF_SHIM_H_
#define BSP_REF_SHIM_H_

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

struct emu_fiber {
  ucontext_t ctx;
  dim3 tid;
  int done;
};

struct emu_state {
  dim3 bidx, bdim, gdim;
  emu_fiber* cur;
  ucontext_t sched;
};

extern emu_state g_emu;

#define threadIdx (g_emu.cur->tid)
#define blockIdx (g_emu.bidx)
#define blockDim (g_emu.bdim)
#define gridDim (g_emu.gdim)

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static __attribute__((aligned(4096)))

static inline void __syncthreads() { swapcontext(&g_emu.cur->ctx, &g_emu.sched); }
static inline void __threadfence() {}

static inline int atomicOr(int* a, int v) { int o = *a; *a = o | v; return o; }
static inline unsigned atomicOr(unsigned* a, unsigned v) { unsigned o = *a; *a = o | v; return o; }
static inline int atomicCAS(int* a, int cmp, int v) { int o = *a; if (o == cmp) *a = v; return o; }
static inline int atomicAdd(int* a, int v) { int o = *a; *a = o + v; return o; }
static inline float atomicAdd(float* a, float v) { float o = *a; *a = o + v; return o; }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }

/* Runs `body(arg)` as a grid of grid.x*grid.y blocks of block.x threads,
 * blocks in order (y outer, x inner), fibers as described above. */
typedef void (*emu_body_fn)(void* arg);
int emu_launch(dim3 grid, dim3 block, emu_body_fn body, void* arg);

#endif
