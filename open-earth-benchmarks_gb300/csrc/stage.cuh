// stage.cuh -- asynchronous staging of FP32 tiles into shared memory, marched along k.
//
// The FP32 stencils are bound by HBM, not by arithmetic, and a CTA that loads its inputs with
// ordinary loads and then computes leaves the memory system idle while it computes; with one
// k-level a CTA the loads in flight per SM fall short of what hides DRAM latency.  Here a CTA
// owns a 32 x 32 (i, j) tile and a chunk of k-levels, and copies each level's input boxes into
// a ring of shared-memory buffers with cp.async (PTX cp.async.ca.shared.global, 4 bytes a
// cell: the reference layout's rows of nx + 2h floats are not 16-byte multiples, so no wider
// or tensor copy can start every row), one level or more ahead of the level it computes.
//
// The reference layout gives no alignment beyond 4 bytes, so the copies are 4-byte cp.async,
// coalesced along i.  A cell outside the box the tile's outputs need is zero-filled, not
// read (src-size 0).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "oeb_common.cuh"
#include "stencil_util.cuh"

namespace oeb {

// cp.async of one 4-byte cell; with ok == false nothing is read and the cell is zero-filled
// (the address must still be a valid one: callers pass a cell of the field's reach).
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, bool ok) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(ok ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// waits until at most N of this thread's committed groups are still in flight
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issues the copies of the W x H box of field g at level offset kofs whose first cell is
// (i0, j0) into s (row-major, W per row).  Cells outside [ib, ie) x [jb, je) are zero-filled;
// `safe` is the address of a cell every call may name (the tile origin's interior cell).
template <int W, int H>
__device__ __forceinline__ void stage_box(float* s, const float* __restrict__ g, int64_t kofs, int i0, int j0,
                                          int64_t sj, int ib, int ie, int jb, int je) {
  const int tid = threadIdx.y * kTX + threadIdx.x;
  const float* safe = g + kofs;
#pragma unroll 2
  for (int e = tid; e < W * H; e += kThreads) {
    const int b = e / W;
    const int a = e - b * W;
    const int i = i0 + a, j = j0 + b;
    const bool ok = i >= ib && i < ie && j >= jb && j < je;
    cp_async4(s + e, ok ? g + kofs + i + (int64_t)j * sj : safe, ok);
  }
}

// k-levels a CTA of a staged kernel marches: enough CTAs for about one wave of
// `ctas_per_sm` CTAs on every SM, at most 16 levels and at least 1.
int staged_kb(int tiles, int nz, int ctas_per_sm);

}  // namespace oeb
