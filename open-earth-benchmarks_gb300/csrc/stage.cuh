// stage.cuh -- asynchronous staging of FP32 tiles into shared memory, marched along k.
//
// The FP32 stencils are bound by HBM, not by arithmetic, and a CTA that loads its inputs with
// ordinary loads and then computes leaves the memory system idle while it computes; with one
// k-level a CTA the loads in flight per SM fall short of what hides DRAM latency.  Here a CTA
// owns a 32 x 32 (i, j) tile and a chunk of k-levels, and copies each level's input boxes into
// a ring of shared-memory buffers with cp.async (PTX cp.async.cg.shared.global, 16-byte
// chunks: the reference layout's rows of nx + 2h floats start at any 4-byte boundary and are
// not 16-byte multiples, so a tensor-map copy cannot address them, but each row's aligned
// chunks can be copied), one level or more ahead of the level it computes.
//
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "oeb_common.cuh"
#include "stencil_util.cuh"

namespace oeb {

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// waits until at most N of this thread's committed groups are still in flight
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// A W x H box of a field staged by rows of 16-byte chunks.  The reference layout gives a row
// no alignment beyond 4 bytes, so each row is copied as the aligned 16-byte chunks that cover
// its cells, and cell (a, b) of the box lands at s[b * SW + mis(b) + a], mis(b) in 0..3 being
// how far the row's first cell lies past the chunk boundary.  Copying whole aligned chunks may
// read up to three cells beyond either end of a row; such cells share a 16-byte granule with a
// cell of the field and are never used.
template <int W, int H>
struct RowBox {
  static constexpr int C = (W + 6) / 4;  // chunks a row: W cells starting anywhere in a chunk
  static constexpr int SW = 4 * C;       // floats a row in shared memory
  static constexpr int N = H * SW;
};

// cp.async of one aligned 16-byte chunk (L2 only, PTX cp.async.cg.shared.global).
__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

// cp.async of one 4-byte cell (PTX cp.async.ca.shared.global with a source size): the cell at
// gmem when ok, else zeros (nothing is read; gmem must still point into the field).  For
// tiles whose phases index the shared copy directly, with no per-row offset.
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, bool ok) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(ok ? 4 : 0) : "memory");
}

// Cells a row of a box lies past its first chunk boundary: (m0 + b * s3) & 3 for row b.
struct RowMis {
  int m0, s3;
  __device__ __forceinline__ int operator()(int b) const { return (m0 + b * s3) & 3; }
};
__device__ __forceinline__ RowMis row_mis(const float* g, int64_t kofs, int ib0, int jb0, int64_t sj) {
  const uintptr_t p = reinterpret_cast<uintptr_t>(g + kofs + ib0 + (int64_t)jb0 * sj);
  return RowMis{(int)((p >> 2) & 3), (int)(sj & 3)};
}

// Issues the copies of the W x H box of field g at level offset kofs whose first cell is
// (ib0, jb0), for the rows j in [jb, je) and the chunks holding a cell i in [ib, ie).
template <int W, int H>
__device__ __forceinline__ void stage_rows(float* s, const float* __restrict__ g, int64_t kofs, int ib0, int jb0,
                                           int64_t sj, int ib, int ie, int jb, int je) {
  constexpr int C = RowBox<W, H>::C, SW = RowBox<W, H>::SW;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  const RowMis mis = row_mis(g, kofs, ib0, jb0, sj);
  for (int e = tid; e < H * C; e += kThreads) {
    const int b = e / C;
    const int c = e - b * C;
    const int j = jb0 + b;
    const int ic = ib0 - mis(b) + 4 * c;  // first cell of the chunk
    if (j < jb || j >= je || ic + 3 < ib || ic >= ie) continue;
    cp_async16(s + b * SW + 4 * c, g + kofs + ic + (int64_t)j * sj);
  }
}

// Reads cell (a, b) of a box staged by stage_rows.
template <int W, int H>
struct RowView {
  const float* s;
  RowMis mis;
  __device__ __forceinline__ float operator()(int a, int b) const { return s[b * RowBox<W, H>::SW + mis(b) + a]; }
};
template <int W, int H>
__device__ __forceinline__ RowView<W, H> row_view(const float* s, const float* g, int64_t kofs, int ib0, int jb0,
                                                  int64_t sj) {
  return RowView<W, H>{s, row_mis(g, kofs, ib0, jb0, sj)};
}

// k-levels a CTA of a staged kernel marches: the most k-chunks per tile that keep every CTA in
// one wave of `ctas_per_sm` CTAs on every SM, then the levels of a chunk (at least 1).
int staged_kb(int tiles, int nz, int ctas_per_sm);

}  // namespace oeb
