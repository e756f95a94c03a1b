// stencil_util.cuh -- device helpers shared by the stencil kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "launch.cuh"
#include "oeb_common.cuh"
#include "precision.cuh"

namespace oeb {

// Threads per CTA of every tiled kernel: 32 lanes along i times 8 rows along j.
constexpr int kTX = 32;
constexpr int kTY = 8;
constexpr int kThreads = kTX * kTY;

// Runs f(a, b) for every cell (a, b) of a W x H region of a shared-memory tile, spread
// over the CTA's threads (a along i, fastest).
template <int W, int H, class F>
__device__ __forceinline__ void for_region(F&& f) {
  const int tid = threadIdx.y * kTX + threadIdx.x;
#pragma unroll 1
  for (int e = tid; e < W * H; e += kThreads) {
    const int b = e / W;
    const int a = e - b * W;
    f(a, b);
  }
}

// for_region over the first w x h cells of the W x H region only (a < w, b < h): a tile at
// the edge of its output box skips the cells no output needs.  Full tiles take the
// compile-time loop.
template <int W, int H, class F>
__device__ __forceinline__ void for_region_lim(int w, int h, F&& f) {
  if (w >= W && h >= H) {
    for_region<W, H>(f);
    return;
  }
  if (w <= 0 || h <= 0) return;
  const int tid = threadIdx.y * kTX + threadIdx.x;
#pragma unroll 1
  for (int e = tid; e < w * h; e += kThreads) {
    const int b = e / w;
    const int a = e - b * w;
    f(a, b);
  }
}

// Brings the 128-byte line holding `p` into L2 (PTX prefetch.global.L2); `p` must lie in a
// field the kernel reads.
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Prefetches into L2, for the 32 x 32 tile at (i0, j0) of plane offset kofs, every line that
// the tile's interior cells (0 <= i < nx, 0 <= j < ny: inside every field's reach) of each of
// the N fields cover (two 128-byte lines a row of 32 doubles, one of 32 floats), spread over
// the CTA's threads.
template <class T, int N>
__device__ __forceinline__ void prefetch_tile(const T* const (&fields)[N], int64_t kofs, int i0, int j0, int nx,
                                              int ny, int sj) {
  constexpr int kLines = 32 * (int)sizeof(T) / 128;  // lines a row
  const int tid = threadIdx.y * kTX + threadIdx.x;
  for (int e = tid; e < N * 32 * kLines; e += kThreads) {
    const int f = e / (32 * kLines), r = (e / kLines) % 32, l = e % kLines;
    const int i = i0 + l * (128 / (int)sizeof(T)), j = j0 + r;
    if (i >= 0 && j >= 0 && i < nx && j < ny) prefetch_l2(fields[f] + kofs + i + (int64_t)j * sj);
  }
}

// Read-only global load through the non-coherent path.  The step kernel (step.cu), whose later
// tasks read what earlier tasks of the same launch wrote, compiles the bodies with
// OEB_COHERENT_LOADS: an ordinary cached load, which observes those writes once the task's wait
// (an acquire, then a CTA barrier) has seen them counted; the non-coherent path is defined only
// for data that nothing writes while the kernel runs.
template <class T>
__device__ __forceinline__ T ld(const T* p) {
#ifdef OEB_COHERENT_LOADS
  return __ldca(p);
#else
  return __ldg(p);
#endif
}

// std::min(0.5, std::max(0.0, x)) with libstdc++'s comparisons (hdiffsmag.h:236, :251):
// max(a,b) = (a < b) ? b : a, min(a,b) = (b < a) ? b : a.  lo is >= +0 and not NaN, so its
// comparison with 0.5 may use the non-negative ordering.
template <class T>
__device__ __forceinline__ T clamp_smag(T x) {
  const T lo = Prec<T>::gt0(x) ? x : T(0.0);
  return Prec<T>::lt_nonneg(lo, T(0.5)) ? lo : T(0.5);
}

// 1 / EARTH_RADIUS folded at compile time in the element type (include/util.h:17-18).
template <class T>
__host__ __device__ constexpr T earth_radius_recip() {
  return T(1.0) / T(6371.229e3);
}

// Rows of a thread's 4 (32 x 32 tile, 8 thread rows) that a kernel unrolls.  The FP64
// kernels' F64i arithmetic is long integer code, and four unrolled copies of a point's work
// overflow the instruction cache (measured: the advection stencils 16-20 % faster rolled).
template <class T>
struct RowUnroll {
  static constexpr int value = 32 / kTY;
};
template <>
struct RowUnroll<F64i> {
  static constexpr int value = 1;
};
// The same for the stencils whose per-point work is longest (advection, pressure gradient):
// FP32 unrolls two rows (measured at 256 x 256 x 80: hadvuv 89 -> 62 us, hadvuv5th 107 ->
// 77 us, nh_p_grad 101 -> 94 us against four; the advection times are those of a build with
// compensated flux sums, since replaced by the plain float sums), FP64 one.
template <class T>
struct HeavyRowUnroll {
  static constexpr int value = 2;
};
template <>
struct HeavyRowUnroll<F64i> {
  static constexpr int value = 1;
};

// Visits, for this thread, the cells (i, j, k) of the box [ilo, ilo+ni) x [jlo, jlo+nj) x
// [k0, k0+kb) of its CTA: blk.x/y pick a 32 x 32 tile, each thread takes 4 rows (U of them
// unrolled).  f(o, i, j) gets the plane-plus-in-plane offset o of (i, j, k) from the
// interior origin.
template <int U = 32 / kTY, class F>
__device__ __forceinline__ void for_box(const uint3& blk, const Dims& d, int ilo, int jlo, int ni, int nj, int kb,
                                        F&& f) {
  const int a = (int)(blk.x * 32 + threadIdx.x);
  if (a >= ni) return;
  const int i = ilo + a;
  const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  const int sj = (int)d.sj;
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
#pragma unroll U
    for (int r = 0; r < 32 / kTY; ++r) {
      const int b = (int)(blk.y * 32 + threadIdx.y) + kTY * r;
      if (b < nj) f(kofs + i + (jlo + b) * sj, i, jlo + b);
    }
  }
}

// for_box over the k-levels [k0, k0+kb) of [0, nk) (nk may exceed the interior's nz: the
// boxes of fields read at k+1), handing f the level as well: f(o, i, j, k).
template <int U = 32 / kTY, class F>
__device__ __forceinline__ void for_box_k(const uint3& blk, int64_t sj, int64_t sk, int ilo, int jlo, int ni, int nj,
                                          int nk, int kb, F&& f) {
  const int a = (int)(blk.x * 32 + threadIdx.x);
  if (a >= ni) return;
  const int i = ilo + a;
  const int k0 = blk.z * kb, k1 = min(k0 + kb, nk);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * sk;
#pragma unroll U
    for (int r = 0; r < 32 / kTY; ++r) {
      const int b = (int)(blk.y * 32 + threadIdx.y) + kTY * r;
      if (b < nj) f(kofs + i + (int64_t)(jlo + b) * sj, i, jlo + b, k);
    }
  }
}

// Grid of a tiled kernel: one CTA per TI x TJ tile of the (i, j) region
// [ilo, ilo+ni) x [jlo, jlo+nj) and per kb k-levels.
inline dim3 tile_grid(int ni, int nj, int nz, int ti, int tj, int kb) {
  return dim3((unsigned)((ni + ti - 1) / ti), (unsigned)((nj + tj - 1) / tj), (unsigned)((nz + kb - 1) / kb));
}

}  // namespace oeb
