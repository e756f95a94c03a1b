// k_fvtp2d.cu -- fvtp2d (kernels/fvtp2d.h:4-177, the serial variant) in FP64 and FP32.
//
// FP64: two launches per call, per k-level tiles of 32 x 32 with every PPM intermediate computed
// once per point into shared memory:
//   1. fvtp2d_q:    y-PPM of q -> fy2 (fvtp2d.h:8-37), x-PPM of q -> fx2 (:84-113), then
//                   q_i (:39-51) and q_j (:115-127).  Tiles cover the extended index range
//                   [-3, N+2) of these arrays; each value is written exactly where the
//                   reference writes it (fy2, q_i: i in [-3,N+2); fx2, q_j: j in [-3,N+2)).
//   2. fvtp2d_flux: x-PPM of q_i -> fx1 (:53-82), y-PPM of q_j -> fy1 (:129-158) and the
//                   transport fluxes fx1 = (fx1+fx2)/2 * xfx, fy1 = (fy1+fy2)/2 * yfx (:160-176).
// q_i, q_j, fx2 and fy2 are outputs of the reference signature; launch 2 reads them back
// from global memory (the FP64 pipe, not HBM, bounds this kernel, so storing them costs
// less than recomputing their aprons).  FP32, bound by memory instead, runs one launch that
// recomputes the aprons (fvtp2d_fused_kernel).
//
// Compiled with --fmad=false (see k_pointwise.cu).  In FP32 the monotonicity flag smt5 is decided
// on the exact product (precision.cuh).
#include <type_traits>

#include "oeb_reach.cuh"
#include "precision.cuh"
#include "stage.cuh"
#include "stencil_util.cuh"
#include "tangent.cuh"

// Built on its own, this file's bodies and helpers are local to it; the step kernel
// (step.cu) includes it with OEB_BODIES_ONLY and a namespace of its own instead.
#ifndef OEB_BODIES_NS
#define OEB_BODIES_NS
#endif
namespace oeb {
namespace OEB_BODIES_NS {

constexpr int kT = 32;

// PPM edge value al(j) = p1 (q(j-1) + q(j)) + p2 (q(j-2) + q(j+1))   (fvtp2d.h:12)
template <class T>
__device__ __forceinline__ T ppm_al(T p1, T p2, T qm2, T qm1, T q0, T qp1) {
  return (p1 * (qm1 + q0)) + (p2 * (qm2 + qp1));
}

// fvtp2d.h:20-23: almq = al - q, br = al(+1) - q, smt5 = almq*br < 0 (b0 = almq + br is formed
// where it is used: ppm_flux uses one of its two b0 operands, so forming it there is one
// addition a flux point, as storing it was one an aux point, of the same operands)
template <class T>
__device__ __forceinline__ void ppm_aux(T al0, T al1, T q0, T* almq, T* br, unsigned char* smt) {
  const T m = al0 - q0;
  const T r = al1 - q0;
  *almq = m;
  *br = r;
  *smt = Prec<T>::prod_lt0(m, r);
}

// fvtp2d.h:28-34: upwind flux at point j from the aux values at j-1 and j.  The flag sum
// smt5(j-1) + smt5(j)*(smt5(j-1)==0) is exactly 1.0 when either flag is set, else 0.0.
// Branch-free: each lane selects the operands of its upwind side and performs that side's
// FP64 operations, (1 - c)(br - c b0) as 1 + (-c) and br + (-(c b0)) -- the same values, an
// IEEE subtraction being the addition of the negation -- so no warp runs both sides.
template <class T>
__device__ __forceinline__ T ppm_flux(T c, T q_m1, T q_0, T almq_m1, T br_m1, T almq_0, T br_0, unsigned char smt_m1,
                                      unsigned char smt_0) {
  const bool pos = gt0(c);
  const T u = T(1.) + (pos ? -c : c);
  const T b0 = (pos ? almq_m1 : almq_0) + (pos ? br_m1 : br_0);  // fvtp2d.h:22 at the upwind side
  const T p = c * b0;
  const T v = (pos ? br_m1 : almq_0) + (pos ? -p : p);
  return Prec<T>::add_flag(pos ? q_m1 : q_0, u * v, (smt_m1 | smt_0) != 0);
}

// ------------------------------ launch 1 ---------------------------------------------
// The y pass (fy2, fyy, then q_i) and the x pass (fx2, fxx, then q_j) are independent given
// q: each CTA does one of them (blk.z's low bit picks the axis) and holds only the part of
// the q tile and the PPM intermediates that pass reads, with fyy / fxx in the place of al,
// which is dead once the aux values are set (37 KB a CTA in FP64; its 42 registers a thread
// allow five CTAs per SM).
// Tile origin (i0, j0) = (-3 + 32 bx, -3 + 32 by).  Shared layout:
//   y pass: q 32 x 39 (i0+a, j0-3+b); al 32 x 35 (i0+a, j0-1+b), then fyy 32 x 33 (i0+a, j0+b)
//           = yfy * fy2, 0 outside fy2's range; almq/br/smt 32 x 34 (i0+a, j0-1+b)
//   x pass: q 38 x 32 (i0-3+a, j0+b); al 35 x 32 (i0-1+a, j0+b), then fxx 33 x 32 (i0+a, j0+b)
//           = xfx * fx2, 0 outside fx2's range; almq/br/smt 34 x 32 (i0-1+a, j0+b)
template <class T>
struct FvQSmem {
  union {
    struct {
      T q[39][32];
      union {
        T al[35][32];
        T fyy[33][32];
      } e;
      T almq[34][32], br[34][32];
      unsigned char smt[34][32];
    } y;
    struct {
      T q[32][38];
      union {
        T al[32][35];
        T fxx[32][33];
      } e;
      T almq[32][34], br[32][34];
      unsigned char smt[32][34];
    } x;
  } w;
};

template <class T>
struct fvtp2d_q_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFvQ);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ q_i, T* __restrict__ q_j,
                                             T* __restrict__ fx2, T* __restrict__ fy2, const T* __restrict__ q,
                                             const T* __restrict__ crx, const T* __restrict__ cry,
                                             const T* __restrict__ ra_x, const T* __restrict__ ra_y,
                                             const T* __restrict__ xfx, const T* __restrict__ yfx,
                                             const T* __restrict__ area, T p1, T p2, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FvQSmem<T>& s = *reinterpret_cast<FvQSmem<T>*>(smem_raw);
    const int i0 = -3 + (int)blk.x * kT, j0 = -3 + (int)blk.y * kT;
    const int sj = (int)d.sj;
    const int nx = d.nx, ny = d.ny;
    const bool ypass = (blk.z & 1u) == 0;
    const int k0 = (int)(blk.z >> 1) * kb, k1 = min(k0 + kb, d.nz);
    // the cells each phase needs for this tile's outputs (fewer at the output box's far
    // edge: the box is nx+5 wide, so the last tile column holds a few useful columns only)
    auto lim = [](int v, int hi) { return max(0, min(v, hi)); };
    auto qok = [&](int i, int j) { return i >= -3 && i < nx + 3 && j >= -3 && j < ny + 3; };
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      if (ypass) {
        auto& w = s.w.y;
        const int ax = lim(nx + 2 - i0, 32);   // columns of fy2 and q_i
        const int yfb = lim(ny + 1 - j0, 33);  // rows of fy2 / fyy
        const int qib = lim(ny - j0, 32);      // rows of q_i
        const T* const late[4] = {cry, yfx, area, ra_y};  // read after the PPM phases
        prefetch_tile(late, kofs, i0, j0, nx, ny, sj);
        // (one row more than the phases read, so that full tiles take the compile-time loop)
        for_region_lim<32, 39>(ax, min(39, max(yfb + 6, qib + 3)), [&](int a, int b) {
          const int i = i0 + a, j = j0 - 3 + b;
          w.q[b][a] = qok(i, j) ? ld(q + kofs + i + j * sj) : T(0);
        });
        __syncthreads();
        for_region_lim<32, 35>(ax, yfb + 2, [&](int a, int b) {
          w.e.al[b][a] = ppm_al(p1, p2, w.q[b][a], w.q[b + 1][a], w.q[b + 2][a], w.q[b + 3][a]);
        });
        __syncthreads();
        for_region_lim<32, 34>(ax, yfb + 1, [&](int a, int b) {
          ppm_aux(w.e.al[b][a], w.e.al[b + 1][a], w.q[b + 2][a], &w.almq[b][a], &w.br[b][a], &w.smt[b][a]);
        });
        __syncthreads();
        for_region_lim<32, 33>(ax, yfb, [&](int a, int b) {
          const int i = i0 + a, j = j0 + b;
          T fyy = T(0);
          if (i >= -3 && i < nx + 2 && j >= 0 && j < ny + 1) {  // fvtp2d.h:26-27
            const int64_t o = kofs + i + j * sj;
            const T f = ppm_flux(ld(cry + o), w.q[b + 2][a], w.q[b + 3][a], w.almq[b][a], w.br[b][a],
                                 w.almq[b + 1][a], w.br[b + 1][a], w.smt[b][a], w.smt[b + 1][a]);
            if (b < kT) fy2[o] = f;
            fyy = ld(yfx + o) * f;  // fvtp2d.h:43
          }
          w.e.fyy[b][a] = fyy;  // al is dead: the aux values are set
        });
        __syncthreads();
        // q_i (fvtp2d.h:48)
        for_region_lim<32, 32>(ax, qib, [&](int a, int b) {
          const int i = i0 + a, j = j0 + b;
          if (i >= -3 && i < nx + 2 && j >= 0 && j < ny) {
            const int64_t o = kofs + i + j * sj;
            q_i[o] = (((w.q[b + 3][a] * ld(area + o)) + w.e.fyy[b][a]) - w.e.fyy[b + 1][a]) / ld(ra_y + o);
          }
        });
        __syncthreads();
      } else {
        auto& w = s.w.x;
        const int xfa = lim(nx + 1 - i0, 33);  // columns of fx2 / fxx
        const int by = lim(ny + 2 - j0, 32);   // rows of fx2 and q_j
        const int qja = lim(nx - i0, 32);      // columns of q_j
        const T* const late[4] = {crx, xfx, area, ra_x};
        prefetch_tile(late, kofs, i0, j0, nx, ny, sj);
        for_region_lim<38, 32>(min(38, max(xfa + 5, qja + 3)), by, [&](int a, int b) {
          const int i = i0 - 3 + a, j = j0 + b;
          w.q[b][a] = qok(i, j) ? ld(q + kofs + i + j * sj) : T(0);
        });
        __syncthreads();
        for_region_lim<35, 32>(xfa + 2, by, [&](int a, int b) {
          w.e.al[b][a] = ppm_al(p1, p2, w.q[b][a], w.q[b][a + 1], w.q[b][a + 2], w.q[b][a + 3]);
        });
        __syncthreads();
        for_region_lim<34, 32>(xfa + 1, by, [&](int a, int b) {
          ppm_aux(w.e.al[b][a], w.e.al[b][a + 1], w.q[b][a + 2], &w.almq[b][a], &w.br[b][a], &w.smt[b][a]);
        });
        __syncthreads();
        for_region_lim<33, 32>(xfa, by, [&](int a, int b) {
          const int i = i0 + a, j = j0 + b;
          T fxx = T(0);
          if (i >= 0 && i < nx + 1 && j >= -3 && j < ny + 2) {  // fvtp2d.h:102-103
            const int64_t o = kofs + i + j * sj;
            const T f = ppm_flux(ld(crx + o), w.q[b][a + 2], w.q[b][a + 3], w.almq[b][a], w.br[b][a],
                                 w.almq[b][a + 1], w.br[b][a + 1], w.smt[b][a], w.smt[b][a + 1]);
            if (a < kT) fx2[o] = f;
            fxx = ld(xfx + o) * f;  // fvtp2d.h:119
          }
          w.e.fxx[b][a] = fxx;  // al is dead: the aux values are set
        });
        __syncthreads();
        // q_j (fvtp2d.h:124)
        for_region_lim<32, 32>(qja, by, [&](int a, int b) {
          const int i = i0 + a, j = j0 + b;
          if (i >= 0 && i < nx && j >= -3 && j < ny + 2) {
            const int64_t o = kofs + i + j * sj;
            q_j[o] = (((w.q[b][a + 3] * ld(area + o)) + w.e.fxx[b][a]) - w.e.fxx[b][a + 1]) / ld(ra_x + o);
          }
        });
        __syncthreads();
      }
    }
  }
};

// Grid of launch 1: the tiles of the output box [-3, n+2)^2, twice along z (one CTA per axis).
inline dim3 q_grid(const Dims& d, int kb) {
  dim3 g = tile_grid(d.nx + 5, d.ny + 5, d.nz, kT, kT, kb);
  g.z *= 2;
  return g;
}

// ------------------------------ launch 2 ---------------------------------------------
// The x sweep (fx1 from q_i) and the y sweep (fy1 from q_j) are independent: each CTA does
// one of them (blk.z's low bit picks the axis), so a CTA holds one field and one set of PPM
// intermediates (36 KB in FP64: six CTAs per SM) and half the dependent phases.
// Interior tile origin (i0, j0).  Shared layout:
//   x sweep: qi 37 x 32 (i0-3+a, j0+b); al 34 x 32 (i0-1+a, j0+b); almq/br/smt 33 x 32 (i0-1+a, j0+b)
//   y sweep: qj 32 x 37 (i0+a, j0-3+b); al 32 x 34 (i0+a, j0-1+b); almq/br/smt 32 x 33 (i0+a, j0-1+b)
template <class T>
struct FvFluxSmem {
  union {
    struct {
      T qi[32][37];
      T al[32][34];
      T almq[32][33], br[32][33];
      unsigned char smt[32][33];
    } x;
    struct {
      T qj[37][32];
      T al[34][32];
      T almq[33][32], br[33][32];
      unsigned char smt[33][32];
    } y;
  } w;
};

template <class T>
struct fvtp2d_flux_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFvFlux);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ fx1, T* __restrict__ fy1,
                                             const T* __restrict__ q_i, const T* __restrict__ q_j,
                                             const T* __restrict__ fx2, const T* __restrict__ fy2,
                                             const T* __restrict__ crx, const T* __restrict__ cry,
                                             const T* __restrict__ xfx, const T* __restrict__ yfx, T p1, T p2, Dims d,
                                             int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FvFluxSmem<T>& s = *reinterpret_cast<FvFluxSmem<T>*>(smem_raw);
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int sj = (int)d.sj;
    const int nx = d.nx, ny = d.ny;
    const bool ysweep = (blk.z & 1u) != 0;
    const int k0 = (int)(blk.z >> 1) * kb, k1 = min(k0 + kb, d.nz);
    // outputs of this tile (fewer at the domain's far edge) and what each phase needs for them
    const int vx = max(0, min(kT, nx - i0)), vy = max(0, min(kT, ny - j0));
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      if (!ysweep) {
        // ---- x-PPM of q_i -> fx1 and the x transport flux
        const T* const late[3] = {crx, fx2, xfx};  // read in the last phase only
        prefetch_tile(late, kofs, i0, j0, nx, ny, sj);
        for_region_lim<37, 32>(vx + 5, vy, [&](int a, int b) {
          const int i = i0 - 3 + a, j = j0 + b;
          s.w.x.qi[b][a] = (i < nx + 2 && j < ny) ? ld(q_i + kofs + i + j * sj) : T(0);
        });
        __syncthreads();
        for_region_lim<34, 32>(vx + 2, vy, [&](int a, int b) {
          s.w.x.al[b][a] = ppm_al(p1, p2, s.w.x.qi[b][a], s.w.x.qi[b][a + 1], s.w.x.qi[b][a + 2], s.w.x.qi[b][a + 3]);
        });
        __syncthreads();
        for_region_lim<33, 32>(vx + 1, vy, [&](int a, int b) {
          ppm_aux(s.w.x.al[b][a], s.w.x.al[b][a + 1], s.w.x.qi[b][a + 2], &s.w.x.almq[b][a], &s.w.x.br[b][a],
                &s.w.x.smt[b][a]);
        });
        __syncthreads();
        for_region_lim<32, 32>(vx, vy, [&](int a, int b) {
          const int i = i0 + a, j = j0 + b;
          if (i < nx && j < ny) {
            const int64_t o = kofs + i + j * sj;
            const T f = ppm_flux(ld(crx + o), s.w.x.qi[b][a + 2], s.w.x.qi[b][a + 3], s.w.x.almq[b][a], s.w.x.br[b][a],
                                 s.w.x.almq[b][a + 1], s.w.x.br[b][a + 1], s.w.x.smt[b][a], s.w.x.smt[b][a + 1]);
            fx1[o] = (scale2<-1>(f + ld(fx2 + o)) * ld(xfx + o));  // fvtp2d.h:164
          }
        });
        __syncthreads();
      } else {
        // ---- y-PPM of q_j -> fy1 and the y transport flux
        const T* const late[3] = {cry, fy2, yfx};
        prefetch_tile(late, kofs, i0, j0, nx, ny, sj);
        for_region_lim<32, 37>(vx, vy + 5, [&](int a, int b) {
          const int i = i0 + a, j = j0 - 3 + b;
          s.w.y.qj[b][a] = (i < nx && j < ny + 2) ? ld(q_j + kofs + i + j * sj) : T(0);
        });
        __syncthreads();
        for_region_lim<32, 34>(vx, vy + 2, [&](int a, int b) {
          s.w.y.al[b][a] = ppm_al(p1, p2, s.w.y.qj[b][a], s.w.y.qj[b + 1][a], s.w.y.qj[b + 2][a], s.w.y.qj[b + 3][a]);
        });
        __syncthreads();
        for_region_lim<32, 33>(vx, vy + 1, [&](int a, int b) {
          ppm_aux(s.w.y.al[b][a], s.w.y.al[b + 1][a], s.w.y.qj[b + 2][a], &s.w.y.almq[b][a], &s.w.y.br[b][a],
                &s.w.y.smt[b][a]);
        });
        __syncthreads();
        for_region_lim<32, 32>(vx, vy, [&](int a, int b) {
          const int i = i0 + a, j = j0 + b;
          if (i < nx && j < ny) {
            const int64_t o = kofs + i + j * sj;
            const T f = ppm_flux(ld(cry + o), s.w.y.qj[b + 2][a], s.w.y.qj[b + 3][a], s.w.y.almq[b][a], s.w.y.br[b][a],
                                 s.w.y.almq[b + 1][a], s.w.y.br[b + 1][a], s.w.y.smt[b][a], s.w.y.smt[b + 1][a]);
            fy1[o] = (scale2<-1>(f + ld(fy2 + o)) * ld(yfx + o));  // fvtp2d.h:173
          }
        });
        __syncthreads();
      }
    }
  }
};

// Grid of launch 2: the tiles of the interior, twice along z (one CTA per axis).
inline dim3 flux_grid(const Dims& d, int kb) {
  dim3 g = tile_grid(d.nx, d.ny, d.nz, kT, kT, kb);
  g.z *= 2;
  return g;
}

// ------------------------------ FP32: one launch -------------------------------------
// The FP32 call is bound by memory, and the two launches above move 2.1x its algorithmic
// bytes: launch 2 reads back q_i, q_j, fx2 and fy2, which launch 1 has just written.  Here one
// CTA per interior 32 x 32 tile and k-level does both sweeps of q over a 3-cell apron, in
// shared memory, and then the sweeps of q_i and q_j: nothing it writes is read back.
//   y pass of q on the columns [i0-3, i0+34): fy2 on rows [j0, j0+33), q_i on [j0, j0+32);
//   x pass of q on the rows [j0-3, j0+34): fx2 on columns [i0, i0+33), q_j on [i0, i0+32);
//   x-PPM of q_i and y-PPM of q_j on the tile: fx1 and fy1.
// The apron costs about 16 % more PPM arithmetic than the two launches.  Each value of q_i,
// q_j, fx2 and fy2 is written by the one tile that owns it: its own columns (rows), plus the
// three before the first tile and the extra ones after the last (those arrays' boxes reach
// 3 cells before the interior and 1 or 2 after it).  The arithmetic is launch 1's and launch
// 2's, operation for operation, so the results are the same bits.
// Shared layout (per k-level), tile origin (i0, j0), 37 = the apron width:
//   q    : 39 x 39, (i0-3+a, j0-3+b)
//   y pass (columns i0-3+a, a < 37): ya = al on rows j0-1+b (35), then fyy on rows j0+b (33);
//          ym, yr, ys = almq, br, smt5 on rows j0-1+b (34); qi on rows j0+b (32)
//   x pass (rows j0-3+b, b < 37): xa = al on columns i0-1+a (35), then fxx on i0+a (33);
//          xm, xr, xs on columns i0-1+a (34); qj on columns i0+a (32)
//   fx2c, fy2c: fx2 and fy2 on the tile (32 x 32)
//   second stage, over the dead aux arrays: x-PPM of qi (al on i0-1+a, 34; aux 33) and
//   y-PPM of qj (al on j0-1+b, 34; aux 33)
template <class T>
struct FvFusedSmem {
  T q[39][39];
  T ya[35][37];
  T ym[34][37], yr[34][37];
  unsigned char ys[34][37];
  T qi[32][37];
  T xa[37][35];
  T xm[37][34], xr[37][34];
  unsigned char xs[37][34];
  T qj[37][32];
  T fx2c[32][32], fy2c[32][32];
};

// Asks L2 for the lines of field f (level offset kofs) that hold the cells [ilo, ihi) x
// [jlo, jhi) (empty ranges ask nothing), spread over the CTA's threads; the ranges lie in the
// field's reach.
template <class T>
__device__ __forceinline__ void prefetch_box(const T* f, int64_t kofs, int ilo, int ihi, int jlo, int jhi, int sj) {
  if (ihi <= ilo || jhi <= jlo) return;
  const uintptr_t first = reinterpret_cast<uintptr_t>(f + kofs + ilo) / 128;
  const int lines = (int)((reinterpret_cast<uintptr_t>(f + kofs + ihi - 1) / 128) - first) + 1;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  for (int e = tid; e < lines * (jhi - jlo); e += kThreads) {
    const int r = e / lines, l = e - r * lines;
    const T* row = f + kofs + (int64_t)(jlo + r) * sj;
    const uintptr_t a = (reinterpret_cast<uintptr_t>(row + ilo) / 128 + l) * 128;
    // the line's first cell of the range (clamped into it), so the address lies in the field
    const uintptr_t lo = reinterpret_cast<uintptr_t>(row + ilo), hi = reinterpret_cast<uintptr_t>(row + ihi - 1);
    prefetch_l2(reinterpret_cast<const void*>(a < lo ? lo : (a > hi ? hi : a)));
  }
}

template <class T>
struct fvtp2d_fused_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFvFused);  // the step kernel's id
  static constexpr int kCtasPerSm = 4;
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ q_i, T* __restrict__ q_j,
                                             T* __restrict__ fx1, T* __restrict__ fx2, T* __restrict__ fy1,
                                             T* __restrict__ fy2, const T* __restrict__ q, const T* __restrict__ crx,
                                             const T* __restrict__ cry, const T* __restrict__ ra_x,
                                             const T* __restrict__ ra_y, const T* __restrict__ xfx,
                                             const T* __restrict__ yfx, const T* __restrict__ area, T p1, T p2, Dims d,
                                             int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FvFusedSmem<T>& s = *reinterpret_cast<FvFusedSmem<T>*>(smem_raw);
    // second-stage arrays over the dead aux arrays of the first
    T(*xa2)[34] = reinterpret_cast<T(*)[34]>(&s.ym[0][0]);  // x-PPM of qi: al, 32 rows x 34
    T(*xm2)[33] = reinterpret_cast<T(*)[33]>(&s.yr[0][0]);  // almq, 32 x 33
    T(*xr2)[33] = reinterpret_cast<T(*)[33]>(&s.ya[0][0]);  // br, 32 x 33
    unsigned char(*xs2)[33] = reinterpret_cast<unsigned char(*)[33]>(&s.ys[0][0]);
    T(*ya3)[32] = reinterpret_cast<T(*)[32]>(&s.xm[0][0]);  // y-PPM of qj: al, 34 rows x 32
    T(*ym3)[32] = reinterpret_cast<T(*)[32]>(&s.xr[0][0]);  // almq, 33 x 32
    T(*yr3)[32] = reinterpret_cast<T(*)[32]>(&s.xa[0][0]);  // br, 33 x 32
    unsigned char(*ys3)[32] = reinterpret_cast<unsigned char(*)[32]>(&s.xs[0][0]);
    const int i0 = (int)blk.x * kT, j0 = (int)blk.y * kT;
    const int sj = (int)d.sj;
    const int nx = d.nx, ny = d.ny;
    const int k0 = (int)blk.z * kb, k1 = min(k0 + kb, d.nz);
    // cells this tile owns in the extended boxes of fy2 / q_i (columns) and fx2 / q_j (rows)
    const int ci0 = i0 == 0 ? -3 : i0, ci1 = i0 + kT >= nx ? nx + 2 : i0 + kT;
    const int rj0 = j0 == 0 ? -3 : j0, rj1 = j0 + kT >= ny ? ny + 2 : j0 + kT;
    const int fyr1 = j0 + kT >= ny ? ny + 1 : j0 + kT;  // rows of fy2 owned
    const int fxc1 = i0 + kT >= nx ? nx + 1 : i0 + kT;  // columns of fx2 owned
    auto qok = [&](int i, int j) { return i >= -3 && i < nx + 3 && j >= -3 && j < ny + 3; };
    // L2 prefetches: at each level, the inputs its later phases read, and the next level's q
    // (the loads of the late phases and of the next q tile then find their lines in L2)
    auto late_prefetch = [&](int64_t kofs) {
      prefetch_box(cry, kofs, max(i0 - 3, -3), min(i0 + 34, nx + 2), max(j0, 0), min(j0 + 33, ny + 1), sj);
      prefetch_box(yfx, kofs, max(i0 - 3, -3), min(i0 + 34, nx + 2), max(j0, 0), min(j0 + 33, ny + 1), sj);
      prefetch_box(crx, kofs, max(i0, 0), min(i0 + 33, nx + 1), max(j0 - 3, -3), min(j0 + 34, ny + 2), sj);
      prefetch_box(xfx, kofs, max(i0, 0), min(i0 + 33, nx + 1), max(j0 - 3, -3), min(j0 + 34, ny + 2), sj);
      prefetch_box(area, kofs, max(i0 - 3, -3), min(i0 + 34, nx + 2), max(j0 - 3, -3), min(j0 + 34, ny + 2), sj);
      prefetch_box(ra_y, kofs, max(i0 - 3, -3), min(i0 + 34, nx + 2), max(j0, 0), min(j0 + 32, ny), sj);
      prefetch_box(ra_x, kofs, max(i0, 0), min(i0 + 32, nx), max(j0 - 3, -3), min(j0 + 34, ny + 2), sj);
    };
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      late_prefetch(kofs);
      for_region<39, 39>([&](int a, int b) {
        const int i = i0 - 3 + a, j = j0 - 3 + b;
        s.q[b][a] = qok(i, j) ? ld(q + kofs + i + j * sj) : T(0);
      });
      if (k + 1 < k1)
        prefetch_box(q, kofs + d.sk, max(i0 - 3, -3), min(i0 + 36, nx + 3), max(j0 - 3, -3), min(j0 + 36, ny + 3), sj);
      __syncthreads();
      // edge values (fvtp2d.h:12, :57, :88, :133)
      for_region<37, 35>([&](int a, int b) {
        s.ya[b][a] = ppm_al(p1, p2, s.q[b][a], s.q[b + 1][a], s.q[b + 2][a], s.q[b + 3][a]);
      });
      for_region<35, 37>([&](int a, int b) {
        s.xa[b][a] = ppm_al(p1, p2, s.q[b][a], s.q[b][a + 1], s.q[b][a + 2], s.q[b][a + 3]);
      });
      __syncthreads();
      for_region<37, 34>([&](int a, int b) {
        ppm_aux(s.ya[b][a], s.ya[b + 1][a], s.q[b + 2][a], &s.ym[b][a], &s.yr[b][a], &s.ys[b][a]);
      });
      for_region<34, 37>([&](int a, int b) {
        ppm_aux(s.xa[b][a], s.xa[b][a + 1], s.q[b][a + 2], &s.xm[b][a], &s.xr[b][a], &s.xs[b][a]);
      });
      __syncthreads();
      // fy2 (fvtp2d.h:26-34) on (i0-3+a, j0+b) and fyy = yfx fy2 (:43), over the dead al
      for_region<37, 33>([&](int a, int b) {
        const int i = i0 - 3 + a, j = j0 + b;
        T fyy = T(0);
        if (i >= -3 && i < nx + 2 && j >= 0 && j < ny + 1) {
          const int64_t o = kofs + i + j * sj;
          const T f = ppm_flux(ld(cry + o), s.q[b + 2][a], s.q[b + 3][a], s.ym[b][a], s.yr[b][a], s.ym[b + 1][a],
                               s.yr[b + 1][a], s.ys[b][a], s.ys[b + 1][a]);
          if (i >= ci0 && i < ci1 && j < fyr1) fy2[o] = f;
          if (a >= 3 && a < 3 + kT && b < kT) s.fy2c[b][a - 3] = f;
          fyy = ld(yfx + o) * f;
        }
        s.ya[b][a] = fyy;
      });
      // fx2 (fvtp2d.h:102-110) on (i0+a, j0-3+b) and fxx = xfx fx2 (:119)
      for_region<33, 37>([&](int a, int b) {
        const int i = i0 + a, j = j0 - 3 + b;
        T fxx = T(0);
        if (i >= 0 && i < nx + 1 && j >= -3 && j < ny + 2) {
          const int64_t o = kofs + i + j * sj;
          const T f = ppm_flux(ld(crx + o), s.q[b][a + 2], s.q[b][a + 3], s.xm[b][a], s.xr[b][a], s.xm[b][a + 1],
                               s.xr[b][a + 1], s.xs[b][a], s.xs[b][a + 1]);
          if (j >= rj0 && j < rj1 && i < fxc1) fx2[o] = f;
          if (b >= 3 && b < 3 + kT && a < kT) s.fx2c[b - 3][a] = f;
          fxx = ld(xfx + o) * f;
        }
        s.xa[b][a] = fxx;
      });
      __syncthreads();
      // q_i (fvtp2d.h:48) on (i0-3+a, j0+b) and q_j (:124) on (i0+a, j0-3+b)
      for_region<37, 32>([&](int a, int b) {
        const int i = i0 - 3 + a, j = j0 + b;
        T v = T(0);
        if (i >= -3 && i < nx + 2 && j >= 0 && j < ny) {
          const int64_t o = kofs + i + j * sj;
          v = (((s.q[b + 3][a] * ld(area + o)) + s.ya[b][a]) - s.ya[b + 1][a]) / ld(ra_y + o);
          if (i >= ci0 && i < ci1) q_i[o] = v;
        }
        s.qi[b][a] = v;
      });
      for_region<32, 37>([&](int a, int b) {
        const int i = i0 + a, j = j0 - 3 + b;
        T v = T(0);
        if (i >= 0 && i < nx && j >= -3 && j < ny + 2) {
          const int64_t o = kofs + i + j * sj;
          v = (((s.q[b][a + 3] * ld(area + o)) + s.xa[b][a]) - s.xa[b][a + 1]) / ld(ra_x + o);
          if (j >= rj0 && j < rj1) q_j[o] = v;
        }
        s.qj[b][a] = v;
      });
      __syncthreads();
      // x-PPM of q_i (fvtp2d.h:53-82) and y-PPM of q_j (:129-158): edge values
      for_region<34, 32>([&](int a, int b) {
        xa2[b][a] = ppm_al(p1, p2, s.qi[b][a], s.qi[b][a + 1], s.qi[b][a + 2], s.qi[b][a + 3]);
      });
      for_region<32, 34>([&](int a, int b) {
        ya3[b][a] = ppm_al(p1, p2, s.qj[b][a], s.qj[b + 1][a], s.qj[b + 2][a], s.qj[b + 3][a]);
      });
      __syncthreads();
      for_region<33, 32>([&](int a, int b) {
        ppm_aux(xa2[b][a], xa2[b][a + 1], s.qi[b][a + 2], &xm2[b][a], &xr2[b][a], &xs2[b][a]);
      });
      for_region<32, 33>([&](int a, int b) {
        ppm_aux(ya3[b][a], ya3[b + 1][a], s.qj[b + 2][a], &ym3[b][a], &yr3[b][a], &ys3[b][a]);
      });
      __syncthreads();
      // fx1, fy1 (fvtp2d.h:164, :173)
      for_region<32, 32>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        if (i < nx && j < ny) {
          const int64_t o = kofs + i + j * sj;
          const T fx = ppm_flux(ld(crx + o), s.qi[b][a + 2], s.qi[b][a + 3], xm2[b][a], xr2[b][a], xm2[b][a + 1],
                                xr2[b][a + 1], xs2[b][a], xs2[b][a + 1]);
          fx1[o] = (scale2<-1>(fx + s.fx2c[b][a]) * ld(xfx + o));
          const T fy = ppm_flux(ld(cry + o), s.qj[b + 2][a], s.qj[b + 3][a], ym3[b][a], yr3[b][a], ym3[b + 1][a],
                                yr3[b + 1][a], ys3[b][a], ys3[b + 1][a]);
          fy1[o] = (scale2<-1>(fy + s.fy2c[b][a]) * ld(yfx + o));
        }
      });
      __syncthreads();
    }
  }
};

constexpr int kKB = 1;  // k-levels per CTA by default (the most CTAs hide latency best)

template <class T, class M3>
oeb_status fvtp2d_entry(const M3* q_i, const M3* q_j, const M3* fx1, const M3* fx2, const M3* fy1, const M3* fy2,
                        const M3* q, const M3* crx, const M3* cry, const M3* ra_x, const M3* ra_y, const M3* xfx,
                        const M3* yfx, const M3* area, T p1, T p2, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gqi, gqj, gfx1, gfx2, gfy1, gfy2, gq, gcx, gcy, grx, gry, gxf, gyf, gar;
  const Reach rx_ext = kFvFx2;  // fx2 written, crx and xfx read: i in [0,N], j in [-3,N+1]
  const Reach ry_ext = kFvFy2;  // fy2 written, cry and yfx read: i in [-3,N+1], j in [0,N]
  OEB_TRY((check_field3<T>(q_i, *dom, kFvQi, &gqi)));
  OEB_TRY((check_field3<T>(q_j, *dom, kFvQj, &gqj)));
  OEB_TRY((check_field3<T>(fx1, *dom, kInterior, &gfx1)));
  OEB_TRY((check_field3<T>(fx2, *dom, rx_ext, &gfx2)));
  OEB_TRY((check_field3<T>(fy1, *dom, kInterior, &gfy1)));
  OEB_TRY((check_field3<T>(fy2, *dom, ry_ext, &gfy2)));
  OEB_TRY((check_field3<T>(q, *dom, Reach{3, 3, 3, 3, 0, 0}, &gq)));
  OEB_TRY((check_field3<T>(crx, *dom, rx_ext, &gcx)));
  OEB_TRY((check_field3<T>(cry, *dom, ry_ext, &gcy)));
  OEB_TRY((check_field3<T>(ra_x, *dom, Reach{0, 0, 3, 2, 0, 0}, &grx)));
  OEB_TRY((check_field3<T>(ra_y, *dom, Reach{3, 2, 0, 0, 0, 0}, &gry)));
  OEB_TRY((check_field3<T>(xfx, *dom, rx_ext, &gxf)));
  OEB_TRY((check_field3<T>(yfx, *dom, ry_ext, &gyf)));
  OEB_TRY((check_field3<T>(area, *dom, Reach{3, 2, 3, 2, 0, 0}, &gar)));
  OEB_TRY(check_same_strides<T>({&gqi, &gqj, &gfx1, &gfx2, &gfy1, &gfy2, &gq, &gcx, &gcy, &grx, &gry, &gxf,
                                      &gyf, &gar}));
  OEB_TRY(check_no_alias({gqi.lo, gqi.hi, gqj.lo, gqj.hi, gfx1.lo, gfx1.hi, gfx2.lo, gfx2.hi, gfy1.lo, gfy1.hi,
                          gfy2.lo, gfy2.hi},
                         {gq.lo, gq.hi, gcx.lo, gcx.hi, gcy.lo, gcy.hi, grx.lo, grx.hi, gry.lo, gry.hi, gxf.lo,
                          gxf.hi, gyf.lo, gyf.hi, gar.lo, gar.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gq.sj, gq.sk};
  cudaStream_t st = (cudaStream_t)stream;
  const int kb = tuned_kb(kKB);
  if constexpr (std::is_same<T, float>::value) {
    // FP32 is bound by memory: one launch, nothing read back
    const int tiles = ((d.nx + kT - 1) / kT) * ((d.ny + kT - 1) / kT);
    const int kbf = tuned_kb(staged_kb(tiles, d.nz, fvtp2d_fused_kernel<T>::kCtasPerSm));
    return launch<fvtp2d_fused_kernel<T>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kbf), sizeof(FvFusedSmem<T>), st,
                                          gqi.origin, gqj.origin, gfx1.origin, gfx2.origin, gfy1.origin, gfy2.origin,
                                          gq.origin, gcx.origin, gcy.origin, grx.origin, gry.origin, gxf.origin,
                                          gyf.origin, gar.origin, p1, p2, d, kbf);
  }
  OEB_TRY(launch<fvtp2d_q_kernel<T>>(q_grid(d, kb), sizeof(FvQSmem<T>), st,
                                     gqi.origin, gqj.origin, gfx2.origin, gfy2.origin, gq.origin, gcx.origin,
                                     gcy.origin, grx.origin, gry.origin, gxf.origin, gyf.origin, gar.origin, p1, p2, d,
                                     kb));
  return launch<fvtp2d_flux_kernel<T>>(flux_grid(d, kb), sizeof(FvFluxSmem<T>), st,
                                       gfx1.origin, gfy1.origin, gqi.origin, gqj.origin, gfx2.origin, gfy2.origin,
                                       gcx.origin, gcy.origin, gxf.origin, gyf.origin, p1, p2, d, kb);
}

// Tangent-linear fvtp2d with respect to q (the PPM flags frozen at q; the Courant numbers,
// fluxes and areas are parameters): derivatives of all six outputs, on Dual<T>.
template <class T, class M3>
oeb_status fvtp2d_tl_entry(const M3* dq_i, const M3* dq_j, const M3* dfx1, const M3* dfx2, const M3* dfy1,
                           const M3* dfy2, const M3* q, const M3* crx, const M3* cry, const M3* ra_x, const M3* ra_y,
                           const M3* xfx, const M3* yfx, const M3* area, const M3* dq, T p1, T p2,
                           const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(fvtp2d_entry<T>(dq_i, dq_j, dfx1, dfx2, dfy1, dfy2, q, crx, cry, ra_x, ra_y, xfx, yfx, area, p1, p2, dom,
                            stream));
    OEB_TRY(fvtp2d_entry<T>(dq_i, dq_j, dfx1, dfx2, dfy1, dfy2, dq, crx, cry, ra_x, ra_y, xfx, yfx, area, p1, p2, dom,
                            stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  cudaStream_t st = (cudaStream_t)stream;
  DualArrays<T> arr(st);
  D *x, *cx, *cy, *rx, *ry, *xf, *yf, *ar, *oqi, *oqj, *ofx1, *ofx2, *ofy1, *ofy2;
  OEB_TRY(arr.pack(q, dq, &x));
  OEB_TRY(arr.pack(crx, (const M3*)nullptr, &cx));
  OEB_TRY(arr.pack(cry, (const M3*)nullptr, &cy));
  OEB_TRY(arr.pack(ra_x, (const M3*)nullptr, &rx));
  OEB_TRY(arr.pack(ra_y, (const M3*)nullptr, &ry));
  OEB_TRY(arr.pack(xfx, (const M3*)nullptr, &xf));
  OEB_TRY(arr.pack(yfx, (const M3*)nullptr, &yf));
  OEB_TRY(arr.pack(area, (const M3*)nullptr, &ar));
  OEB_TRY(arr.alloc(dq_i, &oqi));
  OEB_TRY(arr.alloc(dq_j, &oqj));
  OEB_TRY(arr.alloc(dfx1, &ofx1));
  OEB_TRY(arr.alloc(dfx2, &ofx2));
  OEB_TRY(arr.alloc(dfy1, &ofy1));
  OEB_TRY(arr.alloc(dfy2, &ofy2));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, q->strides[1], q->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<fvtp2d_q_kernel<D>>(q_grid(d, kb), sizeof(FvQSmem<D>), st, oqi,
                                     oqj, ofx2, ofy2, x, cx, cy, rx, ry, xf, yf, ar, D(p1), D(p2), d, kb));
  OEB_TRY(launch<fvtp2d_flux_kernel<D>>(flux_grid(d, kb), sizeof(FvFluxSmem<D>), st, ofx1,
                                        ofy1, oqi, oqj, ofx2, ofy2, cx, cy, xf, yf, D(p1), D(p2), d, kb));
  OEB_TRY(arr.unpack(dq_i->aligned + dq_i->offset, oqi, *dom, kFvQi, d.sj, d.sk));
  OEB_TRY(arr.unpack(dq_j->aligned + dq_j->offset, oqj, *dom, kFvQj, d.sj, d.sk));
  OEB_TRY(arr.unpack(dfx1->aligned + dfx1->offset, ofx1, *dom, kInterior, d.sj, d.sk));
  OEB_TRY(arr.unpack(dfx2->aligned + dfx2->offset, ofx2, *dom, kFvFx2, d.sj, d.sk));
  OEB_TRY(arr.unpack(dfy1->aligned + dfy1->offset, ofy1, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dfy2->aligned + dfy2->offset, ofy2, *dom, kFvFy2, d.sj, d.sk);
}

// ============================== adjoint ===========================================
// fvtp2d is linear in q once the PPM flags smt5 (and the upwind choice c > 0) are frozen
// at the state.  With ybar = (fx1b, fy1b) on the interior and gx = xfx fx1b / 2,
// gy = yfx fy1b / 2, the transpose is (fvtp2d.h:39-51, 115-127, 160-176 read backwards):
//   q_ib = PPMx^T(gx) on q_i's flags,  q_jb = PPMy^T(gy) on q_j's flags
//   fy2b = gy + yfx (q_ib / ra_y - q_ib(j-1) / ra_y(j-1)),  fx2b = gx + xfx (q_jb / ra_x - q_jb(i-1) / ra_x(i-1))
//   qb   = area/ra_y q_ib + area/ra_x q_jb + PPMy^T(fy2b) + PPMx^T(fx2b)
// q_i and q_j are recomputed by the forward kernel (recompute, not store).  The transpose
// of one PPM sweep (fvtp2d.h:20-34) is, per flux point j with tb = s (1 -+ c) Fb:
//   B0(j) = [c(j+1)>0] (-c(j+1)) tb(j+1) + [c(j)<=0] c(j) tb(j),  ALM(j) = [c(j)<=0] tb(j) + B0(j)
//   BR(j) = [c(j+1)>0] tb(j+1) + B0(j),  AL(j) = ALM(j) + BR(j-1)
//   gb(j) = [c(j+1)>0] Fb(j+1) + [c(j)<=0] Fb(j) - ALM(j) - BR(j)
//           + p1 (AL(j+1) + AL(j)) + p2 (AL(j+2) + AL(j-1))
// computed per CTA on a 32-line x 44-position shared window (positions A-5 .. A+38 along the
// sweep axis for the 32 outputs A .. A+31).

constexpr int kW = 44;  // window along the sweep axis: outputs A..A+31 need A-5 .. A+38

// Lines a CTA sweeps: 16 in FP64 (23 KB a CTA: the registers, not shared memory, then bound
// the CTAs per SM, at five or six against four with 32 lines), 32 in FP32 (eight CTAs per SM
// either way).
template <class T>
constexpr int adj_lines() {
  return 16;  // FP32: 16 measured faster than 32 (the FP32 adjoint 0.194 -> 0.172 ms at 128 x 128 x 80)
}

// gs and als are dead once the flags smt are set; tb and al take their places
template <class T, int LN>
struct PpmAdjSmem {
  union {
    T gs[LN][kW];  // state values of the swept field
    T al[LN][kW];
  } u0;
  union {
    T als[LN][kW];  // state edge values al
    T tb[LN][kW];
  } u1;
  T alm[LN][kW];
  T br[LN][kW];
  unsigned char smt[LN][kW];
};

// One transposed PPM sweep along AXIS (0: i, 1: j) for outputs A..A+nout-1 on lines
// L0..L0+nl-1 (nout <= 32, nl <= LN: a tile at the edge of its output box works on its own part of
// the window and lines only; every phase's window shrinks by the 32 - nout missing outputs).
// gst(p, l): state value at axis position p of line l (0 where the field is not defined);
// cv(p, l): Courant number at flux point p (any value elsewhere);
// fb(p, l): flux adjoint at p (0 off the flux points);  put(a, l, v): receives gbar(a).
template <class T, int AXIS, int LN, class GS, class CV, class FB, class PUT>
__device__ __forceinline__ void ppm_sweep_adjoint(PpmAdjSmem<T, LN>& s, int A, int L0, int nout, int nl, T p1, T p2,
                                                  GS&& gst, CV&& cv, FB&& fb, PUT&& put) {
  const int cut = 32 - nout;
  const bool full = cut == 0 && nl == LN;
  auto region = [&](int w0, int w1, auto&& f) {
    const int tid = threadIdx.y * kTX + threadIdx.x;
    if (full) {  // compile-time extents
      const int W = w1 - w0;
      for (int e = tid; e < W * LN; e += kThreads) {
        int w, l;
        if (AXIS == 0) {
          l = e / W;
          w = w0 + (e - l * W);
        } else {
          w = w0 + e / LN;
          l = e - (e / LN) * LN;
        }
        f(w, l);
      }
      return;
    }
    const int W = w1 - cut - w0;
    if (W <= 0 || nl <= 0) return;
    for (int e = tid; e < W * nl; e += kThreads) {
      int w, l;
      if (AXIS == 0) {
        l = e / W;
        w = w0 + (e - l * W);
      } else {
        w = w0 + e / nl;
        l = e - (e / nl) * nl;
      }
      f(w, l);
    }
  };
  region(0, kW, [&](int w, int l) { s.u0.gs[l][w] = gst(A - 5 + w, L0 + l); });
  __syncthreads();
  region(2, kW - 1, [&](int w, int l) {
    s.u1.als[l][w] = (p1 * (s.u0.gs[l][w - 1] + s.u0.gs[l][w])) + (p2 * (s.u0.gs[l][w - 2] + s.u0.gs[l][w + 1]));
  });
  __syncthreads();
  region(2, kW - 2, [&](int w, int l) {
    s.smt[l][w] = Prec<T>::prod_lt0(s.u1.als[l][w] - s.u0.gs[l][w], s.u1.als[l][w + 1] - s.u0.gs[l][w]);
  });
  __syncthreads();
  region(3, kW - 2, [&](int w, int l) {
    const int p = A - 5 + w;
    const T f = fb(p, L0 + l);
    T t = T(0);
    if (f != T(0) && (s.smt[l][w - 1] | s.smt[l][w])) {
      const T c = cv(p, L0 + l);
      t = f * ((c > T(0)) ? (T(1) - c) : (T(1) + c));
    }
    s.u1.tb[l][w] = t;
  });
  __syncthreads();
  region(3, kW - 3, [&](int w, int l) {
    const int p = A - 5 + w;
    const T t0 = s.u1.tb[l][w], t1 = s.u1.tb[l][w + 1];
    T b0 = T(0), am = T(0), bb = T(0);
    if (t1 != T(0)) {
      const T c1 = cv(p + 1, L0 + l);
      if (c1 > T(0)) {
        b0 = -c1 * t1;
        bb = t1;
      }
    }
    if (t0 != T(0)) {
      const T c0 = cv(p, L0 + l);
      if (!(c0 > T(0))) {
        b0 = b0 + c0 * t0;
        am = t0;
      }
    }
    s.alm[l][w] = am + b0;
    s.br[l][w] = bb + b0;
  });
  __syncthreads();
  region(4, kW - 3, [&](int w, int l) { s.u0.al[l][w] = s.alm[l][w] + s.br[l][w - 1]; });
  __syncthreads();
  region(5, 5 + 32, [&](int w, int l) {
    const int a = A - 5 + w;
    T g = fma(p1, s.u0.al[l][w + 1] + s.u0.al[l][w], fma(p2, s.u0.al[l][w + 2] + s.u0.al[l][w - 1], -s.alm[l][w])) - s.br[l][w];
    const T f1 = fb(a + 1, L0 + l);
    if (f1 != T(0) && cv(a + 1, L0 + l) > T(0)) g = g + f1;
    const T f0 = fb(a, L0 + l);
    if (f0 != T(0) && !(cv(a, L0 + l) > T(0))) g = g + f0;
    put(a, L0 + l, g);
  });
  __syncthreads();
}

// Pass 1: q_ib over i in [-3,N+2), j in [0,N) and q_jb over i in [0,N), j in [-3,N+2).
template <class T>
struct fvtp2d_adj_qij_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFvAdjQij);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ qib, T* __restrict__ qjb,
                                             const T* __restrict__ q_i, const T* __restrict__ q_j,
                                             const T* __restrict__ crx, const T* __restrict__ cry,
                                             const T* __restrict__ xfx, const T* __restrict__ yfx,
                                             const T* __restrict__ fx1b, const T* __restrict__ fy1b, T p1, T p2,
                                             Dims d, int AXIS_Y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int LN = adj_lines<T>();
    PpmAdjSmem<T, LN>& s = *reinterpret_cast<PpmAdjSmem<T, LN>*>(smem_raw);
    const int nx = d.nx, ny = d.ny, sj = (int)d.sj;
    const int64_t kofs = (int64_t)blk.z * d.sk;
    if (!AXIS_Y) {
      // x sweep of fx1 on q_i: outputs i in [-3, nx+2), lines j in [0, ny)
      const int A = -3 + (int)blk.x * 32, L0 = (int)blk.y * LN;
      ppm_sweep_adjoint<T, 0, LN>(
          s, A, L0, max(0, min(32, nx + 2 - A)), max(0, min(LN, ny - L0)), p1, p2,
          [&](int p, int l) { return (p >= -3 && p < nx + 2 && l < ny) ? ld(q_i + kofs + p + l * sj) : T(0); },
          [&](int p, int l) { return ld(crx + kofs + p + l * sj); },
          [&](int p, int l) {
            return (p >= 0 && p < nx && l < ny) ? (T(0.5) * ld(xfx + kofs + p + l * sj)) * ld(fx1b + kofs + p + l * sj)
                                               : T(0);
          },
          [&](int a, int l, T v) {
            if (a >= -3 && a < nx + 2 && l < ny) qib[kofs + a + l * sj] = v;
          });
    } else {
      // y sweep of fy1 on q_j: outputs j in [-3, ny+2), lines i in [0, nx)
      const int A = -3 + (int)blk.x * 32, L0 = (int)blk.y * LN;
      ppm_sweep_adjoint<T, 1, LN>(
          s, A, L0, max(0, min(32, ny + 2 - A)), max(0, min(LN, nx - L0)), p1, p2,
          [&](int p, int l) { return (p >= -3 && p < ny + 2 && l < nx) ? ld(q_j + kofs + l + p * sj) : T(0); },
          [&](int p, int l) { return ld(cry + kofs + l + p * sj); },
          [&](int p, int l) {
            return (p >= 0 && p < ny && l < nx) ? (T(0.5) * ld(yfx + kofs + l + p * sj)) * ld(fy1b + kofs + l + p * sj)
                                               : T(0);
          },
          [&](int a, int l, T v) {
            if (a >= -3 && a < ny + 2 && l < nx) qjb[kofs + l + a * sj] = v;
          });
    }
  }
};

// Pass 2: fy2b on [-3,N+2) x [0,N+1) and fx2b on [0,N+1) x [-3,N+2).
// fy2b(i,j) = g + yfx (ry(i,j) - ry(i,j-1)) with ry = q_ib / ra_y on rows [0, N) (0 elsewhere),
// fx2b(i,j) = g + xfx (rx(i,j) - rx(i-1,j)) with rx = q_jb / ra_x on columns [0, N): each
// quotient is read by two neighbouring points, so a CTA divides once per cell into shared
// memory (ry over its 33 rows j0-1.., rx over its 33 columns i0-1..) and forms both fluxes
// from there.  Tile origin (i0, j0) = (-3 + 32 bx, -3 + 32 by).
template <class T>
struct AdjF2Smem {
  T ry[33][32];  // (i0+a, j0-1+b)
  T rx[32][33];  // (i0-1+a, j0+b)
};

template <class T>
struct fvtp2d_adj_f2_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFvAdjF2);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ fx2b, T* __restrict__ fy2b,
                                             const T* __restrict__ qib, const T* __restrict__ qjb,
                                             const T* __restrict__ xfx, const T* __restrict__ yfx,
                                             const T* __restrict__ ra_x, const T* __restrict__ ra_y,
                                             const T* __restrict__ fx1b, const T* __restrict__ fy1b, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    AdjF2Smem<T>& s = *reinterpret_cast<AdjF2Smem<T>*>(smem_raw);
    const int nx = d.nx, ny = d.ny;
    const int64_t sj = d.sj;
    const int i0 = -3 + (int)blk.x * kT, j0 = -3 + (int)blk.y * kT;
    // outputs of this tile in the box [-3, nx+2) x [-3, ny+2)
    const int vx = max(0, min(kT, nx + 2 - i0)), vy = max(0, min(kT, ny + 2 - j0));
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      for_region_lim<32, 33>(vx, vy + 1, [&](int a, int b) {
        const int i = i0 + a, r = j0 - 1 + b;
        const int64_t o = kofs + i + r * sj;
        s.ry[b][a] = (r >= 0 && r < ny && i < nx + 2) ? qib[o] / ld(ra_y + o) : T(0);
      });
      for_region_lim<33, 32>(vx + 1, vy, [&](int a, int b) {
        const int c = i0 - 1 + a, j = j0 + b;
        const int64_t o = kofs + c + j * sj;
        s.rx[b][a] = (c >= 0 && c < nx && j < ny + 2) ? qjb[o] / ld(ra_x + o) : T(0);
      });
      __syncthreads();
      for_region_lim<32, 32>(vx, vy, [&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        const int64_t o = kofs + i + j * sj;
        const bool interior = i >= 0 && i < nx && j >= 0 && j < ny;
        if (j >= 0 && j < ny + 1) {
          T g = interior ? (T(0.5) * ld(yfx + o)) * ld(fy1b + o) : T(0);
          fy2b[o] = g + ld(yfx + o) * (s.ry[b + 1][a] - s.ry[b][a]);
        }
        if (i >= 0 && i < nx + 1) {
          T g = interior ? (T(0.5) * ld(xfx + o)) * ld(fx1b + o) : T(0);
          fx2b[o] = g + ld(xfx + o) * (s.rx[b][a + 1] - s.rx[b][a]);
        }
      });
      __syncthreads();
    }
  }
};

// Pass 3: qb on [-3,N+3)^2: area terms + PPMx^T(fx2b) (x sweep, writes), then
// pass 4: + PPMy^T(fy2b) (y sweep, adds).
template <class T>
struct fvtp2d_adj_q_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFvAdjQ);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ qb, const T* __restrict__ q,
                                             const T* __restrict__ crx, const T* __restrict__ cry,
                                             const T* __restrict__ area, const T* __restrict__ ra_x,
                                             const T* __restrict__ ra_y, const T* __restrict__ qib,
                                             const T* __restrict__ qjb, const T* __restrict__ fx2b,
                                             const T* __restrict__ fy2b, T p1, T p2, Dims d, int AXIS_Y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int LN = adj_lines<T>();
    PpmAdjSmem<T, LN>& s = *reinterpret_cast<PpmAdjSmem<T, LN>*>(smem_raw);
    const int nx = d.nx, ny = d.ny, sj = (int)d.sj;
    const int64_t kofs = (int64_t)blk.z * d.sk;
    auto qval = [&](int i, int j) {
      return (i >= -3 && i < nx + 3 && j >= -3 && j < ny + 3) ? ld(q + kofs + i + j * sj) : T(0);
    };
    const int A = -3 + (int)blk.x * 32, L0 = -3 + (int)blk.y * LN;
    if (!AXIS_Y) {
      // x sweep of fx2 on q: flux points i in [0, nx+1), lines j in [-3, ny+2)
      ppm_sweep_adjoint<T, 0, LN>(
          s, A, L0, max(0, min(32, nx + 3 - A)), max(0, min(LN, ny + 3 - L0)), p1, p2,
          [&](int p, int l) { return qval(p, l); },
          [&](int p, int l) { return ld(crx + kofs + p + l * sj); },
          [&](int p, int l) {
            return (p >= 0 && p < nx + 1 && l >= -3 && l < ny + 2) ? fx2b[kofs + p + l * sj] : T(0);
          },
          [&](int a, int l, T v) {
            if (a >= -3 && a < nx + 3 && l >= -3 && l < ny + 3) {
              const int64_t o = kofs + a + l * sj;
              T acc = v;
              if (a >= -3 && a < nx + 2 && l >= 0 && l < ny) acc = acc + (ld(area + o) / ld(ra_y + o)) * qib[o];
              if (a >= 0 && a < nx && l >= -3 && l < ny + 2) acc = acc + (ld(area + o) / ld(ra_x + o)) * qjb[o];
              qb[o] = acc;
            }
          });
    } else {
      // y sweep of fy2 on q: flux points j in [0, ny+1), lines i in [-3, nx+2); adds to qb
      ppm_sweep_adjoint<T, 1, LN>(
          s, A, L0, max(0, min(32, ny + 3 - A)), max(0, min(LN, nx + 3 - L0)), p1, p2,
          [&](int p, int l) { return qval(l, p); },
          [&](int p, int l) { return ld(cry + kofs + l + p * sj); },
          [&](int p, int l) {
            return (p >= 0 && p < ny + 1 && l >= -3 && l < nx + 2) ? fy2b[kofs + l + p * sj] : T(0);
          },
          [&](int a, int l, T v) {
            if (a >= -3 && a < ny + 3 && l >= -3 && l < nx + 3) qb[kofs + l + a * sj] = qb[kofs + l + a * sj] + v;
          });
    }
  }
};

template <class T, class M3>
oeb_status fvtp2d_adj_entry(const M3* qb, const M3* q, const M3* crx, const M3* cry, const M3* ra_x, const M3* ra_y,
                            const M3* xfx, const M3* yfx, const M3* area, const M3* fx1b, const M3* fy1b, T p1, T p2,
                            const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gqb, gq, gcx, gcy, grx, gry, gxf, gyf, gar, gf1, gg1;
  OEB_TRY((check_field3<T>(qb, *dom, Reach{3, 3, 3, 3, 0, 0}, &gqb)));
  OEB_TRY((check_field3<T>(q, *dom, Reach{3, 3, 3, 3, 0, 0}, &gq)));
  OEB_TRY((check_field3<T>(crx, *dom, kFvFx2, &gcx)));
  OEB_TRY((check_field3<T>(cry, *dom, kFvFy2, &gcy)));
  OEB_TRY((check_field3<T>(ra_x, *dom, Reach{0, 0, 3, 2, 0, 0}, &grx)));
  OEB_TRY((check_field3<T>(ra_y, *dom, Reach{3, 2, 0, 0, 0, 0}, &gry)));
  OEB_TRY((check_field3<T>(xfx, *dom, kFvFx2, &gxf)));
  OEB_TRY((check_field3<T>(yfx, *dom, kFvFy2, &gyf)));
  OEB_TRY((check_field3<T>(area, *dom, Reach{3, 2, 3, 2, 0, 0}, &gar)));
  OEB_TRY((check_field3<T>(fx1b, *dom, kInterior, &gf1)));
  OEB_TRY((check_field3<T>(fy1b, *dom, kInterior, &gg1)));
  OEB_TRY(check_same_strides<T>({&gqb, &gq, &gcx, &gcy, &grx, &gry, &gxf, &gyf, &gar, &gf1, &gg1}));
  OEB_TRY(check_no_alias({gqb.lo, gqb.hi}, {gq.lo, gq.hi, gcx.lo, gcx.hi, gcy.lo, gcy.hi, grx.lo, grx.hi, gry.lo,
                                            gry.hi, gxf.lo, gxf.hi, gyf.lo, gyf.hi, gar.lo, gar.hi, gf1.lo, gf1.hi,
                                            gg1.lo, gg1.hi}));
  OEB_RETURN_IF_VALIDATING();
  cudaStream_t st = (cudaStream_t)stream;
  // scratch in q's layout: q_i, q_j, fx2, fy2 (forward recompute), q_ib, q_jb, fx2b, fy2b
  const T* start = (q->allocated && q->allocated <= q->aligned) ? q->allocated : q->aligned;
  const int64_t last = (q->sizes[0] - 1) * q->strides[0] + (q->sizes[1] - 1) * q->strides[1] +
                       (q->sizes[2] - 1) * q->strides[2];
  const int64_t n = (int64_t)(q->aligned - start) + last + 1;
  const int64_t org = (int64_t)(q->aligned - start) + q->offset;
  void* buf = nullptr;
  OEB_TRY(scratch_alloc(&buf, (size_t)n * 8 * sizeof(T), st));
  T* base = static_cast<T*>(buf);
  T *sqi = base + org, *sqj = base + n + org, *sfx2 = base + 2 * n + org, *sfy2 = base + 3 * n + org,
    *qib = base + 4 * n + org, *qjb = base + 5 * n + org, *fx2b = base + 6 * n + org, *fy2b = base + 7 * n + org;
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gq.sj, gq.sk};
  const int kb = tuned_kb(kKB);
  constexpr int LN = adj_lines<T>();
  const size_t ps = sizeof(PpmAdjSmem<T, LN>);
  oeb_status stt = launch<fvtp2d_q_kernel<T>>(q_grid(d, kb), sizeof(FvQSmem<T>), st,
                                              sqi, sqj, sfx2, sfy2, gq.origin, gcx.origin, gcy.origin, grx.origin,
                                              gry.origin, gxf.origin, gyf.origin, gar.origin, p1, p2, d, kb);
  // the x and y sweeps of the two PPM adjoints (axis flag 0 / 1)
  for (int axis = 0; axis < 2 && stt == OEB_OK; ++axis) {
    const int a = axis ? d.ny : d.nx, l = axis ? d.nx : d.ny;
    stt = launch<fvtp2d_adj_qij_kernel<T>>(dim3((a + 5 + 31) / 32, (l + LN - 1) / LN, d.nz), ps, st, qib, qjb, sqi, sqj,
                                           gcx.origin, gcy.origin, gxf.origin, gyf.origin, gf1.origin, gg1.origin, p1,
                                           p2, d, axis);
  }
  if (stt == OEB_OK)
    stt = launch<fvtp2d_adj_f2_kernel<T>>(tile_grid(d.nx + 5, d.ny + 5, d.nz, kT, kT, kb), sizeof(AdjF2Smem<T>), st,
                                          fx2b, fy2b, qib,
                                          qjb, gxf.origin, gyf.origin, grx.origin, gry.origin, gf1.origin, gg1.origin, d,
                                          kb);
  for (int axis = 0; axis < 2 && stt == OEB_OK; ++axis) {
    const int a = axis ? d.ny : d.nx, l = axis ? d.nx : d.ny;
    stt = launch<fvtp2d_adj_q_kernel<T>>(dim3((a + 6 + 31) / 32, (l + 6 + LN - 1) / LN, d.nz), ps, st, gqb.origin,
                                         gq.origin, gcx.origin, gcy.origin, gar.origin, grx.origin, gry.origin, qib, qjb,
                                         fx2b, fy2b, p1, p2, d, axis);
  }
  scratch_free(buf, st);
  return stt;
}

}  // namespace
}  // namespace oeb

#ifndef OEB_BODIES_ONLY  // the entry points

using namespace oeb;

#define OEB_FV_ENTRY(S, T)                                                                                          \
  extern "C" oeb_status oeb_fvtp2d_##S(                                                                            \
      const oeb_memref3d_##S* q_i, const oeb_memref3d_##S* q_j, const oeb_memref3d_##S* fx1,                        \
      const oeb_memref3d_##S* fx2, const oeb_memref3d_##S* fy1, const oeb_memref3d_##S* fy2,                        \
      const oeb_memref3d_##S* q, const oeb_memref3d_##S* crx, const oeb_memref3d_##S* cry,                          \
      const oeb_memref3d_##S* ra_x, const oeb_memref3d_##S* ra_y, const oeb_memref3d_##S* xfx,                      \
      const oeb_memref3d_##S* yfx, const oeb_memref3d_##S* area, T p1, T p2, const oeb_domain* dom, void* stream) {  \
    return fvtp2d_entry<T>(q_i, q_j, fx1, fx2, fy1, fy2, q, crx, cry, ra_x, ra_y, xfx, yfx, area, p1, p2, dom,       \
                           stream);                                                                                \
  }                                                                                                                \
  extern "C" oeb_status oeb_fvtp2d_tl_##S(                                                                         \
      const oeb_memref3d_##S* dq_i, const oeb_memref3d_##S* dq_j, const oeb_memref3d_##S* dfx1,                     \
      const oeb_memref3d_##S* dfx2, const oeb_memref3d_##S* dfy1, const oeb_memref3d_##S* dfy2,                     \
      const oeb_memref3d_##S* q, const oeb_memref3d_##S* crx, const oeb_memref3d_##S* cry,                          \
      const oeb_memref3d_##S* ra_x, const oeb_memref3d_##S* ra_y, const oeb_memref3d_##S* xfx,                      \
      const oeb_memref3d_##S* yfx, const oeb_memref3d_##S* area, const oeb_memref3d_##S* dq, T p1, T p2,            \
      const oeb_domain* dom, void* stream) {                                                                       \
    return fvtp2d_tl_entry<T>(dq_i, dq_j, dfx1, dfx2, dfy1, dfy2, q, crx, cry, ra_x, ra_y, xfx, yfx, area, dq, p1,  \
                              p2, dom, stream);                                                                    \
  }                                                                                                                \
  extern "C" oeb_status oeb_fvtp2d_adj_##S(                                                                        \
      const oeb_memref3d_##S* qb, const oeb_memref3d_##S* q, const oeb_memref3d_##S* crx,                          \
      const oeb_memref3d_##S* cry, const oeb_memref3d_##S* ra_x, const oeb_memref3d_##S* ra_y,                      \
      const oeb_memref3d_##S* xfx, const oeb_memref3d_##S* yfx, const oeb_memref3d_##S* area,                       \
      const oeb_memref3d_##S* fx1b, const oeb_memref3d_##S* fy1b, T p1, T p2, const oeb_domain* dom,                \
      void* stream) {                                                                                              \
    return fvtp2d_adj_entry<T>(qb, q, crx, cry, ra_x, ra_y, xfx, yfx, area, fx1b, fy1b, p1, p2, dom, stream);      \
  }

OEB_FV_ENTRY(f64, double)
OEB_FV_ENTRY(f32, float)

#endif  // OEB_BODIES_ONLY
