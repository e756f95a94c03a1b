// k_fvtp2d.cu -- fvtp2d (kernels/fvtp2d.h:4-177, the serial variant) in FP64 and FP32.
//
// Two launches per call, per k-level tiles of 32 x 32 with every PPM intermediate computed
// once per point into shared memory:
//   1. fvtp2d_q:    y-PPM of q -> fy2 (fvtp2d.h:8-37), x-PPM of q -> fx2 (:84-113), then
//                   q_i (:39-51) and q_j (:115-127).  Tiles cover the extended index range
//                   [-3, N+2) of these arrays; each value is written exactly where the
//                   reference writes it (fy2, q_i: i in [-3,N+2); fx2, q_j: j in [-3,N+2)).
//   2. fvtp2d_flux: x-PPM of q_i -> fx1 (:53-82), y-PPM of q_j -> fy1 (:129-158) and the
//                   transport fluxes fx1 = (fx1+fx2)/2 * xfx, fy1 = (fy1+fy2)/2 * yfx (:160-176).
// q_i, q_j, fx2 and fy2 are outputs of the reference signature; launch 2 reads them back
// from global memory (the FP64 pipe, not HBM, bounds this kernel, so storing them costs
// less than recomputing their aprons).
//
// Compiled with --fmad=false (see k_pointwise.cu).  In FP32 the monotonicity flag smt5 is decided
// on the exact product (precision.cuh).
#include "oeb_reach.cuh"
#include "precision.cuh"
#include "stencil_util.cuh"

namespace oeb {
namespace {

constexpr int kT = 32;

// PPM edge value al(j) = p1 (q(j-1) + q(j)) + p2 (q(j-2) + q(j+1))   (fvtp2d.h:12)
template <class T>
__device__ __forceinline__ T ppm_al(T p1, T p2, T qm2, T qm1, T q0, T qp1) {
  return (p1 * (qm1 + q0)) + (p2 * (qm2 + qp1));
}

// fvtp2d.h:20-23: almq = al - q, br = al(+1) - q, b0 = almq + br, smt5 = almq*br < 0
template <class T>
__device__ __forceinline__ void ppm_aux(T al0, T al1, T q0, T* almq, T* br, T* b0, unsigned char* smt) {
  const T m = al0 - q0;
  const T r = al1 - q0;
  *almq = m;
  *br = r;
  *b0 = m + r;
  *smt = Prec<T>::prod_lt0(m, r);
}

// fvtp2d.h:28-34: upwind flux at point j from the aux values at j-1 and j.  The flag sum
// smt5(j-1) + smt5(j)*(smt5(j-1)==0) is exactly 1.0 when either flag is set, else 0.0.
template <class T>
__device__ __forceinline__ T ppm_flux(T c, T q_m1, T q_0, T br_m1, T b0_m1, T almq_0, T b0_0, unsigned char smt_m1,
                                      unsigned char smt_0) {
  const T smt = (smt_m1 | smt_0) ? T(1.0) : T(0.0);
  if (c > T(0.)) {
    const T t = (T(1.) - c) * (br_m1 - (c * b0_m1));
    return q_m1 + (t * smt);
  } else {
    const T t = (T(1.) + c) * (almq_0 + (c * b0_0));
    return q_0 + (t * smt);
  }
}

// ------------------------------ launch 1 ---------------------------------------------
// Tile origin (i0, j0) = (-3 + 32 bx, -3 + 32 by).  Shared layout:
//   q    : 38 x 39, (i0-3+a, j0-3+b)
//   y pass: al 32 x 35 (i0+a, j0-1+b); almq/br/b0/smt 32 x 34 (i0+a, j0-1+b)
//   x pass: al 35 x 32 (i0-1+a, j0+b); almq/br/b0/smt 34 x 32 (i0-1+a, j0+b)
//   fyy  : 32 x 33 (i0+a, j0+b) = yfx * fy2, 0 outside fy2's range
//   fxx  : 33 x 32 (i0+a, j0+b) = xfx * fx2, 0 outside fx2's range
template <class T>
struct FvQSmem {
  T q[39][38];
  union {
    struct {
      T al[35][32];
      T almq[34][32], br[34][32], b0[34][32];
      unsigned char smt[34][32];
    } y;
    struct {
      T al[32][35];
      T almq[32][34], br[32][34], b0[32][34];
      unsigned char smt[32][34];
    } x;
  } w;
  T fyy[33][32];
  T fxx[32][33];
};

template <class T>
__global__ void __launch_bounds__(kThreads) fvtp2d_q_kernel(T* __restrict__ q_i, T* __restrict__ q_j,
                                                            T* __restrict__ fx2, T* __restrict__ fy2,
                                                            const T* __restrict__ q, const T* __restrict__ crx,
                                                            const T* __restrict__ cry, const T* __restrict__ ra_x,
                                                            const T* __restrict__ ra_y, const T* __restrict__ xfx,
                                                            const T* __restrict__ yfx, const T* __restrict__ area,
                                                            T p1, T p2, Dims d, int kb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FvQSmem<T>& s = *reinterpret_cast<FvQSmem<T>*>(smem_raw);
  const int i0 = -3 + (int)blockIdx.x * kT, j0 = -3 + (int)blockIdx.y * kT;
  const int sj = (int)d.sj;
  const int nx = d.nx, ny = d.ny;
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, d.nz);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
    for_region<38, 39>([&](int a, int b) {
      const int i = i0 - 3 + a, j = j0 - 3 + b;
      const bool ok = i >= -3 && i < nx + 3 && j >= -3 && j < ny + 3;
      s.q[b][a] = ok ? ld(q + kofs + i + j * sj) : T(0);
    });
    __syncthreads();
    // ---- y-PPM of q -> fy2, fyy
    for_region<32, 35>([&](int a, int b) {
      s.w.y.al[b][a] = ppm_al(p1, p2, s.q[b][a + 3], s.q[b + 1][a + 3], s.q[b + 2][a + 3], s.q[b + 3][a + 3]);
    });
    __syncthreads();
    for_region<32, 34>([&](int a, int b) {
      ppm_aux(s.w.y.al[b][a], s.w.y.al[b + 1][a], s.q[b + 2][a + 3], &s.w.y.almq[b][a], &s.w.y.br[b][a],
              &s.w.y.b0[b][a], &s.w.y.smt[b][a]);
    });
    __syncthreads();
    for_region<32, 33>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      T fyy = T(0);
      if (i >= -3 && i < nx + 2 && j >= 0 && j < ny + 1) {  // fvtp2d.h:26-27
        const int64_t o = kofs + i + j * sj;
        const T f = ppm_flux(ld(cry + o), s.q[b + 2][a + 3], s.q[b + 3][a + 3], s.w.y.br[b][a], s.w.y.b0[b][a],
                                  s.w.y.almq[b + 1][a], s.w.y.b0[b + 1][a], s.w.y.smt[b][a], s.w.y.smt[b + 1][a]);
        if (b < kT) fy2[o] = f;
        fyy = ld(yfx + o) * f;  // fvtp2d.h:43
      }
      s.fyy[b][a] = fyy;
    });
    __syncthreads();
    // ---- x-PPM of q -> fx2, fxx
    for_region<35, 32>([&](int a, int b) {
      s.w.x.al[b][a] = ppm_al(p1, p2, s.q[b + 3][a], s.q[b + 3][a + 1], s.q[b + 3][a + 2], s.q[b + 3][a + 3]);
    });
    __syncthreads();
    for_region<34, 32>([&](int a, int b) {
      ppm_aux(s.w.x.al[b][a], s.w.x.al[b][a + 1], s.q[b + 3][a + 2], &s.w.x.almq[b][a], &s.w.x.br[b][a],
              &s.w.x.b0[b][a], &s.w.x.smt[b][a]);
    });
    __syncthreads();
    for_region<33, 32>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      T fxx = T(0);
      if (i >= 0 && i < nx + 1 && j >= -3 && j < ny + 2) {  // fvtp2d.h:102-103
        const int64_t o = kofs + i + j * sj;
        const T f = ppm_flux(ld(crx + o), s.q[b + 3][a + 2], s.q[b + 3][a + 3], s.w.x.br[b][a], s.w.x.b0[b][a],
                                  s.w.x.almq[b][a + 1], s.w.x.b0[b][a + 1], s.w.x.smt[b][a], s.w.x.smt[b][a + 1]);
        if (a < kT) fx2[o] = f;
        fxx = ld(xfx + o) * f;  // fvtp2d.h:119
      }
      s.fxx[b][a] = fxx;
    });
    __syncthreads();
    // ---- q_i (fvtp2d.h:48) and q_j (fvtp2d.h:124)
    for_region<32, 32>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      const int64_t o = kofs + i + j * sj;
      const T qc = s.q[b + 3][a + 3];
      if (i >= -3 && i < nx + 2 && j >= 0 && j < ny) {
        q_i[o] = (((qc * ld(area + o)) + s.fyy[b][a]) - s.fyy[b + 1][a]) / ld(ra_y + o);
      }
      if (i >= 0 && i < nx && j >= -3 && j < ny + 2) {
        q_j[o] = (((qc * ld(area + o)) + s.fxx[b][a]) - s.fxx[b][a + 1]) / ld(ra_x + o);
      }
    });
    __syncthreads();
  }
}

// ------------------------------ launch 2 ---------------------------------------------
// Interior tile origin (i0, j0).  Shared layout:
//   qi : 37 x 32, (i0-3+a, j0+b)      qj : 32 x 37, (i0+a, j0-3+b)
//   x pass: al 34 x 32 (i0-1+a, j0+b); almq/br/b0/smt 33 x 32 (i0-1+a, j0+b)
//   y pass: al 32 x 34 (i0+a, j0-1+b); almq/br/b0/smt 32 x 33 (i0+a, j0-1+b)
template <class T>
struct FvFluxSmem {
  T qi[32][37];
  T qj[37][32];
  union {
    struct {
      T al[32][34];
      T almq[32][33], br[32][33], b0[32][33];
      unsigned char smt[32][33];
    } x;
    struct {
      T al[34][32];
      T almq[33][32], br[33][32], b0[33][32];
      unsigned char smt[33][32];
    } y;
  } w;
};

template <class T>
__global__ void __launch_bounds__(kThreads) fvtp2d_flux_kernel(T* __restrict__ fx1, T* __restrict__ fy1,
                                                               const T* __restrict__ q_i, const T* __restrict__ q_j,
                                                               const T* __restrict__ fx2, const T* __restrict__ fy2,
                                                               const T* __restrict__ crx, const T* __restrict__ cry,
                                                               const T* __restrict__ xfx, const T* __restrict__ yfx,
                                                               T p1, T p2, Dims d, int kb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FvFluxSmem<T>& s = *reinterpret_cast<FvFluxSmem<T>*>(smem_raw);
  const int i0 = blockIdx.x * kT, j0 = blockIdx.y * kT;
  const int sj = (int)d.sj;
  const int nx = d.nx, ny = d.ny;
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, d.nz);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
    for_region<37, 32>([&](int a, int b) {
      const int i = i0 - 3 + a, j = j0 + b;
      s.qi[b][a] = (i < nx + 2 && j < ny) ? ld(q_i + kofs + i + j * sj) : T(0);
    });
    for_region<32, 37>([&](int a, int b) {
      const int i = i0 + a, j = j0 - 3 + b;
      s.qj[b][a] = (i < nx && j < ny + 2) ? ld(q_j + kofs + i + j * sj) : T(0);
    });
    __syncthreads();
    // ---- x-PPM of q_i -> fx1 and the x transport flux
    for_region<34, 32>([&](int a, int b) {
      s.w.x.al[b][a] = ppm_al(p1, p2, s.qi[b][a], s.qi[b][a + 1], s.qi[b][a + 2], s.qi[b][a + 3]);
    });
    __syncthreads();
    for_region<33, 32>([&](int a, int b) {
      ppm_aux(s.w.x.al[b][a], s.w.x.al[b][a + 1], s.qi[b][a + 2], &s.w.x.almq[b][a], &s.w.x.br[b][a],
              &s.w.x.b0[b][a], &s.w.x.smt[b][a]);
    });
    __syncthreads();
    for_region<32, 32>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      if (i < nx && j < ny) {
        const int64_t o = kofs + i + j * sj;
        const T f = ppm_flux(ld(crx + o), s.qi[b][a + 2], s.qi[b][a + 3], s.w.x.br[b][a], s.w.x.b0[b][a],
                                  s.w.x.almq[b][a + 1], s.w.x.b0[b][a + 1], s.w.x.smt[b][a], s.w.x.smt[b][a + 1]);
        fx1[o] = ((T(0.5) * (f + ld(fx2 + o))) * ld(xfx + o));  // fvtp2d.h:164
      }
    });
    __syncthreads();
    // ---- y-PPM of q_j -> fy1 and the y transport flux
    for_region<32, 34>([&](int a, int b) {
      s.w.y.al[b][a] = ppm_al(p1, p2, s.qj[b][a], s.qj[b + 1][a], s.qj[b + 2][a], s.qj[b + 3][a]);
    });
    __syncthreads();
    for_region<32, 33>([&](int a, int b) {
      ppm_aux(s.w.y.al[b][a], s.w.y.al[b + 1][a], s.qj[b + 2][a], &s.w.y.almq[b][a], &s.w.y.br[b][a],
              &s.w.y.b0[b][a], &s.w.y.smt[b][a]);
    });
    __syncthreads();
    for_region<32, 32>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      if (i < nx && j < ny) {
        const int64_t o = kofs + i + j * sj;
        const T f = ppm_flux(ld(cry + o), s.qj[b + 2][a], s.qj[b + 3][a], s.w.y.br[b][a], s.w.y.b0[b][a],
                                  s.w.y.almq[b + 1][a], s.w.y.b0[b + 1][a], s.w.y.smt[b][a], s.w.y.smt[b + 1][a]);
        fy1[o] = ((T(0.5) * (f + ld(fy2 + o))) * ld(yfx + o));  // fvtp2d.h:173
      }
    });
    __syncthreads();
  }
}

constexpr int kKB = 4;

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
  OEB_TRY(ensure_dyn_smem((const void*)fvtp2d_q_kernel<T>, (int)sizeof(FvQSmem<T>)));
  OEB_TRY(ensure_dyn_smem((const void*)fvtp2d_flux_kernel<T>, (int)sizeof(FvFluxSmem<T>)));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gq.sj, gq.sk};
  cudaStream_t st = (cudaStream_t)stream;
  fvtp2d_q_kernel<T><<<tile_grid(d.nx + 5, d.ny + 5, d.nz, kT, kT, kKB), dim3(kTX, kTY), sizeof(FvQSmem<T>), st>>>(
      gqi.origin, gqj.origin, gfx2.origin, gfy2.origin, gq.origin, gcx.origin, gcy.origin, grx.origin, gry.origin,
      gxf.origin, gyf.origin, gar.origin, p1, p2, d, kKB);
  OEB_TRY(after_launch());
  fvtp2d_flux_kernel<T><<<tile_grid(d.nx, d.ny, d.nz, kT, kT, kKB), dim3(kTX, kTY), sizeof(FvFluxSmem<T>), st>>>(
      gfx1.origin, gfy1.origin, gqi.origin, gqj.origin, gfx2.origin, gfy2.origin, gcx.origin, gcy.origin, gxf.origin,
      gyf.origin, p1, p2, d, kKB);
  return after_launch();
}

}  // namespace
}  // namespace oeb

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
  }

OEB_FV_ENTRY(f64, double)
OEB_FV_ENTRY(f32, float)
