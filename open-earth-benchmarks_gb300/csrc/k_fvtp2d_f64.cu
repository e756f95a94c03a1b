// k_fvtp2d_f64.cu -- FP64 fvtp2d (kernels/fvtp2d.h:4-177, the serial variant).
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
// Compiled with --fmad=false (see k_pointwise_f64.cu).
#include "oeb_reach.cuh"
#include "stencil_util.cuh"

namespace oeb {
namespace {

constexpr int kT = 32;

// PPM edge value al(j) = p1 (q(j-1) + q(j)) + p2 (q(j-2) + q(j+1))   (fvtp2d.h:12)
__device__ __forceinline__ double ppm_al(double p1, double p2, double qm2, double qm1, double q0, double qp1) {
  return (p1 * (qm1 + q0)) + (p2 * (qm2 + qp1));
}

struct PpmAux {
  double almq, br, b0;
  unsigned char smt5;
};

// fvtp2d.h:20-23: almq = al - q, br = al(+1) - q, b0 = almq + br, smt5 = almq*br < 0
__device__ __forceinline__ void ppm_aux(double al0, double al1, double q0, double* almq, double* br, double* b0,
                                        unsigned char* smt) {
  const double m = al0 - q0;
  const double r = al1 - q0;
  *almq = m;
  *br = r;
  *b0 = m + r;
  *smt = (m * r) < 0.0;
}

// fvtp2d.h:28-34: upwind flux at point j from the aux values at j-1 and j.  The flag sum
// smt5(j-1) + smt5(j)*(smt5(j-1)==0) is exactly 1.0 when either flag is set, else 0.0.
__device__ __forceinline__ double ppm_flux(double c, double q_m1, double q_0, double br_m1, double b0_m1,
                                           double almq_0, double b0_0, unsigned char smt_m1, unsigned char smt_0) {
  const double smt = (smt_m1 | smt_0) ? 1.0 : 0.0;
  if (c > 0.) {
    const double t = (1. - c) * (br_m1 - (c * b0_m1));
    return q_m1 + (t * smt);
  } else {
    const double t = (1. + c) * (almq_0 + (c * b0_0));
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
struct FvQSmem {
  double q[39][38];
  union {
    struct {
      double al[35][32];
      double almq[34][32], br[34][32], b0[34][32];
      unsigned char smt[34][32];
    } y;
    struct {
      double al[32][35];
      double almq[32][34], br[32][34], b0[32][34];
      unsigned char smt[32][34];
    } x;
  } w;
  double fyy[33][32];
  double fxx[32][33];
};

__global__ void __launch_bounds__(kThreads) fvtp2d_q_f64_kernel(
    double* __restrict__ q_i, double* __restrict__ q_j, double* __restrict__ fx2, double* __restrict__ fy2,
    const double* __restrict__ q, const double* __restrict__ crx, const double* __restrict__ cry,
    const double* __restrict__ ra_x, const double* __restrict__ ra_y, const double* __restrict__ xfx,
    const double* __restrict__ yfx, const double* __restrict__ area, double p1, double p2, Dims d, int kb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FvQSmem& s = *reinterpret_cast<FvQSmem*>(smem_raw);
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
      s.q[b][a] = ok ? ld(q + kofs + i + j * sj) : 0.0;
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
      double fyy = 0.0;
      if (i >= -3 && i < nx + 2 && j >= 0 && j < ny + 1) {  // fvtp2d.h:26-27
        const int64_t o = kofs + i + j * sj;
        const double f = ppm_flux(ld(cry + o), s.q[b + 2][a + 3], s.q[b + 3][a + 3], s.w.y.br[b][a], s.w.y.b0[b][a],
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
      double fxx = 0.0;
      if (i >= 0 && i < nx + 1 && j >= -3 && j < ny + 2) {  // fvtp2d.h:102-103
        const int64_t o = kofs + i + j * sj;
        const double f = ppm_flux(ld(crx + o), s.q[b + 3][a + 2], s.q[b + 3][a + 3], s.w.x.br[b][a], s.w.x.b0[b][a],
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
      const double qc = s.q[b + 3][a + 3];
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
struct FvFluxSmem {
  double qi[32][37];
  double qj[37][32];
  union {
    struct {
      double al[32][34];
      double almq[32][33], br[32][33], b0[32][33];
      unsigned char smt[32][33];
    } x;
    struct {
      double al[34][32];
      double almq[33][32], br[33][32], b0[33][32];
      unsigned char smt[33][32];
    } y;
  } w;
};

__global__ void __launch_bounds__(kThreads) fvtp2d_flux_f64_kernel(
    double* __restrict__ fx1, double* __restrict__ fy1, const double* __restrict__ q_i,
    const double* __restrict__ q_j, const double* __restrict__ fx2, const double* __restrict__ fy2,
    const double* __restrict__ crx, const double* __restrict__ cry, const double* __restrict__ xfx,
    const double* __restrict__ yfx, double p1, double p2, Dims d, int kb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FvFluxSmem& s = *reinterpret_cast<FvFluxSmem*>(smem_raw);
  const int i0 = blockIdx.x * kT, j0 = blockIdx.y * kT;
  const int sj = (int)d.sj;
  const int nx = d.nx, ny = d.ny;
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, d.nz);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
    for_region<37, 32>([&](int a, int b) {
      const int i = i0 - 3 + a, j = j0 + b;
      s.qi[b][a] = (i < nx + 2 && j < ny) ? ld(q_i + kofs + i + j * sj) : 0.0;
    });
    for_region<32, 37>([&](int a, int b) {
      const int i = i0 + a, j = j0 - 3 + b;
      s.qj[b][a] = (i < nx && j < ny + 2) ? ld(q_j + kofs + i + j * sj) : 0.0;
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
        const double f = ppm_flux(ld(crx + o), s.qi[b][a + 2], s.qi[b][a + 3], s.w.x.br[b][a], s.w.x.b0[b][a],
                                  s.w.x.almq[b][a + 1], s.w.x.b0[b][a + 1], s.w.x.smt[b][a], s.w.x.smt[b][a + 1]);
        fx1[o] = ((0.5 * (f + ld(fx2 + o))) * ld(xfx + o));  // fvtp2d.h:164
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
        const double f = ppm_flux(ld(cry + o), s.qj[b + 2][a], s.qj[b + 3][a], s.w.y.br[b][a], s.w.y.b0[b][a],
                                  s.w.y.almq[b + 1][a], s.w.y.b0[b + 1][a], s.w.y.smt[b][a], s.w.y.smt[b + 1][a]);
        fy1[o] = ((0.5 * (f + ld(fy2 + o))) * ld(yfx + o));  // fvtp2d.h:173
      }
    });
    __syncthreads();
  }
}

constexpr int kKB = 4;

}  // namespace
}  // namespace oeb

using namespace oeb;

extern "C" oeb_status oeb_fvtp2d_f64(const oeb_memref3d_f64* q_i, const oeb_memref3d_f64* q_j,
                                     const oeb_memref3d_f64* fx1, const oeb_memref3d_f64* fx2,
                                     const oeb_memref3d_f64* fy1, const oeb_memref3d_f64* fy2,
                                     const oeb_memref3d_f64* q, const oeb_memref3d_f64* crx,
                                     const oeb_memref3d_f64* cry, const oeb_memref3d_f64* ra_x,
                                     const oeb_memref3d_f64* ra_y, const oeb_memref3d_f64* xfx,
                                     const oeb_memref3d_f64* yfx, const oeb_memref3d_f64* area, double p1, double p2,
                                     const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gqi, gqj, gfx1, gfx2, gfy1, gfy2, gq, gcx, gcy, grx, gry, gxf, gyf, gar;
  const Reach rx_ext = kFvFx2;  // fx2 written, crx and xfx read: i in [0,N], j in [-3,N+1]
  const Reach ry_ext = kFvFy2;  // fy2 written, cry and yfx read: i in [-3,N+1], j in [0,N]
  OEB_TRY((check_field3<double>(q_i, *dom, kFvQi, &gqi)));
  OEB_TRY((check_field3<double>(q_j, *dom, kFvQj, &gqj)));
  OEB_TRY((check_field3<double>(fx1, *dom, kInterior, &gfx1)));
  OEB_TRY((check_field3<double>(fx2, *dom, rx_ext, &gfx2)));
  OEB_TRY((check_field3<double>(fy1, *dom, kInterior, &gfy1)));
  OEB_TRY((check_field3<double>(fy2, *dom, ry_ext, &gfy2)));
  OEB_TRY((check_field3<double>(q, *dom, Reach{3, 3, 3, 3, 0, 0}, &gq)));
  OEB_TRY((check_field3<double>(crx, *dom, rx_ext, &gcx)));
  OEB_TRY((check_field3<double>(cry, *dom, ry_ext, &gcy)));
  OEB_TRY((check_field3<double>(ra_x, *dom, Reach{0, 0, 3, 2, 0, 0}, &grx)));
  OEB_TRY((check_field3<double>(ra_y, *dom, Reach{3, 2, 0, 0, 0, 0}, &gry)));
  OEB_TRY((check_field3<double>(xfx, *dom, rx_ext, &gxf)));
  OEB_TRY((check_field3<double>(yfx, *dom, ry_ext, &gyf)));
  OEB_TRY((check_field3<double>(area, *dom, Reach{3, 2, 3, 2, 0, 0}, &gar)));
  OEB_TRY(check_same_strides<double>({&gqi, &gqj, &gfx1, &gfx2, &gfy1, &gfy2, &gq, &gcx, &gcy, &grx, &gry, &gxf,
                                      &gyf, &gar}));
  OEB_TRY(check_no_alias({gqi.lo, gqi.hi, gqj.lo, gqj.hi, gfx1.lo, gfx1.hi, gfx2.lo, gfx2.hi, gfy1.lo, gfy1.hi,
                          gfy2.lo, gfy2.hi},
                         {gq.lo, gq.hi, gcx.lo, gcx.hi, gcy.lo, gcy.hi, grx.lo, grx.hi, gry.lo, gry.hi, gxf.lo,
                          gxf.hi, gyf.lo, gyf.hi, gar.lo, gar.hi}));
  OEB_RETURN_IF_VALIDATING();
  OEB_TRY(ensure_dyn_smem((const void*)fvtp2d_q_f64_kernel, (int)sizeof(FvQSmem)));
  OEB_TRY(ensure_dyn_smem((const void*)fvtp2d_flux_f64_kernel, (int)sizeof(FvFluxSmem)));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gq.sj, gq.sk};
  cudaStream_t st = (cudaStream_t)stream;
  fvtp2d_q_f64_kernel<<<tile_grid(d.nx + 5, d.ny + 5, d.nz, kT, kT, kKB), dim3(kTX, kTY), sizeof(FvQSmem), st>>>(
      gqi.origin, gqj.origin, gfx2.origin, gfy2.origin, gq.origin, gcx.origin, gcy.origin, grx.origin, gry.origin,
      gxf.origin, gyf.origin, gar.origin, p1, p2, d, kKB);
  OEB_TRY(after_launch());
  fvtp2d_flux_f64_kernel<<<tile_grid(d.nx, d.ny, d.nz, kT, kT, kKB), dim3(kTX, kTY), sizeof(FvFluxSmem), st>>>(
      gfx1.origin, gfy1.origin, gqi.origin, gqj.origin, gfx2.origin, gfy2.origin, gcx.origin, gcy.origin, gxf.origin,
      gyf.origin, p1, p2, d, kKB);
  return after_launch();
}
