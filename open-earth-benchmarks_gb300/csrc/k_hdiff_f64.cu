// k_hdiff_f64.cu -- FP64 horizontal diffusion stencils whose intermediates are shared by
// neighbouring points: hdiffsa (kernels/hdiffsa.h:95-123) and hdiffsmag
// (kernels/hdiffsmag.h:205-263).
//
// The reference's OpenMP variants recompute each intermediate for every point that uses it
// (three laplacians per point in hdiffsa, three T^2 and three S^2 per point in hdiffsmag).
// On GB300 the FP64 pipe, not HBM, bounds these kernels, so here every intermediate is
// computed once per (i, j, k) into a shared-memory tile (plus a one- or two-cell apron) and
// read by its neighbours.  Reusing a value is exact: it is the same expression on the same
// operands.  Differences are stored once and their negations used where the reference
// subtracts in the other order (x - y == -(y - x) exactly in IEEE round-to-nearest).
//
// Compiled with --fmad=false (see k_pointwise_f64.cu).  One CTA of 32 x 8 threads per
// 32 x 32 tile and KB k-levels.
#include "stencil_util.cuh"

namespace oeb {
namespace {

constexpr int kT = 32;  // tile edge

// ============================== hdiffsa ===========================================
// Shared layout (per k-level), tile origin (i0, j0):
//   in  : 36 x 36, (i0-2+a, j0-2+b)
//   dy  : 34 x 35, (i0-1+a, j0-2+b)   dy(i,j)  = in(i,j+1) - in(i,j)
//   lap : 34 x 34, (i0-1+a, j0-1+b)
//   flx : 33 x 32, (i0-1+a, j0+b)
//   fly : 32 x 33, (i0+a,   j0-1+b)
struct HdiffsaSmem {
  double in[36][36];
  double dy[35][34];
  double lap[34][34];
  double flx[32][33];
  double fly[33][32];
  double crlato[34];  // j0-1+b
  double crlatu[34];
};

__global__ void __launch_bounds__(kThreads) hdiffsa_f64_kernel(double* __restrict__ out,
                                                               const double* __restrict__ in,
                                                               const double* __restrict__ mask,
                                                               const double* __restrict__ crlato,
                                                               const double* __restrict__ crlatu, int64_t s1d,
                                                               Dims d, int kb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HdiffsaSmem& s = *reinterpret_cast<HdiffsaSmem*>(smem_raw);
  const int i0 = blockIdx.x * kT, j0 = blockIdx.y * kT;
  const int sj = (int)d.sj;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  if (tid < 34) {
    const int j = j0 - 1 + tid;
    const bool ok = j >= -1 && j < d.ny + 1;
    s.crlato[tid] = ok ? ld(crlato + (int64_t)j * s1d) : 0.0;
    s.crlatu[tid] = ok ? ld(crlatu + (int64_t)j * s1d) : 0.0;
  }
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, d.nz);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
    const double* pin = in + kofs;
    for_region<36, 36>([&](int a, int b) {
      const int i = i0 - 2 + a, j = j0 - 2 + b;
      const bool ok = i >= -2 && i < d.nx + 2 && j >= -2 && j < d.ny + 2;
      s.in[b][a] = ok ? ld(pin + i + j * sj) : 0.0;
    });
    __syncthreads();
    for_region<34, 35>([&](int a, int b) { s.dy[b][a] = s.in[b + 1][a + 1] - s.in[b][a + 1]; });
    __syncthreads();
    // hdiffsa.h:101: in(i-1)+in(i+1) - 2 in + crlato (in(j+1)-in) + crlatu (in(j-1)-in)
    for_region<34, 34>([&](int a, int b) {
      const double c = s.in[b + 1][a + 1];
      s.lap[b][a] = (((s.in[b + 1][a] + s.in[b + 1][a + 2]) - 2.0 * c) + s.crlato[b] * s.dy[b + 1][a]) +
                    s.crlatu[b] * (-s.dy[b][a]);
    });
    __syncthreads();
    // hdiffsa.h:106-113: limited fluxes
    for_region<33, 32>([&](int a, int b) {
      double f = s.lap[b + 1][a + 1] - s.lap[b + 1][a];
      if (f * (s.in[b + 2][a + 2] - s.in[b + 2][a + 1]) > 0) f = 0;
      s.flx[b][a] = f;
    });
    for_region<32, 33>([&](int a, int b) {
      double f = s.crlato[b] * (s.lap[b + 1][a + 1] - s.lap[b][a + 1]);
      if (f * s.dy[b + 1][a + 1] > 0) f = 0;
      s.fly[b][a] = f;
    });
    __syncthreads();
    // hdiffsa.h:118-119
    for_region<32, 32>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      if (i < d.nx && j < d.ny) {
        const int64_t o = kofs + i + j * sj;
        out[o] = s.in[b + 2][a + 2] + (((s.flx[b][a] - s.flx[b][a + 1]) + s.fly[b][a]) - s.fly[b + 1][a]) * ld(mask + o);
      }
    });
    __syncthreads();
  }
}

// ============================== hdiffsmag =========================================
// Shared layout (per k-level), tile origin (i0, j0):
//   u, v : 34 x 34, (i0-1+a, j0-1+b)
//   dxu  : 33 x 33, (i0-1+a, j0+b)     u(i+1,j) - u(i,j)
//   dyv  : 33 x 33, (i0+a,   j0-1+b)   v(i,j+1) - v(i,j)
//   dyu  : 33 x 33, (i0-1+a, j0-1+b)   u(i,j+1) - u(i,j)
//   dxv  : 33 x 33, (i0-1+a, j0-1+b)   v(i+1,j) - v(i,j)
//   tsq  : 33 x 33, (i0+a,   j0+b)     T_s^2
//   ssq  : 33 x 33, (i0-1+a, j0-1+b)   S_uv^2
struct HdiffsmagSmem {
  double u[34][34];
  double v[34][34];
  double dxu[33][33];
  double dyv[33][33];
  double dyu[33][33];
  double dxv[33][33];
  double tsq[33][33];
  double ssq[33][33];
  double acrlat0[34];  // j0-1+b
  double crlato[32], crlatu[32], crlavo[32], crlavu[32];
};

__global__ void __launch_bounds__(kThreads) hdiffsmag_f64_kernel(
    double* __restrict__ uout, double* __restrict__ vout, const double* __restrict__ uin,
    const double* __restrict__ vin, const double* __restrict__ mask, const double* __restrict__ crlavo,
    const double* __restrict__ crlavu, const double* __restrict__ crlato, const double* __restrict__ crlatu,
    const double* __restrict__ acrlat0, int64_t s1d, double eddlat, double eddlon, double tau_smag,
    double weight_smag, Dims d, int kb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HdiffsmagSmem& s = *reinterpret_cast<HdiffsmagSmem*>(smem_raw);
  const int i0 = blockIdx.x * kT, j0 = blockIdx.y * kT;
  const int sj = (int)d.sj;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  constexpr double rr = earth_radius_recip<double>();
  if (tid < 34) {
    const int j = j0 - 1 + tid;
    s.acrlat0[tid] = (j >= -1 && j < d.ny + 1) ? ld(acrlat0 + (int64_t)j * s1d) : 0.0;
  } else if (tid >= 64 && tid < 96) {
    const int b = tid - 64, j = j0 + b;
    const bool ok = j < d.ny;
    const int64_t jo = (int64_t)j * s1d;
    s.crlato[b] = ok ? ld(crlato + jo) : 0.0;
    s.crlatu[b] = ok ? ld(crlatu + jo) : 0.0;
    s.crlavo[b] = ok ? ld(crlavo + jo) : 0.0;
    s.crlavu[b] = ok ? ld(crlavu + jo) : 0.0;
  }
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, d.nz);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
    for_region<34, 34>([&](int a, int b) {
      const int i = i0 - 1 + a, j = j0 - 1 + b;
      const bool ok = i >= -1 && i < d.nx + 1 && j >= -1 && j < d.ny + 1;
      const int64_t o = kofs + i + j * sj;
      s.u[b][a] = ok ? ld(uin + o) : 0.0;
      s.v[b][a] = ok ? ld(vin + o) : 0.0;
    });
    __syncthreads();
    for_region<33, 33>([&](int a, int b) {
      s.dxu[b][a] = s.u[b + 1][a + 1] - s.u[b + 1][a];
      s.dyv[b][a] = s.v[b + 1][a + 1] - s.v[b][a + 1];
      s.dyu[b][a] = s.u[b + 1][a] - s.u[b][a];
      s.dxv[b][a] = s.v[b][a + 1] - s.v[b][a];
    });
    __syncthreads();
    // hdiffsmag.h:213 T_s = (v(j-1)-v) eddlat R^-1 - (u(i-1)-u) acrlat0(j) eddlon
    //              :221 S_uv = (u(j+1)-u) eddlat R^-1 + (v(i+1)-v) acrlat0(j) eddlon
    for_region<33, 33>([&](int a, int b) {
      const double ts = ((-s.dyv[b][a]) * eddlat) * rr - ((-s.dxu[b][a]) * s.acrlat0[b + 1]) * eddlon;
      s.tsq[b][a] = ts * ts;
      const double su = (s.dyu[b][a] * eddlat) * rr + (s.dxv[b][a] * s.acrlat0[b]) * eddlon;
      s.ssq[b][a] = su * su;
    });
    __syncthreads();
    for_region<32, 32>([&](int a, int b) {
      const int i = i0 + a, j = j0 + b;
      if (i < d.nx && j < d.ny) {
        const int64_t o = kofs + i + j * sj;
        const double hdweight = weight_smag * ld(mask + o);
        // hdiffsmag.h:233-244
        double smag_u = tau_smag * sqrt(0.5 * (s.tsq[b][a + 1] + s.tsq[b][a]) + 0.5 * (s.ssq[b][a + 1] + s.ssq[b + 1][a + 1])) -
                        hdweight;
        smag_u = clamp_smag(smag_u);
        const double uc = s.u[b + 1][a + 1];
        const double lapu = (((s.u[b + 1][a + 2] + s.u[b + 1][a]) - 2.0 * uc) + s.crlato[b] * s.dyu[b + 1][a + 1]) +
                            s.crlatu[b] * (-s.dyu[b][a + 1]);
        uout[o] = uc + smag_u * lapu;
        // hdiffsmag.h:248-259
        double smag_v = tau_smag * sqrt(0.5 * (s.tsq[b + 1][a] + s.tsq[b][a]) + 0.5 * (s.ssq[b + 1][a] + s.ssq[b + 1][a + 1])) -
                        hdweight;
        smag_v = clamp_smag(smag_v);
        const double vc = s.v[b + 1][a + 1];
        const double lapv = (((s.v[b + 1][a + 2] + s.v[b + 1][a]) - 2.0 * vc) + s.crlavo[b] * s.dyv[b + 1][a]) +
                            s.crlavu[b] * (-s.dyv[b][a]);
        vout[o] = vc + smag_v * lapv;
      }
    });
    __syncthreads();
  }
}

constexpr int kKB = 4;

}  // namespace
}  // namespace oeb

using namespace oeb;

extern "C" oeb_status oeb_hdiffsa_f64(const oeb_memref3d_f64* out, const oeb_memref3d_f64* in,
                                      const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlato,
                                      const oeb_memref1d_f64* crlatu, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gout, gin, gmask;
  Line<double> lo, lu;
  OEB_TRY((check_field3<double>(out, *dom, kInterior, &gout)));
  OEB_TRY((check_field3<double>(in, *dom, Reach{2, 2, 2, 2, 0, 0}, &gin)));
  OEB_TRY((check_field3<double>(mask, *dom, kInterior, &gmask)));
  OEB_TRY((check_field1<double>(crlato, *dom, 1, 1, &lo)));
  OEB_TRY((check_field1<double>(crlatu, *dom, 1, 1, &lu)));
  if (lo.s != lu.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<double>({&gout, &gin, &gmask}));
  OEB_TRY(check_no_alias({gout.lo, gout.hi}, {gin.lo, gin.hi, gmask.lo, gmask.hi, lo.lo, lo.hi, lu.lo, lu.hi}));
  OEB_RETURN_IF_VALIDATING();
  const size_t smem = sizeof(HdiffsaSmem);
  OEB_TRY(ensure_dyn_smem((const void*)hdiffsa_f64_kernel, (int)smem));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gin.sj, gin.sk};
  hdiffsa_f64_kernel<<<tile_grid(d.nx, d.ny, d.nz, kT, kT, kKB), dim3(kTX, kTY), smem, (cudaStream_t)stream>>>(
      gout.origin, gin.origin, gmask.origin, lo.origin, lu.origin, lo.s, d, kKB);
  return after_launch();
}

extern "C" oeb_status oeb_hdiffsmag_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                        const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                        const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlavo,
                                        const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato,
                                        const oeb_memref1d_f64* crlatu, const oeb_memref1d_f64* acrlat0,
                                        double eddlat, double eddlon, double tau_smag, double weight_smag,
                                        const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gu, gv, gui, gvi, gm;
  Line<double> lvo, lvu, lto, ltu, la0;
  OEB_TRY((check_field3<double>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<double>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<double>(uin, *dom, Reach{1, 1, 1, 1, 0, 0}, &gui)));
  OEB_TRY((check_field3<double>(vin, *dom, Reach{1, 1, 1, 1, 0, 0}, &gvi)));
  OEB_TRY((check_field3<double>(mask, *dom, kInterior, &gm)));
  OEB_TRY((check_field1<double>(crlavo, *dom, 0, 0, &lvo)));
  OEB_TRY((check_field1<double>(crlavu, *dom, 0, 0, &lvu)));
  OEB_TRY((check_field1<double>(crlato, *dom, 0, 0, &lto)));
  OEB_TRY((check_field1<double>(crlatu, *dom, 0, 0, &ltu)));
  OEB_TRY((check_field1<double>(acrlat0, *dom, 1, 1, &la0)));
  if (lvu.s != lvo.s || lto.s != lvo.s || ltu.s != lvo.s || la0.s != lvo.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<double>({&gu, &gv, &gui, &gvi, &gm}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi},
                         {gui.lo, gui.hi, gvi.lo, gvi.hi, gm.lo, gm.hi, lvo.lo, lvo.hi, lvu.lo, lvu.hi, lto.lo,
                          lto.hi, ltu.lo, ltu.hi, la0.lo, la0.hi}));
  OEB_RETURN_IF_VALIDATING();
  const size_t smem = sizeof(HdiffsmagSmem);
  OEB_TRY(ensure_dyn_smem((const void*)hdiffsmag_f64_kernel, (int)smem));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
  hdiffsmag_f64_kernel<<<tile_grid(d.nx, d.ny, d.nz, kT, kT, kKB), dim3(kTX, kTY), smem, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, gm.origin, lvo.origin, lvu.origin, lto.origin, ltu.origin,
      la0.origin, lvo.s, eddlat, eddlon, tau_smag, weight_smag, d, kKB);
  return after_launch();
}
