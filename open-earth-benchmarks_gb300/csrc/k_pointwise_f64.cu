// k_pointwise_f64.cu -- FP64 stencils whose intermediates are used only at their own point:
// laplace, uvbke, p_grad_c, nh_p_grad, hadvuv and hadvuv5th.
//
// Compiled with --fmad=false: every a*b+c is rounded twice, exactly as the reference
// compiled without FP contraction, and double division and square root are IEEE
// round-to-nearest on both sides, so the results are bit-identical to the reference
// OpenMP kernels.  Expression trees keep the reference's order and parenthesisation; a
// subexpression that occurs twice in the reference is computed once here (same operands,
// same value).
//
// One CTA of 32 x 8 threads covers a 32 x 32 (i, j) tile and KB k-levels; each thread
// computes 4 rows.  Neighbour reads go through L1.
#include "stencil_util.cuh"

namespace oeb {
namespace {

constexpr int kTI = 32, kTJ = 32, kRows = kTJ / kTY;

// Visits the points of this thread: f(o, j) with o the in-plane offset of (i, j) plus the
// plane offset of k.
template <class F>
__device__ __forceinline__ void for_points(const Dims& d, int kb, F&& f) {
  const int i = blockIdx.x * kTI + threadIdx.x;
  if (i >= d.nx) return;
  const int k0 = blockIdx.z * kb;
  const int k1 = min(k0 + kb, d.nz);
  const int sj = (int)d.sj;
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      const int j = blockIdx.y * kTJ + threadIdx.y + kTY * r;
      if (j < d.ny) f(kofs + i + j * sj, j);
    }
  }
}

// ---- laplace: kernels/laplace.h:34-43 ----------------------------------------------
__global__ void __launch_bounds__(kThreads) laplace_f64_kernel(const double* __restrict__ in,
                                                               double* __restrict__ out, Dims d, int kb) {
  const int64_t sj = d.sj;
  for_points(d, kb, [&](int64_t o, int) {
    out[o] = -4.0 * ld(in + o) + ((ld(in + o - 1) + ld(in + o + 1)) + (ld(in + o + sj) + ld(in + o - sj)));
  });
}

// ---- uvbke: kernels/uvbke.h:61-75 ----------------------------------------------------
__global__ void __launch_bounds__(kThreads) uvbke_f64_kernel(double* __restrict__ ub, double* __restrict__ vb,
                                                             const double* __restrict__ uc,
                                                             const double* __restrict__ vc,
                                                             const double* __restrict__ cosa,
                                                             const double* __restrict__ rsina, double dt5, Dims d,
                                                             int kb) {
  const int64_t sj = d.sj;
  for_points(d, kb, [&](int64_t o, int) {
    const double su = ld(uc + o - sj) + ld(uc + o);
    const double sv = ld(vc + o - 1) + ld(vc + o);
    const double ca = ld(cosa + o);
    const double rs = ld(rsina + o);
    ub[o] = ((dt5 * (su - (sv * ca))) * rs);
    vb[o] = ((dt5 * (sv - (su * ca))) * rs);
  });
}

// ---- p_grad_c: kernels/p_grad_c.h:80-101 ---------------------------------------------
__global__ void __launch_bounds__(kThreads) p_grad_c_f64_kernel(
    double* __restrict__ uout, double* __restrict__ vout, const double* __restrict__ uin,
    const double* __restrict__ vin, const double* __restrict__ rdxc, const double* __restrict__ rdyc,
    const double* __restrict__ delpc, const double* __restrict__ gz, const double* __restrict__ pkc, double dt2,
    Dims d, int kb) {
  const int64_t sj = d.sj, sk = d.sk;
  for_points(d, kb, [&](int64_t o, int) {
    const double wk = ld(delpc + o);
    const double gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pkc + o), pk1 = ld(pkc + o + sk);
    uout[o] = (ld(uin + o) + (((dt2 * ld(rdxc + o)) / (ld(delpc + o - 1) + wk)) *
                              (((ld(gz + o - 1 + sk) - gz0) * (pk1 - ld(pkc + o - 1))) +
                               ((ld(gz + o - 1) - gz1) * (ld(pkc + o - 1 + sk) - pk0)))));
    vout[o] = (ld(vin + o) + (((dt2 * ld(rdyc + o)) / (ld(delpc + o - sj) + wk)) *
                              (((ld(gz + o - sj + sk) - gz0) * (pk1 - ld(pkc + o - sj))) +
                               ((ld(gz + o - sj) - gz1) * (ld(pkc + o - sj + sk) - pk0)))));
  });
}

// ---- nh_p_grad: kernels/nh_p_grad.h:116-146 --------------------------------------------
__global__ void __launch_bounds__(kThreads) nh_p_grad_f64_kernel(
    double* __restrict__ uout, double* __restrict__ vout, const double* __restrict__ uin,
    const double* __restrict__ vin, const double* __restrict__ rdx, const double* __restrict__ rdy,
    const double* __restrict__ gz, const double* __restrict__ pp, const double* __restrict__ pk3,
    const double* __restrict__ wk1, double dt, Dims d, int kb) {
  const int64_t sj = d.sj, sk = d.sk;
  for_points(d, kb, [&](int64_t o, int) {
    const double pk0 = ld(pk3 + o), pk1 = ld(pk3 + o + sk);
    const double gz0 = ld(gz + o), gz1 = ld(gz + o + sk);
    const double pp0 = ld(pp + o), pp1 = ld(pp + o + sk);
    const double w1 = ld(wk1 + o);
    const double wk = pk1 - pk0;
    // u: neighbour i+1
    {
      const double pkx0 = ld(pk3 + o + 1), pkx1 = ld(pk3 + o + 1 + sk);
      const double wkx = pkx1 - pkx0;
      const double ga = gz1 - ld(gz + o + 1);
      const double gb = gz0 - ld(gz + o + 1 + sk);
      const double du = ((dt / (wk + wkx)) * ((ga * (pkx1 - pk0)) + (gb * (pk1 - pkx0))));
      uout[o] = (((ld(uin + o) + du) +
                  ((dt / (w1 + ld(wk1 + o + 1))) * ((ga * (ld(pp + o + 1 + sk) - pp0)) + (gb * (pp1 - ld(pp + o + 1)))))) *
                 ld(rdx + o));
    }
    // v: neighbour j+1
    {
      const double pky0 = ld(pk3 + o + sj), pky1 = ld(pk3 + o + sj + sk);
      const double wky = pky1 - pky0;
      const double ga = gz1 - ld(gz + o + sj);
      const double gb = gz0 - ld(gz + o + sj + sk);
      const double dv = ((dt / (wk + wky)) * ((ga * (pky1 - pk0)) + (gb * (pk1 - pky0))));
      vout[o] = (((ld(vin + o) + dv) +
                  ((dt / (w1 + ld(wk1 + o + sj))) *
                   ((ga * (ld(pp + o + sj + sk) - pp0)) + (gb * (pp1 - ld(pp + o + sj)))))) *
                 ld(rdy + o));
    }
  });
}

// ---- hadvuv / hadvuv5th: kernels/hadvuv.h:4-27,178-210 and kernels/hadvuv5th.h:4-39,177-201

// 3rd-order upwind advection along one axis (stride s): hadvuv.h:10-16 (x) and :18-24 (y).
__device__ __forceinline__ double adv3_axis(const double* __restrict__ f, int64_t o, int64_t s, double a) {
  constexpr double c6 = -1.0 / 6.0, c3 = -1.0 / 3.0, ch = -0.5;
  if (a > 0) {
    return a * (((c6 * ld(f + o - 2 * s) + ld(f + o - s)) + ch * ld(f + o)) + c3 * ld(f + o + s));
  } else {
    return -a * (((c3 * ld(f + o - s) + ch * ld(f + o)) + ld(f + o + s)) + c6 * ld(f + o + 2 * s));
  }
}

// 5th-order upwind advection along one axis: hadvuv5th.h:10-22 (x) and :24-36 (y).
__device__ __forceinline__ double adv5_axis(const double* __restrict__ f, int64_t o, int64_t s, double a) {
  constexpr double c30 = 1.0 / 30.0, c4 = -1.0 / 4.0, c3 = -1.0 / 3.0, c2 = -1.0 / 2.0, c20 = 1.0 / 20.0;
  if (a > 0) {
    return a * (((((c30 * ld(f + o - 3 * s) + c4 * ld(f + o - 2 * s)) + ld(f + o - s)) + c3 * ld(f + o)) +
                 c2 * ld(f + o + s)) +
                c20 * ld(f + o + 2 * s));
  } else {
    return -a * (((((c20 * ld(f + o - 2 * s) + c2 * ld(f + o - s)) + c3 * ld(f + o)) + ld(f + o + s)) +
                  c4 * ld(f + o + 2 * s)) +
                 c30 * ld(f + o + 3 * s));
  }
}

template <int ORDER>
__global__ void __launch_bounds__(kThreads) hadv_f64_kernel(
    double* __restrict__ uout, double* __restrict__ vout, const double* __restrict__ uin,
    const double* __restrict__ vin, const double* __restrict__ acrlat0, const double* __restrict__ acrlat1,
    const double* __restrict__ tgrlatda0, const double* __restrict__ tgrlatda1, int64_t s1d, double eddlat,
    double eddlon, Dims d, int kb) {
  const int64_t sj = d.sj;
  constexpr double third = 1.0 / 3.0;
  constexpr double rr = earth_radius_recip<double>();
  for_points(d, kb, [&](int64_t o, int j) {
    const int64_t jo = (int64_t)j * s1d;
    const double u0 = ld(uin + o), v0 = ld(vin + o);
    const double um = ld(uin + o - 1) + u0;  // uin(i-1)+uin(i), first pair of both averages
    // u at the u-position and v at the u-position (hadvuv.h:186-189)
    const double u_atupos = third * (um + ld(uin + o + 1));
    const double v_atupos = 0.25 * (((ld(vin + o + 1) + ld(vin + o + 1 - sj)) + v0) + ld(vin + o - sj));
    double ua = ld(acrlat0 + jo) * u_atupos;
    double va = rr * v_atupos;
    double rx, ry;
    if (ORDER == 3) {
      rx = adv3_axis(uin, o, 1, ua);
      ry = adv3_axis(uin, o, sj, va);
    } else {
      rx = adv5_axis(uin, o, 1, ua);
      ry = adv5_axis(uin, o, sj, va);
    }
    const double ures = eddlat * rx + eddlon * ry;
    uout[o] = ures + (ld(tgrlatda0 + jo) * u0) * v_atupos;
    // u and v at the v-position (hadvuv.h:197-206)
    const double u_atvpos = 0.25 * (((um) + ld(uin + o + sj)) + ld(uin + o - 1 + sj));
    const double v_atvpos = third * ((ld(vin + o - sj) + v0) + ld(vin + o + sj));
    ua = ld(acrlat1 + jo) * u_atvpos;
    va = rr * v_atvpos;
    if (ORDER == 3) {
      rx = adv3_axis(vin, o, 1, ua);
      ry = adv3_axis(vin, o, sj, va);
    } else {
      rx = adv5_axis(vin, o, 1, ua);
      ry = adv5_axis(vin, o, sj, va);
    }
    const double vres = eddlat * rx + eddlon * ry;
    vout[o] = vres - (ld(tgrlatda1 + jo) * u_atvpos) * u_atvpos;
  });
}

constexpr int kKB = 4;  // k-levels per CTA

Dims make_dims(const oeb_domain& dom, const Grid<double>& g) {
  return Dims{(int)dom.nx, (int)dom.ny, (int)dom.nz, g.sj, g.sk};
}

dim3 grid_for(const oeb_domain& dom) { return tile_grid((int)dom.nx, (int)dom.ny, (int)dom.nz, kTI, kTJ, kKB); }

}  // namespace
}  // namespace oeb

using namespace oeb;

extern "C" oeb_status oeb_laplace_f64(const oeb_memref3d_f64* in, const oeb_memref3d_f64* out,
                                      const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gin, gout;
  OEB_TRY((check_field3<double>(in, *dom, Reach{1, 1, 1, 1, 0, 0}, &gin)));
  OEB_TRY((check_field3<double>(out, *dom, kInterior, &gout)));
  OEB_TRY(check_same_strides<double>({&gin, &gout}));
  OEB_TRY(check_no_alias({gout.lo, gout.hi}, {gin.lo, gin.hi}));
  OEB_RETURN_IF_VALIDATING();
  laplace_f64_kernel<<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(gin.origin, gout.origin,
                                                                                 make_dims(*dom, gin), kKB);
  return after_launch();
}

extern "C" oeb_status oeb_uvbke_f64(const oeb_memref3d_f64* ub, const oeb_memref3d_f64* vb,
                                    const oeb_memref3d_f64* uc, const oeb_memref3d_f64* vc,
                                    const oeb_memref3d_f64* cosa, const oeb_memref3d_f64* rsina, double dt5,
                                    const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gub, gvb, guc, gvc, gca, grs;
  OEB_TRY((check_field3<double>(ub, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<double>(vb, *dom, kInterior, &gvb)));
  OEB_TRY((check_field3<double>(uc, *dom, Reach{0, 0, 1, 0, 0, 0}, &guc)));
  OEB_TRY((check_field3<double>(vc, *dom, Reach{1, 0, 0, 0, 0, 0}, &gvc)));
  OEB_TRY((check_field3<double>(cosa, *dom, kInterior, &gca)));
  OEB_TRY((check_field3<double>(rsina, *dom, kInterior, &grs)));
  OEB_TRY(check_same_strides<double>({&gub, &gvb, &guc, &gvc, &gca, &grs}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi},
                         {guc.lo, guc.hi, gvc.lo, gvc.hi, gca.lo, gca.hi, grs.lo, grs.hi}));
  OEB_RETURN_IF_VALIDATING();
  uvbke_f64_kernel<<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gub.origin, gvb.origin, guc.origin, gvc.origin, gca.origin, grs.origin, dt5, make_dims(*dom, gub), kKB);
  return after_launch();
}

extern "C" oeb_status oeb_p_grad_c_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                       const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                       const oeb_memref3d_f64* rdxc, const oeb_memref3d_f64* rdyc,
                                       const oeb_memref3d_f64* delpc, const oeb_memref3d_f64* gz,
                                       const oeb_memref3d_f64* pkc, double dt2, const oeb_domain* dom,
                                       void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gu, gv, gui, gvi, grx, gry, gdp, ggz, gpk;
  OEB_TRY((check_field3<double>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<double>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<double>(uin, *dom, kInterior, &gui)));
  OEB_TRY((check_field3<double>(vin, *dom, kInterior, &gvi)));
  OEB_TRY((check_field3<double>(rdxc, *dom, kInterior, &grx)));
  OEB_TRY((check_field3<double>(rdyc, *dom, kInterior, &gry)));
  OEB_TRY((check_field3<double>(delpc, *dom, Reach{1, 0, 1, 0, 0, 0}, &gdp)));
  OEB_TRY((check_field3<double>(gz, *dom, Reach{1, 0, 1, 0, 0, 1}, &ggz)));
  OEB_TRY((check_field3<double>(pkc, *dom, Reach{1, 0, 1, 0, 0, 1}, &gpk)));
  OEB_TRY(check_same_strides<double>({&gu, &gv, &gui, &gvi, &grx, &gry, &gdp, &ggz, &gpk}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi}, {gui.lo, gui.hi, gvi.lo, gvi.hi, grx.lo, grx.hi, gry.lo,
                                                        gry.hi, gdp.lo, gdp.hi, ggz.lo, ggz.hi, gpk.lo, gpk.hi}));
  OEB_RETURN_IF_VALIDATING();
  p_grad_c_f64_kernel<<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, grx.origin, gry.origin, gdp.origin, ggz.origin, gpk.origin, dt2,
      make_dims(*dom, gu), kKB);
  return after_launch();
}

extern "C" oeb_status oeb_nh_p_grad_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                        const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                        const oeb_memref3d_f64* rdx, const oeb_memref3d_f64* rdy,
                                        const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pp,
                                        const oeb_memref3d_f64* pk3, const oeb_memref3d_f64* wk1, double dt,
                                        const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<double> gu, gv, gui, gvi, grx, gry, ggz, gpp, gpk, gw1;
  const Reach r11 = Reach{0, 1, 0, 1, 0, 1};
  OEB_TRY((check_field3<double>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<double>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<double>(uin, *dom, kInterior, &gui)));
  OEB_TRY((check_field3<double>(vin, *dom, kInterior, &gvi)));
  OEB_TRY((check_field3<double>(rdx, *dom, kInterior, &grx)));
  OEB_TRY((check_field3<double>(rdy, *dom, kInterior, &gry)));
  OEB_TRY((check_field3<double>(gz, *dom, r11, &ggz)));
  OEB_TRY((check_field3<double>(pp, *dom, r11, &gpp)));
  OEB_TRY((check_field3<double>(pk3, *dom, r11, &gpk)));
  OEB_TRY((check_field3<double>(wk1, *dom, Reach{0, 1, 0, 1, 0, 0}, &gw1)));
  OEB_TRY(check_same_strides<double>({&gu, &gv, &gui, &gvi, &grx, &gry, &ggz, &gpp, &gpk, &gw1}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi},
                         {gui.lo, gui.hi, gvi.lo, gvi.hi, grx.lo, grx.hi, gry.lo, gry.hi, ggz.lo, ggz.hi, gpp.lo,
                          gpp.hi, gpk.lo, gpk.hi, gw1.lo, gw1.hi}));
  OEB_RETURN_IF_VALIDATING();
  nh_p_grad_f64_kernel<<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, grx.origin, gry.origin, ggz.origin, gpp.origin, gpk.origin,
      gw1.origin, dt, make_dims(*dom, gu), kKB);
  return after_launch();
}

template <int ORDER>
static oeb_status hadv_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout, const oeb_memref3d_f64* uin,
                           const oeb_memref3d_f64* vin, const oeb_memref1d_f64* acrlat0,
                           const oeb_memref1d_f64* acrlat1, const oeb_memref1d_f64* tgrlatda0,
                           const oeb_memref1d_f64* tgrlatda1, double eddlat, double eddlon, const oeb_domain* dom,
                           void* stream) {
  OEB_TRY(check_domain(dom));
  const int h = ORDER == 3 ? 2 : 3;
  Grid<double> gu, gv, gui, gvi;
  Line<double> a0, a1, t0, t1;
  OEB_TRY((check_field3<double>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<double>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<double>(uin, *dom, Reach{h, h, h, h, 0, 0}, &gui)));
  OEB_TRY((check_field3<double>(vin, *dom, Reach{h, h, h, h, 0, 0}, &gvi)));
  OEB_TRY((check_field1<double>(acrlat0, *dom, 0, 0, &a0)));
  OEB_TRY((check_field1<double>(acrlat1, *dom, 0, 0, &a1)));
  OEB_TRY((check_field1<double>(tgrlatda0, *dom, 0, 0, &t0)));
  OEB_TRY((check_field1<double>(tgrlatda1, *dom, 0, 0, &t1)));
  // The four 1-D fields share one stride in the kernel.
  if (a1.s != a0.s || t0.s != a0.s || t1.s != a0.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<double>({&gu, &gv, &gui, &gvi}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi}, {gui.lo, gui.hi, gvi.lo, gvi.hi, a0.lo, a0.hi, a1.lo, a1.hi,
                                                        t0.lo, t0.hi, t1.lo, t1.hi}));
  OEB_RETURN_IF_VALIDATING();
  hadv_f64_kernel<ORDER><<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, a0.origin, a1.origin, t0.origin, t1.origin, a0.s, eddlat, eddlon,
      make_dims(*dom, gu), kKB);
  return after_launch();
}

extern "C" oeb_status oeb_hadvuv_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                     const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                     const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                     const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1,
                                     double eddlat, double eddlon, const oeb_domain* dom, void* stream) {
  return hadv_f64<3>(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom, stream);
}

extern "C" oeb_status oeb_hadvuv5th_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                        const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                        const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                        const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1,
                                        double eddlat, double eddlon, const oeb_domain* dom, void* stream) {
  return hadv_f64<5>(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom, stream);
}
