// k_pointwise.cu -- stencils whose intermediates are used only at their own point:
// laplace, uvbke, p_grad_c, nh_p_grad, hadvuv and hadvuv5th, in FP64 and FP32.
//
// FP64: compiled with --fmad=false, every a*b+c is rounded twice, exactly as the reference
// compiled without FP contraction, and double division and square root are IEEE
// round-to-nearest on both sides, so the results are bit-identical to the reference
// OpenMP kernels.  Expression trees keep the reference's order and parenthesisation; a
// subexpression that occurs twice in the reference is computed once here (same operands,
// same value).  FP32: the same trees in float, with the advection flux sums compensated
// (precision.cuh).
//
// One CTA of 32 x 8 threads covers a 32 x 32 (i, j) tile and KB k-levels; each thread
// computes 4 rows.  Neighbour reads go through L1.
#include "precision.cuh"
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
template <class T>
__global__ void __launch_bounds__(kThreads) laplace_kernel(const T* __restrict__ in, T* __restrict__ out, Dims d,
                                                           int kb) {
  const int64_t sj = d.sj;
  for_points(d, kb, [&](int64_t o, int) {
    out[o] = T(-4.0) * ld(in + o) + ((ld(in + o - 1) + ld(in + o + 1)) + (ld(in + o + sj) + ld(in + o - sj)));
  });
}

// ---- uvbke: kernels/uvbke.h:61-75 ----------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kThreads) uvbke_kernel(T* __restrict__ ub, T* __restrict__ vb,
                                                         const T* __restrict__ uc, const T* __restrict__ vc,
                                                         const T* __restrict__ cosa, const T* __restrict__ rsina,
                                                         T dt5, Dims d, int kb) {
  const int64_t sj = d.sj;
  for_points(d, kb, [&](int64_t o, int) {
    const T su = ld(uc + o - sj) + ld(uc + o);
    const T sv = ld(vc + o - 1) + ld(vc + o);
    const T ca = ld(cosa + o);
    const T rs = ld(rsina + o);
    ub[o] = ((dt5 * (su - (sv * ca))) * rs);
    vb[o] = ((dt5 * (sv - (su * ca))) * rs);
  });
}

// ---- p_grad_c: kernels/p_grad_c.h:80-101 ---------------------------------------------
template <class T>
__global__ void __launch_bounds__(kThreads) p_grad_c_kernel(T* __restrict__ uout, T* __restrict__ vout,
                                                            const T* __restrict__ uin, const T* __restrict__ vin,
                                                            const T* __restrict__ rdxc, const T* __restrict__ rdyc,
                                                            const T* __restrict__ delpc, const T* __restrict__ gz,
                                                            const T* __restrict__ pkc, T dt2, Dims d, int kb) {
  const int64_t sj = d.sj, sk = d.sk;
  for_points(d, kb, [&](int64_t o, int) {
    const T wk = ld(delpc + o);
    const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pkc + o), pk1 = ld(pkc + o + sk);
    uout[o] = (ld(uin + o) + (((dt2 * ld(rdxc + o)) / (ld(delpc + o - 1) + wk)) *
                              (((ld(gz + o - 1 + sk) - gz0) * (pk1 - ld(pkc + o - 1))) +
                               ((ld(gz + o - 1) - gz1) * (ld(pkc + o - 1 + sk) - pk0)))));
    vout[o] = (ld(vin + o) + (((dt2 * ld(rdyc + o)) / (ld(delpc + o - sj) + wk)) *
                              (((ld(gz + o - sj + sk) - gz0) * (pk1 - ld(pkc + o - sj))) +
                               ((ld(gz + o - sj) - gz1) * (ld(pkc + o - sj + sk) - pk0)))));
  });
}

// ---- nh_p_grad: kernels/nh_p_grad.h:116-146 --------------------------------------------
template <class T>
__global__ void __launch_bounds__(kThreads) nh_p_grad_kernel(T* __restrict__ uout, T* __restrict__ vout,
                                                             const T* __restrict__ uin, const T* __restrict__ vin,
                                                             const T* __restrict__ rdx, const T* __restrict__ rdy,
                                                             const T* __restrict__ gz, const T* __restrict__ pp,
                                                             const T* __restrict__ pk3, const T* __restrict__ wk1,
                                                             T dt, Dims d, int kb) {
  const int64_t sj = d.sj, sk = d.sk;
  for_points(d, kb, [&](int64_t o, int) {
    const T pk0 = ld(pk3 + o), pk1 = ld(pk3 + o + sk);
    const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk);
    const T pp0 = ld(pp + o), pp1 = ld(pp + o + sk);
    const T w1 = ld(wk1 + o);
    const T wk = pk1 - pk0;
    // u: neighbour i+1
    {
      const T pkx0 = ld(pk3 + o + 1), pkx1 = ld(pk3 + o + 1 + sk);
      const T wkx = pkx1 - pkx0;
      const T ga = gz1 - ld(gz + o + 1);
      const T gb = gz0 - ld(gz + o + 1 + sk);
      const T du = ((dt / (wk + wkx)) * ((ga * (pkx1 - pk0)) + (gb * (pk1 - pkx0))));
      uout[o] = (((ld(uin + o) + du) +
                  ((dt / (w1 + ld(wk1 + o + 1))) * ((ga * (ld(pp + o + 1 + sk) - pp0)) + (gb * (pp1 - ld(pp + o + 1)))))) *
                 ld(rdx + o));
    }
    // v: neighbour j+1
    {
      const T pky0 = ld(pk3 + o + sj), pky1 = ld(pk3 + o + sj + sk);
      const T wky = pky1 - pky0;
      const T ga = gz1 - ld(gz + o + sj);
      const T gb = gz0 - ld(gz + o + sj + sk);
      const T dv = ((dt / (wk + wky)) * ((ga * (pky1 - pk0)) + (gb * (pk1 - pky0))));
      vout[o] = (((ld(vin + o) + dv) +
                  ((dt / (w1 + ld(wk1 + o + sj))) *
                   ((ga * (ld(pp + o + sj + sk) - pp0)) + (gb * (pp1 - ld(pp + o + sj)))))) *
                 ld(rdy + o));
    }
  });
}

// ---- hadvuv / hadvuv5th: kernels/hadvuv.h:4-27,178-210 and kernels/hadvuv5th.h:4-39,177-201

// 3rd-order upwind advection along one axis (stride s): hadvuv.h:10-16 (x) and :18-24 (y).
template <class T>
__device__ __forceinline__ T adv3_axis(const T* __restrict__ f, int64_t o, int64_t s, T a) {
  constexpr T c6 = T(-1.0) / T(6.0), c3 = T(-1.0) / T(3.0), ch = T(-0.5);
  if (a > 0) {
    Acc<T> acc = Acc<T>::prod(c6, ld(f + o - 2 * s));
    acc.add(ld(f + o - s));
    acc.add_prod(ch, ld(f + o));
    acc.add_prod(c3, ld(f + o + s));
    return a * acc.get();
  } else {
    Acc<T> acc = Acc<T>::prod(c3, ld(f + o - s));
    acc.add_prod(ch, ld(f + o));
    acc.add(ld(f + o + s));
    acc.add_prod(c6, ld(f + o + 2 * s));
    return -a * acc.get();
  }
}

// 5th-order upwind advection along one axis: hadvuv5th.h:10-22 (x) and :24-36 (y).
template <class T>
__device__ __forceinline__ T adv5_axis(const T* __restrict__ f, int64_t o, int64_t s, T a) {
  constexpr T c30 = T(1.0) / T(30.0), c4 = T(-1.0) / T(4.0), c3 = T(-1.0) / T(3.0), c2 = T(-1.0) / T(2.0),
              c20 = T(1.0) / T(20.0);
  if (a > 0) {
    Acc<T> acc = Acc<T>::prod(c30, ld(f + o - 3 * s));
    acc.add_prod(c4, ld(f + o - 2 * s));
    acc.add(ld(f + o - s));
    acc.add_prod(c3, ld(f + o));
    acc.add_prod(c2, ld(f + o + s));
    acc.add_prod(c20, ld(f + o + 2 * s));
    return a * acc.get();
  } else {
    Acc<T> acc = Acc<T>::prod(c20, ld(f + o - 2 * s));
    acc.add_prod(c2, ld(f + o - s));
    acc.add_prod(c3, ld(f + o));
    acc.add(ld(f + o + s));
    acc.add_prod(c4, ld(f + o + 2 * s));
    acc.add_prod(c30, ld(f + o + 3 * s));
    return -a * acc.get();
  }
}

template <class T, int ORDER>
__global__ void __launch_bounds__(kThreads) hadv_kernel(T* __restrict__ uout, T* __restrict__ vout,
                                                        const T* __restrict__ uin, const T* __restrict__ vin,
                                                        const T* __restrict__ acrlat0, const T* __restrict__ acrlat1,
                                                        const T* __restrict__ tgrlatda0,
                                                        const T* __restrict__ tgrlatda1, int64_t s1d, T eddlat,
                                                        T eddlon, Dims d, int kb) {
  const int64_t sj = d.sj;
  constexpr T third = T(1.0) / T(3.0);
  constexpr T rr = earth_radius_recip<T>();
  for_points(d, kb, [&](int64_t o, int j) {
    const int64_t jo = (int64_t)j * s1d;
    const T u0 = ld(uin + o), v0 = ld(vin + o);
    const T um = ld(uin + o - 1) + u0;  // uin(i-1)+uin(i), first pair of both averages
    // u at the u-position and v at the u-position (hadvuv.h:186-189)
    const T u_atupos = third * (um + ld(uin + o + 1));
    const T v_atupos = T(0.25) * (((ld(vin + o + 1) + ld(vin + o + 1 - sj)) + v0) + ld(vin + o - sj));
    T ua = ld(acrlat0 + jo) * u_atupos;
    T va = rr * v_atupos;
    T rx, ry;
    if (ORDER == 3) {
      rx = adv3_axis(uin, o, 1, ua);
      ry = adv3_axis(uin, o, sj, va);
    } else {
      rx = adv5_axis(uin, o, 1, ua);
      ry = adv5_axis(uin, o, sj, va);
    }
    const T ures = eddlat * rx + eddlon * ry;
    uout[o] = ures + (ld(tgrlatda0 + jo) * u0) * v_atupos;
    // u and v at the v-position (hadvuv.h:197-206)
    const T u_atvpos = T(0.25) * (((um) + ld(uin + o + sj)) + ld(uin + o - 1 + sj));
    const T v_atvpos = third * ((ld(vin + o - sj) + v0) + ld(vin + o + sj));
    ua = ld(acrlat1 + jo) * u_atvpos;
    va = rr * v_atvpos;
    if (ORDER == 3) {
      rx = adv3_axis(vin, o, 1, ua);
      ry = adv3_axis(vin, o, sj, va);
    } else {
      rx = adv5_axis(vin, o, 1, ua);
      ry = adv5_axis(vin, o, sj, va);
    }
    const T vres = eddlat * rx + eddlon * ry;
    vout[o] = vres - (ld(tgrlatda1 + jo) * u_atvpos) * u_atvpos;
  });
}

constexpr int kKB = 4;  // k-levels per CTA

template <class T>
Dims make_dims(const oeb_domain& dom, const Grid<T>& g) {
  return Dims{(int)dom.nx, (int)dom.ny, (int)dom.nz, g.sj, g.sk};
}

dim3 grid_for(const oeb_domain& dom) { return tile_grid((int)dom.nx, (int)dom.ny, (int)dom.nz, kTI, kTJ, kKB); }

// ------------------------------ entry points -----------------------------------------

template <class T, class M3>
oeb_status laplace_entry(const M3* in, const M3* out, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gin, gout;
  OEB_TRY((check_field3<T>(in, *dom, Reach{1, 1, 1, 1, 0, 0}, &gin)));
  OEB_TRY((check_field3<T>(out, *dom, kInterior, &gout)));
  OEB_TRY(check_same_strides<T>({&gin, &gout}));
  OEB_TRY(check_no_alias({gout.lo, gout.hi}, {gin.lo, gin.hi}));
  OEB_RETURN_IF_VALIDATING();
  laplace_kernel<T><<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(gin.origin, gout.origin,
                                                                                make_dims(*dom, gin), kKB);
  return after_launch();
}

template <class T, class M3>
oeb_status uvbke_entry(const M3* ub, const M3* vb, const M3* uc, const M3* vc, const M3* cosa, const M3* rsina,
                       double dt5, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gub, gvb, guc, gvc, gca, grs;
  OEB_TRY((check_field3<T>(ub, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<T>(vb, *dom, kInterior, &gvb)));
  OEB_TRY((check_field3<T>(uc, *dom, Reach{0, 0, 1, 0, 0, 0}, &guc)));
  OEB_TRY((check_field3<T>(vc, *dom, Reach{1, 0, 0, 0, 0, 0}, &gvc)));
  OEB_TRY((check_field3<T>(cosa, *dom, kInterior, &gca)));
  OEB_TRY((check_field3<T>(rsina, *dom, kInterior, &grs)));
  OEB_TRY(check_same_strides<T>({&gub, &gvb, &guc, &gvc, &gca, &grs}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi},
                         {guc.lo, guc.hi, gvc.lo, gvc.hi, gca.lo, gca.hi, grs.lo, grs.hi}));
  OEB_RETURN_IF_VALIDATING();
  uvbke_kernel<T><<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gub.origin, gvb.origin, guc.origin, gvc.origin, gca.origin, grs.origin, T(dt5), make_dims(*dom, gub), kKB);
  return after_launch();
}

template <class T, class M3>
oeb_status p_grad_c_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdxc,
                          const M3* rdyc, const M3* delpc, const M3* gz, const M3* pkc, T dt2,
                          const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gu, gv, gui, gvi, grx, gry, gdp, ggz, gpk;
  OEB_TRY((check_field3<T>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<T>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<T>(uin, *dom, kInterior, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, kInterior, &gvi)));
  OEB_TRY((check_field3<T>(rdxc, *dom, kInterior, &grx)));
  OEB_TRY((check_field3<T>(rdyc, *dom, kInterior, &gry)));
  OEB_TRY((check_field3<T>(delpc, *dom, Reach{1, 0, 1, 0, 0, 0}, &gdp)));
  OEB_TRY((check_field3<T>(gz, *dom, Reach{1, 0, 1, 0, 0, 1}, &ggz)));
  OEB_TRY((check_field3<T>(pkc, *dom, Reach{1, 0, 1, 0, 0, 1}, &gpk)));
  OEB_TRY(check_same_strides<T>({&gu, &gv, &gui, &gvi, &grx, &gry, &gdp, &ggz, &gpk}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi}, {gui.lo, gui.hi, gvi.lo, gvi.hi, grx.lo, grx.hi, gry.lo,
                                                        gry.hi, gdp.lo, gdp.hi, ggz.lo, ggz.hi, gpk.lo, gpk.hi}));
  OEB_RETURN_IF_VALIDATING();
  p_grad_c_kernel<T><<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, grx.origin, gry.origin, gdp.origin, ggz.origin, gpk.origin, dt2,
      make_dims(*dom, gu), kKB);
  return after_launch();
}

template <class T, class M3>
oeb_status nh_p_grad_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdx,
                           const M3* rdy, const M3* gz, const M3* pp, const M3* pk3, const M3* wk1, T dt,
                           const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gu, gv, gui, gvi, grx, gry, ggz, gpp, gpk, gw1;
  const Reach r11 = Reach{0, 1, 0, 1, 0, 1};
  OEB_TRY((check_field3<T>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<T>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<T>(uin, *dom, kInterior, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, kInterior, &gvi)));
  OEB_TRY((check_field3<T>(rdx, *dom, kInterior, &grx)));
  OEB_TRY((check_field3<T>(rdy, *dom, kInterior, &gry)));
  OEB_TRY((check_field3<T>(gz, *dom, r11, &ggz)));
  OEB_TRY((check_field3<T>(pp, *dom, r11, &gpp)));
  OEB_TRY((check_field3<T>(pk3, *dom, r11, &gpk)));
  OEB_TRY((check_field3<T>(wk1, *dom, Reach{0, 1, 0, 1, 0, 0}, &gw1)));
  OEB_TRY(check_same_strides<T>({&gu, &gv, &gui, &gvi, &grx, &gry, &ggz, &gpp, &gpk, &gw1}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi},
                         {gui.lo, gui.hi, gvi.lo, gvi.hi, grx.lo, grx.hi, gry.lo, gry.hi, ggz.lo, ggz.hi, gpp.lo,
                          gpp.hi, gpk.lo, gpk.hi, gw1.lo, gw1.hi}));
  OEB_RETURN_IF_VALIDATING();
  nh_p_grad_kernel<T><<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, grx.origin, gry.origin, ggz.origin, gpp.origin, gpk.origin,
      gw1.origin, dt, make_dims(*dom, gu), kKB);
  return after_launch();
}

template <class T, int ORDER, class M3, class M1>
oeb_status hadv_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M1* acrlat0,
                      const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, T eddlat, T eddlon,
                      const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  const int h = ORDER == 3 ? 2 : 3;
  Grid<T> gu, gv, gui, gvi;
  Line<T> a0, a1, t0, t1;
  OEB_TRY((check_field3<T>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<T>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<T>(uin, *dom, Reach{h, h, h, h, 0, 0}, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, Reach{h, h, h, h, 0, 0}, &gvi)));
  OEB_TRY((check_field1<T>(acrlat0, *dom, 0, 0, &a0)));
  OEB_TRY((check_field1<T>(acrlat1, *dom, 0, 0, &a1)));
  OEB_TRY((check_field1<T>(tgrlatda0, *dom, 0, 0, &t0)));
  OEB_TRY((check_field1<T>(tgrlatda1, *dom, 0, 0, &t1)));
  // The four 1-D fields share one stride in the kernel.
  if (a1.s != a0.s || t0.s != a0.s || t1.s != a0.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<T>({&gu, &gv, &gui, &gvi}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi}, {gui.lo, gui.hi, gvi.lo, gvi.hi, a0.lo, a0.hi, a1.lo, a1.hi,
                                                        t0.lo, t0.hi, t1.lo, t1.hi}));
  OEB_RETURN_IF_VALIDATING();
  hadv_kernel<T, ORDER><<<grid_for(*dom), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, a0.origin, a1.origin, t0.origin, t1.origin, a0.s, eddlat, eddlon,
      make_dims(*dom, gu), kKB);
  return after_launch();
}

}  // namespace
}  // namespace oeb

using namespace oeb;

#define OEB_M3(S) oeb_memref3d_##S
#define OEB_M1(S) oeb_memref1d_##S

#define OEB_POINTWISE_ENTRIES(S, T)                                                                                \
  extern "C" oeb_status oeb_laplace_##S(const OEB_M3(S) * in, const OEB_M3(S) * out, const oeb_domain* dom,        \
                                        void* stream) {                                                            \
    return laplace_entry<T>(in, out, dom, stream);                                                                 \
  }                                                                                                                \
  extern "C" oeb_status oeb_uvbke_##S(const OEB_M3(S) * ub, const OEB_M3(S) * vb, const OEB_M3(S) * uc,            \
                                      const OEB_M3(S) * vc, const OEB_M3(S) * cosa, const OEB_M3(S) * rsina,       \
                                      double dt5, const oeb_domain* dom, void* stream) {                           \
    return uvbke_entry<T>(ub, vb, uc, vc, cosa, rsina, dt5, dom, stream);                                          \
  }                                                                                                                \
  extern "C" oeb_status oeb_p_grad_c_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,    \
                                         const OEB_M3(S) * vin, const OEB_M3(S) * rdxc, const OEB_M3(S) * rdyc,    \
                                         const OEB_M3(S) * delpc, const OEB_M3(S) * gz, const OEB_M3(S) * pkc,     \
                                         T dt2, const oeb_domain* dom, void* stream) {                             \
    return p_grad_c_entry<T>(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, dt2, dom, stream);                  \
  }                                                                                                                \
  extern "C" oeb_status oeb_nh_p_grad_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,   \
                                          const OEB_M3(S) * vin, const OEB_M3(S) * rdx, const OEB_M3(S) * rdy,     \
                                          const OEB_M3(S) * gz, const OEB_M3(S) * pp, const OEB_M3(S) * pk3,       \
                                          const OEB_M3(S) * wk1, T dt, const oeb_domain* dom, void* stream) {      \
    return nh_p_grad_entry<T>(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, dt, dom, stream);                  \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,      \
                                       const OEB_M3(S) * vin, const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1, \
                                       const OEB_M1(S) * tgrlatda0, const OEB_M1(S) * tgrlatda1, T eddlat,         \
                                       T eddlon, const oeb_domain* dom, void* stream) {                            \
    return hadv_entry<T, 3>(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom,     \
                            stream);                                                                               \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv5th_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,   \
                                          const OEB_M3(S) * vin, const OEB_M1(S) * acrlat0,                        \
                                          const OEB_M1(S) * acrlat1, const OEB_M1(S) * tgrlatda0,                  \
                                          const OEB_M1(S) * tgrlatda1, T eddlat, T eddlon, const oeb_domain* dom,  \
                                          void* stream) {                                                          \
    return hadv_entry<T, 5>(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom,     \
                            stream);                                                                               \
  }

OEB_POINTWISE_ENTRIES(f64, double)
OEB_POINTWISE_ENTRIES(f32, float)
