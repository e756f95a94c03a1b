// include/oeb/fastwavesuv.h -- drop-in replacement of the reference's kernels/fastwavesuv.h (kernels/fastwavesuv.h:4-7).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_fastwavesuv_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
#ifndef FASTWAVESUV_H
#define FASTWAVESUV_H

#include "oeb_dropin.hpp"

inline void fastwavesuv(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& utens, const Storage3D& vtens, const Storage3D& wgtfac, const Storage3D& ppuv, const Storage3D& hhl, const Storage3D& rho, const Storage1D& fx, Storage3D& ppgk, Storage3D& ppgc, Storage3D& ppgu, Storage3D& ppgv, const ElementType edadlat, const ElementType dt) {
  (void)ppgk; (void)ppgc; (void)ppgu; (void)ppgv;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_uout = oeb_dropin::m3(uout);
  const auto m_vout = oeb_dropin::m3(vout);
  const auto m_uin = oeb_dropin::m3(uin);
  const auto m_vin = oeb_dropin::m3(vin);
  const auto m_utens = oeb_dropin::m3(utens);
  const auto m_vtens = oeb_dropin::m3(vtens);
  const auto m_wgtfac = oeb_dropin::m3(wgtfac);
  const auto m_ppuv = oeb_dropin::m3(ppuv);
  const auto m_hhl = oeb_dropin::m3(hhl);
  const auto m_rho = oeb_dropin::m3(rho);
  const auto m_fx = oeb_dropin::m1(fx);
  oeb_dropin::dispatch(uin.alignedPtr, "fastwavesuv", [&](void* s_, bool dev_) {
    return oeb_dropin::call_fastwavesuv(&m_uout, &m_vout, &m_uin, &m_vin, &m_utens, &m_vtens, &m_wgtfac, &m_ppuv, &m_hhl, &m_rho, &m_fx, edadlat, dt, &d_, s_, dev_);
  });
}

inline void fastwavesuv_fullfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& utens, const Storage3D& vtens, const Storage3D& wgtfac, const Storage3D& ppuv, const Storage3D& hhl, const Storage3D& rho, const Storage1D& fx, Storage3D& ppgk, Storage3D& ppgc, Storage3D& ppgu, Storage3D& ppgv, const ElementType edadlat, const ElementType dt) { fastwavesuv(uout, vout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, ppgk, ppgc, ppgu, ppgv, edadlat, dt); }

inline void fastwavesuv_partialfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& utens, const Storage3D& vtens, const Storage3D& wgtfac, const Storage3D& ppuv, const Storage3D& hhl, const Storage3D& rho, const Storage1D& fx, Storage3D& ppgk, Storage3D& ppgc, Storage3D& ppgu, Storage3D& ppgv, const ElementType edadlat, const ElementType dt) { fastwavesuv(uout, vout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, ppgk, ppgc, ppgu, ppgv, edadlat, dt); }

inline void fastwavesuv_openmp(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& utens, const Storage3D& vtens, const Storage3D& wgtfac, const Storage3D& ppuv, const Storage3D& hhl, const Storage3D& rho, const Storage1D& fx, Storage3D& ppgk, Storage3D& ppgc, Storage3D& ppgu, Storage3D& ppgv, const ElementType edadlat, const ElementType dt) { fastwavesuv(uout, vout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, ppgk, ppgc, ppgu, ppgv, edadlat, dt); }

#endif  // FASTWAVESUV_H
