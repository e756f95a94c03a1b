// include/oeb/hadvuv.h -- drop-in replacement of the reference's kernels/hadvuv.h (kernels/hadvuv.h:29-32).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_hadvuv_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
// advectionDriver (the reference's per-point helper) is part of the GPU kernel and is not
// exported.
#ifndef HADVUV_H
#define HADVUV_H

#include "oeb_dropin.hpp"

inline void hadvuv(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage1D& acrlat0, const Storage1D& acrlat1, const Storage1D& tgrlatda0, const Storage1D& tgrlatda1, Storage3D& uatupos, Storage3D& vatupos, Storage3D& uatvpos, Storage3D& vatvpos, Storage3D& uavg, Storage3D& vavg, Storage3D& ures, Storage3D& vres, const ElementType eddlat, const ElementType eddlon) {
  (void)uatupos; (void)vatupos; (void)uatvpos; (void)vatvpos; (void)uavg; (void)vavg; (void)ures; (void)vres;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_uout = oeb_dropin::m3(uout);
  const auto m_vout = oeb_dropin::m3(vout);
  const auto m_uin = oeb_dropin::m3(uin);
  const auto m_vin = oeb_dropin::m3(vin);
  const auto m_acrlat0 = oeb_dropin::m1(acrlat0);
  const auto m_acrlat1 = oeb_dropin::m1(acrlat1);
  const auto m_tgrlatda0 = oeb_dropin::m1(tgrlatda0);
  const auto m_tgrlatda1 = oeb_dropin::m1(tgrlatda1);
  oeb_dropin::dispatch(uin.alignedPtr, "hadvuv", [&](void* s_, bool dev_) {
    return oeb_dropin::call_hadvuv(&m_uout, &m_vout, &m_uin, &m_vin, &m_acrlat0, &m_acrlat1, &m_tgrlatda0, &m_tgrlatda1, eddlat, eddlon, &d_, s_, dev_);
  });
}

inline void hadvuv_fullfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage1D& acrlat0, const Storage1D& acrlat1, const Storage1D& tgrlatda0, const Storage1D& tgrlatda1, Storage3D& uatupos, Storage3D& vatupos, Storage3D& uatvpos, Storage3D& vatvpos, Storage3D& uavg, Storage3D& vavg, Storage3D& ures, Storage3D& vres, const ElementType eddlat, const ElementType eddlon) { hadvuv(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, uatupos, vatupos, uatvpos, vatvpos, uavg, vavg, ures, vres, eddlat, eddlon); }

inline void hadvuv_partialfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage1D& acrlat0, const Storage1D& acrlat1, const Storage1D& tgrlatda0, const Storage1D& tgrlatda1, Storage3D& uatupos, Storage3D& vatupos, Storage3D& uatvpos, Storage3D& vatvpos, Storage3D& uavg, Storage3D& vavg, Storage3D& ures, Storage3D& vres, const ElementType eddlat, const ElementType eddlon) { hadvuv(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, uatupos, vatupos, uatvpos, vatvpos, uavg, vavg, ures, vres, eddlat, eddlon); }

inline void hadvuv_openmp(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage1D& acrlat0, const Storage1D& acrlat1, const Storage1D& tgrlatda0, const Storage1D& tgrlatda1, Storage3D& uatupos, Storage3D& vatupos, Storage3D& uatvpos, Storage3D& vatvpos, Storage3D& uavg, Storage3D& vavg, Storage3D& ures, Storage3D& vres, const ElementType eddlat, const ElementType eddlon) { hadvuv(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, uatupos, vatupos, uatvpos, vatvpos, uavg, vavg, ures, vres, eddlat, eddlon); }

#endif  // HADVUV_H
