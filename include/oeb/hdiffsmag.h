// include/oeb/hdiffsmag.h -- drop-in replacement of the reference's kernels/hdiffsmag.h (kernels/hdiffsmag.h:4-7).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_hdiffsmag_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
// hdiffsmag (default variant) differs from hdiffsmag_openmp at the domain border in the
// reference (kernels/hdiffsmag.h:8-58); every variant here computes the openmp result.
#ifndef HDIFFSMAG_H
#define HDIFFSMAG_H

#include "oeb_dropin.hpp"

inline void hdiffsmag(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& mask, const Storage1D& crlavo, const Storage1D& crlavu, const Storage1D& crlato, const Storage1D& crlatu, const Storage1D& acrlat0, Storage3D& T_sqr_s, Storage3D& S_sqr_uv, const ElementType eddlat, const ElementType eddlon, const ElementType tau_smag, const ElementType weight_smag) {
  (void)T_sqr_s; (void)S_sqr_uv;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_uout = oeb_dropin::m3(uout);
  const auto m_vout = oeb_dropin::m3(vout);
  const auto m_uin = oeb_dropin::m3(uin);
  const auto m_vin = oeb_dropin::m3(vin);
  const auto m_mask = oeb_dropin::m3(mask);
  const auto m_crlavo = oeb_dropin::m1(crlavo);
  const auto m_crlavu = oeb_dropin::m1(crlavu);
  const auto m_crlato = oeb_dropin::m1(crlato);
  const auto m_crlatu = oeb_dropin::m1(crlatu);
  const auto m_acrlat0 = oeb_dropin::m1(acrlat0);
  oeb_dropin::dispatch(uin.alignedPtr, "hdiffsmag", [&](void* s_, bool dev_) {
    return oeb_dropin::call_hdiffsmag(&m_uout, &m_vout, &m_uin, &m_vin, &m_mask, &m_crlavo, &m_crlavu, &m_crlato, &m_crlatu, &m_acrlat0, eddlat, eddlon, tau_smag, weight_smag, &d_, s_, dev_);
  });
}

inline void hdiffsmag_fullfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& mask, const Storage1D& crlavo, const Storage1D& crlavu, const Storage1D& crlato, const Storage1D& crlatu, const Storage1D& acrlat0, Storage3D& T_sqr_s, Storage3D& S_sqr_uv, const ElementType eddlat, const ElementType eddlon, const ElementType tau_smag, const ElementType weight_smag) { hdiffsmag(uout, vout, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, T_sqr_s, S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); }

inline void hdiffsmag_partialfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& mask, const Storage1D& crlavo, const Storage1D& crlavu, const Storage1D& crlato, const Storage1D& crlatu, const Storage1D& acrlat0, Storage3D& T_sqr_s, Storage3D& S_sqr_uv, const ElementType eddlat, const ElementType eddlon, const ElementType tau_smag, const ElementType weight_smag) { hdiffsmag(uout, vout, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, T_sqr_s, S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); }

inline void hdiffsmag_openmp(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& mask, const Storage1D& crlavo, const Storage1D& crlavu, const Storage1D& crlato, const Storage1D& crlatu, const Storage1D& acrlat0, Storage3D& T_sqr_s, Storage3D& S_sqr_uv, const ElementType eddlat, const ElementType eddlon, const ElementType tau_smag, const ElementType weight_smag) { hdiffsmag(uout, vout, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, T_sqr_s, S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); }

#endif  // HDIFFSMAG_H
