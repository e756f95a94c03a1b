// include/oeb/hdiffsa.h -- drop-in replacement of the reference's kernels/hdiffsa.h (kernels/hdiffsa.h:4-5).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_hdiffsa_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
#ifndef HDIFFSA_H
#define HDIFFSA_H

#include "oeb_dropin.hpp"

inline void hdiffsa(Storage3D& out, const Storage3D& in, const Storage3D& mask, const Storage1D& crlato, const Storage1D& crlatu, Storage3D& lap, Storage3D& flx, Storage3D& fly) {
  (void)lap; (void)flx; (void)fly;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_out = oeb_dropin::m3(out);
  const auto m_in = oeb_dropin::m3(in);
  const auto m_mask = oeb_dropin::m3(mask);
  const auto m_crlato = oeb_dropin::m1(crlato);
  const auto m_crlatu = oeb_dropin::m1(crlatu);
  oeb_dropin::dispatch(in.alignedPtr, "hdiffsa", [&](void* s_, bool dev_) {
    return oeb_dropin::call_hdiffsa(&m_out, &m_in, &m_mask, &m_crlato, &m_crlatu, &d_, s_, dev_);
  });
}

inline void hdiffsa_fullfusion(Storage3D& out, const Storage3D& in, const Storage3D& mask, const Storage1D& crlato, const Storage1D& crlatu, Storage3D& lap, Storage3D& flx, Storage3D& fly) { hdiffsa(out, in, mask, crlato, crlatu, lap, flx, fly); }

inline void hdiffsa_partialfusion(Storage3D& out, const Storage3D& in, const Storage3D& mask, const Storage1D& crlato, const Storage1D& crlatu, Storage3D& lap, Storage3D& flx, Storage3D& fly) { hdiffsa(out, in, mask, crlato, crlatu, lap, flx, fly); }

inline void hdiffsa_openmp(Storage3D& out, const Storage3D& in, const Storage3D& mask, const Storage1D& crlato, const Storage1D& crlatu, Storage3D& lap, Storage3D& flx, Storage3D& fly) { hdiffsa(out, in, mask, crlato, crlatu, lap, flx, fly); }

#endif  // HDIFFSA_H
