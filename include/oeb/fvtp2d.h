// include/oeb/fvtp2d.h -- drop-in replacement of the reference's kernels/fvtp2d.h (kernels/fvtp2d.h:4-7).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_fvtp2d_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
// Reads the driver's p1 and p2, as the reference does (src/fvtp2d.cpp:11-12).
// fvtp2d_fullfusion reads a stale scratch value in the reference (kernels/fvtp2d.h:195-196);
// here it computes fvtp2d.
#ifndef FVTP2D_H
#define FVTP2D_H

#include "oeb_dropin.hpp"

inline void fvtp2d(Storage3D& q_i, Storage3D& q_j, Storage3D& fx1, Storage3D& fx2, Storage3D& fy1, Storage3D& fy2, const Storage3D& q, const Storage3D& crx, const Storage3D& cry, const Storage3D& ra_x, const Storage3D& ra_y, const Storage3D& xfx, const Storage3D& yfx, const Storage3D& area, Storage3D& fxx, Storage3D& fyy, Storage3D& al, Storage3D& almq, Storage3D& br, Storage3D& b0, Storage3D& smt5) {
  (void)fxx; (void)fyy; (void)al; (void)almq; (void)br; (void)b0; (void)smt5;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_q_i = oeb_dropin::m3(q_i);
  const auto m_q_j = oeb_dropin::m3(q_j);
  const auto m_fx1 = oeb_dropin::m3(fx1);
  const auto m_fx2 = oeb_dropin::m3(fx2);
  const auto m_fy1 = oeb_dropin::m3(fy1);
  const auto m_fy2 = oeb_dropin::m3(fy2);
  const auto m_q = oeb_dropin::m3(q);
  const auto m_crx = oeb_dropin::m3(crx);
  const auto m_cry = oeb_dropin::m3(cry);
  const auto m_ra_x = oeb_dropin::m3(ra_x);
  const auto m_ra_y = oeb_dropin::m3(ra_y);
  const auto m_xfx = oeb_dropin::m3(xfx);
  const auto m_yfx = oeb_dropin::m3(yfx);
  const auto m_area = oeb_dropin::m3(area);
  oeb_dropin::dispatch(q.alignedPtr, "fvtp2d", [&](void* s_, bool dev_) {
    return oeb_dropin::call_fvtp2d(&m_q_i, &m_q_j, &m_fx1, &m_fx2, &m_fy1, &m_fy2, &m_q, &m_crx, &m_cry, &m_ra_x, &m_ra_y, &m_xfx, &m_yfx, &m_area, (ElementType)(p1), (ElementType)(p2), &d_, s_, dev_);
  });
}

inline void fvtp2d_fullfusion(Storage3D& q_i, Storage3D& q_j, Storage3D& fx1, Storage3D& fx2, Storage3D& fy1, Storage3D& fy2, const Storage3D& q, const Storage3D& crx, const Storage3D& cry, const Storage3D& ra_x, const Storage3D& ra_y, const Storage3D& xfx, const Storage3D& yfx, const Storage3D& area, Storage3D& fxx, Storage3D& fyy, Storage3D& al, Storage3D& almq, Storage3D& br, Storage3D& b0, Storage3D& smt5) { fvtp2d(q_i, q_j, fx1, fx2, fy1, fy2, q, crx, cry, ra_x, ra_y, xfx, yfx, area, fxx, fyy, al, almq, br, b0, smt5); }

#endif  // FVTP2D_H
