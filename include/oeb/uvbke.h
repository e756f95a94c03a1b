// include/oeb/uvbke.h -- drop-in replacement of the reference's kernels/uvbke.h (kernels/uvbke.h:4-5).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_uvbke_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
// Reads the driver's dt5, as the reference does (src/uvbke.cpp:11-12).
#ifndef UVBKE_H
#define UVBKE_H

#include "oeb_dropin.hpp"

inline void uvbke(Storage3D& ub, Storage3D& vb, const Storage3D& uc, const Storage3D& vc, const Storage3D& cosa, const Storage3D& rsina) {
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_ub = oeb_dropin::m3(ub);
  const auto m_vb = oeb_dropin::m3(vb);
  const auto m_uc = oeb_dropin::m3(uc);
  const auto m_vc = oeb_dropin::m3(vc);
  const auto m_cosa = oeb_dropin::m3(cosa);
  const auto m_rsina = oeb_dropin::m3(rsina);
  oeb_dropin::dispatch(uc.alignedPtr, "uvbke", [&](void* s_, bool dev_) {
    return oeb_dropin::call_uvbke(&m_ub, &m_vb, &m_uc, &m_vc, &m_cosa, &m_rsina, (double)(dt5), &d_, s_, dev_);
  });
}

inline void uvbke_fullfusion(Storage3D& ub, Storage3D& vb, const Storage3D& uc, const Storage3D& vc, const Storage3D& cosa, const Storage3D& rsina) { uvbke(ub, vb, uc, vc, cosa, rsina); }

inline void uvbke_partialfusion(Storage3D& ub, Storage3D& vb, const Storage3D& uc, const Storage3D& vc, const Storage3D& cosa, const Storage3D& rsina) { uvbke(ub, vb, uc, vc, cosa, rsina); }

inline void uvbke_openmp(Storage3D& ub, Storage3D& vb, const Storage3D& uc, const Storage3D& vc, const Storage3D& cosa, const Storage3D& rsina) { uvbke(ub, vb, uc, vc, cosa, rsina); }

#endif  // UVBKE_H
