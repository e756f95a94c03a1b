// include/oeb/laplace.h -- drop-in replacement of the reference's kernels/laplace.h (kernels/laplace.h:4).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_laplace_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
#ifndef LAPLACE_H
#define LAPLACE_H

#include "oeb_dropin.hpp"

inline void laplace(const Storage3D& in, Storage3D& out) {
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_in = oeb_dropin::m3(in);
  const auto m_out = oeb_dropin::m3(out);
  oeb_dropin::dispatch(in.alignedPtr, "laplace", [&](void* s_, bool dev_) {
    return oeb_dropin::call_laplace(&m_in, &m_out, &d_, s_, dev_);
  });
}

inline void laplace_fullfusion(const Storage3D& in, Storage3D& out) { laplace(in, out); }

inline void laplace_partialfusion(const Storage3D& in, Storage3D& out) { laplace(in, out); }

inline void laplace_openmp(const Storage3D& in, Storage3D& out) { laplace(in, out); }

#endif  // LAPLACE_H
