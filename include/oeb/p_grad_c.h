// include/oeb/p_grad_c.h -- drop-in replacement of the reference's kernels/p_grad_c.h (kernels/p_grad_c.h:4-6).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_p_grad_c_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
// p_grad_c (default variant) reads an unset halo of its scratch wk in the reference
// (kernels/p_grad_c.h:8-21); every variant here computes the openmp result.
#ifndef P_GRAD_C_H
#define P_GRAD_C_H

#include "oeb_dropin.hpp"

inline void p_grad_c(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdxc, const Storage3D& rdyc, const Storage3D& delpc, const Storage3D& gz, const Storage3D& pkc, Storage3D& wk, const ElementType dt2) {
  (void)wk;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_uout = oeb_dropin::m3(uout);
  const auto m_vout = oeb_dropin::m3(vout);
  const auto m_uin = oeb_dropin::m3(uin);
  const auto m_vin = oeb_dropin::m3(vin);
  const auto m_rdxc = oeb_dropin::m3(rdxc);
  const auto m_rdyc = oeb_dropin::m3(rdyc);
  const auto m_delpc = oeb_dropin::m3(delpc);
  const auto m_gz = oeb_dropin::m3(gz);
  const auto m_pkc = oeb_dropin::m3(pkc);
  oeb_dropin::dispatch(uin.alignedPtr, "p_grad_c", [&](void* s_, bool dev_) {
    return oeb_dropin::call_p_grad_c(&m_uout, &m_vout, &m_uin, &m_vin, &m_rdxc, &m_rdyc, &m_delpc, &m_gz, &m_pkc, dt2, &d_, s_, dev_);
  });
}

inline void p_grad_c_fullfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdxc, const Storage3D& rdyc, const Storage3D& delpc, const Storage3D& gz, const Storage3D& pkc, Storage3D& wk, const ElementType dt2) { p_grad_c(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, wk, dt2); }

inline void p_grad_c_partialfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdxc, const Storage3D& rdyc, const Storage3D& delpc, const Storage3D& gz, const Storage3D& pkc, Storage3D& wk, const ElementType dt2) { p_grad_c(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, wk, dt2); }

inline void p_grad_c_openmp(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdxc, const Storage3D& rdyc, const Storage3D& delpc, const Storage3D& gz, const Storage3D& pkc, Storage3D& wk, const ElementType dt2) { p_grad_c(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, wk, dt2); }

#endif  // P_GRAD_C_H
