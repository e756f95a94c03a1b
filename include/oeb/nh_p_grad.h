// include/oeb/nh_p_grad.h -- drop-in replacement of the reference's kernels/nh_p_grad.h (kernels/nh_p_grad.h:4-6).
//
// Same functions, same signatures, same include guard; each runs the GB300 stencil through
// the C ABI (oeb_nh_p_grad_f64 / _f32, device or host buffers) -- see oeb_dropin.hpp.  Include it
// after util.h, as the reference kernels are.
#ifndef NH_P_GRAD_H
#define NH_P_GRAD_H

#include "oeb_dropin.hpp"

inline void nh_p_grad(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdx, const Storage3D& rdy, const Storage3D& gz, const Storage3D& pp, const Storage3D& pk3, const Storage3D& wk1, Storage3D& wk, Storage3D& du, Storage3D& dv, const ElementType dt) {
  (void)wk; (void)du; (void)dv;  // scratch of the reference signature: not used
  const oeb_domain d_ = oeb_dropin::domain(domain_size, domain_height);
  const auto m_uout = oeb_dropin::m3(uout);
  const auto m_vout = oeb_dropin::m3(vout);
  const auto m_uin = oeb_dropin::m3(uin);
  const auto m_vin = oeb_dropin::m3(vin);
  const auto m_rdx = oeb_dropin::m3(rdx);
  const auto m_rdy = oeb_dropin::m3(rdy);
  const auto m_gz = oeb_dropin::m3(gz);
  const auto m_pp = oeb_dropin::m3(pp);
  const auto m_pk3 = oeb_dropin::m3(pk3);
  const auto m_wk1 = oeb_dropin::m3(wk1);
  oeb_dropin::dispatch(uin.alignedPtr, "nh_p_grad", [&](void* s_, bool dev_) {
    return oeb_dropin::call_nh_p_grad(&m_uout, &m_vout, &m_uin, &m_vin, &m_rdx, &m_rdy, &m_gz, &m_pp, &m_pk3, &m_wk1, dt, &d_, s_, dev_);
  });
}

inline void nh_p_grad_fullfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdx, const Storage3D& rdy, const Storage3D& gz, const Storage3D& pp, const Storage3D& pk3, const Storage3D& wk1, Storage3D& wk, Storage3D& du, Storage3D& dv, const ElementType dt) { nh_p_grad(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, wk, du, dv, dt); }

inline void nh_p_grad_partialfusion(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdx, const Storage3D& rdy, const Storage3D& gz, const Storage3D& pp, const Storage3D& pk3, const Storage3D& wk1, Storage3D& wk, Storage3D& du, Storage3D& dv, const ElementType dt) { nh_p_grad(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, wk, du, dv, dt); }

inline void nh_p_grad_openmp(Storage3D& uout, Storage3D& vout, const Storage3D& uin, const Storage3D& vin, const Storage3D& rdx, const Storage3D& rdy, const Storage3D& gz, const Storage3D& pp, const Storage3D& pk3, const Storage3D& wk1, Storage3D& wk, Storage3D& du, Storage3D& dv, const ElementType dt) { nh_p_grad(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, wk, du, dv, dt); }

#endif  // NH_P_GRAD_H
