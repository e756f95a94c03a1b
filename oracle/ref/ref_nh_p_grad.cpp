// ref_nh_p_grad.cpp -- reference harness for kernels/nh_p_grad.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/nh_p_grad.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_nh_p_grad_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef NH_P_GRAD_H
#include "nh_p_grad.h"
}  // namespace oebns_nh_p_grad_f64

namespace oebns_nh_p_grad_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef NH_P_GRAD_H
#include "nh_p_grad.h"
}  // namespace oebns_nh_p_grad_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_nh_p_grad_##SUF(int variant, const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdx, const M3* rdy, const M3* gz, const M3* pp, const M3* pk3, const M3* wk1, const M3* wk, const M3* du, const M3* dv, T dt, int64_t n, int64_t nz) { \
    using namespace oebns_nh_p_grad_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_uout = OEB_S3(uout); Storage3D s_vout = OEB_S3(vout); Storage3D s_uin = OEB_S3(uin); Storage3D s_vin = OEB_S3(vin); Storage3D s_rdx = OEB_S3(rdx); Storage3D s_rdy = OEB_S3(rdy); Storage3D s_gz = OEB_S3(gz); Storage3D s_pp = OEB_S3(pp); Storage3D s_pk3 = OEB_S3(pk3); Storage3D s_wk1 = OEB_S3(wk1); Storage3D s_wk = OEB_S3(wk); Storage3D s_du = OEB_S3(du); Storage3D s_dv = OEB_S3(dv);                                                                              \
    switch (variant) {                                                                   \
      case 0: nh_p_grad(s_uout, s_vout, s_uin, s_vin, s_rdx, s_rdy, s_gz, s_pp, s_pk3, s_wk1, s_wk, s_du, s_dv, dt); break; \
      case 1: nh_p_grad_fullfusion(s_uout, s_vout, s_uin, s_vin, s_rdx, s_rdy, s_gz, s_pp, s_pk3, s_wk1, s_wk, s_du, s_dv, dt); break; \
      case 2: nh_p_grad_partialfusion(s_uout, s_vout, s_uin, s_vin, s_rdx, s_rdy, s_gz, s_pp, s_pk3, s_wk1, s_wk, s_du, s_dv, dt); break; \
      default: nh_p_grad_openmp(s_uout, s_vout, s_uin, s_vin, s_rdx, s_rdy, s_gz, s_pp, s_pk3, s_wk1, s_wk, s_du, s_dv, dt); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
