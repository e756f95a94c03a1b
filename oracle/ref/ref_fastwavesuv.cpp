// ref_fastwavesuv.cpp -- reference harness for kernels/fastwavesuv.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/fastwavesuv.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_fastwavesuv_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef FASTWAVESUV_H
#include "fastwavesuv.h"
}  // namespace oebns_fastwavesuv_f64

namespace oebns_fastwavesuv_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef FASTWAVESUV_H
#include "fastwavesuv.h"
}  // namespace oebns_fastwavesuv_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_fastwavesuv_##SUF(int variant, const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* utens, const M3* vtens, const M3* wgtfac, const M3* ppuv, const M3* hhl, const M3* rho, const M1* fx, const M3* ppgk, const M3* ppgc, const M3* ppgu, const M3* ppgv, T edadlat, T dt, int64_t n, int64_t nz) { \
    using namespace oebns_fastwavesuv_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_uout = OEB_S3(uout); Storage3D s_vout = OEB_S3(vout); Storage3D s_uin = OEB_S3(uin); Storage3D s_vin = OEB_S3(vin); Storage3D s_utens = OEB_S3(utens); Storage3D s_vtens = OEB_S3(vtens); Storage3D s_wgtfac = OEB_S3(wgtfac); Storage3D s_ppuv = OEB_S3(ppuv); Storage3D s_hhl = OEB_S3(hhl); Storage3D s_rho = OEB_S3(rho); Storage3D s_ppgk = OEB_S3(ppgk); Storage3D s_ppgc = OEB_S3(ppgc); Storage3D s_ppgu = OEB_S3(ppgu); Storage3D s_ppgv = OEB_S3(ppgv); Storage1D s_fx = OEB_S1(fx);                                                                              \
    switch (variant) {                                                                   \
      case 0: fastwavesuv(s_uout, s_vout, s_uin, s_vin, s_utens, s_vtens, s_wgtfac, s_ppuv, s_hhl, s_rho, s_fx, s_ppgk, s_ppgc, s_ppgu, s_ppgv, edadlat, dt); break; \
      case 1: fastwavesuv_fullfusion(s_uout, s_vout, s_uin, s_vin, s_utens, s_vtens, s_wgtfac, s_ppuv, s_hhl, s_rho, s_fx, s_ppgk, s_ppgc, s_ppgu, s_ppgv, edadlat, dt); break; \
      case 2: fastwavesuv_partialfusion(s_uout, s_vout, s_uin, s_vin, s_utens, s_vtens, s_wgtfac, s_ppuv, s_hhl, s_rho, s_fx, s_ppgk, s_ppgc, s_ppgu, s_ppgv, edadlat, dt); break; \
      default: fastwavesuv_openmp(s_uout, s_vout, s_uin, s_vin, s_utens, s_vtens, s_wgtfac, s_ppuv, s_hhl, s_rho, s_fx, s_ppgk, s_ppgc, s_ppgu, s_ppgv, edadlat, dt); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
