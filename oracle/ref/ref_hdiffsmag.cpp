// ref_hdiffsmag.cpp -- reference harness for kernels/hdiffsmag.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/hdiffsmag.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_hdiffsmag_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef HDIFFSMAG_H
#include "hdiffsmag.h"
}  // namespace oebns_hdiffsmag_f64

namespace oebns_hdiffsmag_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef HDIFFSMAG_H
#include "hdiffsmag.h"
}  // namespace oebns_hdiffsmag_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_hdiffsmag_##SUF(int variant, const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* mask, const M1* crlavo, const M1* crlavu, const M1* crlato, const M1* crlatu, const M1* acrlat0, const M3* T_sqr_s, const M3* S_sqr_uv, T eddlat, T eddlon, T tau_smag, T weight_smag, int64_t n, int64_t nz) { \
    using namespace oebns_hdiffsmag_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_uout = OEB_S3(uout); Storage3D s_vout = OEB_S3(vout); Storage3D s_uin = OEB_S3(uin); Storage3D s_vin = OEB_S3(vin); Storage3D s_mask = OEB_S3(mask); Storage3D s_T_sqr_s = OEB_S3(T_sqr_s); Storage3D s_S_sqr_uv = OEB_S3(S_sqr_uv); Storage1D s_crlavo = OEB_S1(crlavo); Storage1D s_crlavu = OEB_S1(crlavu); Storage1D s_crlato = OEB_S1(crlato); Storage1D s_crlatu = OEB_S1(crlatu); Storage1D s_acrlat0 = OEB_S1(acrlat0);                                                                              \
    switch (variant) {                                                                   \
      case 0: hdiffsmag(s_uout, s_vout, s_uin, s_vin, s_mask, s_crlavo, s_crlavu, s_crlato, s_crlatu, s_acrlat0, s_T_sqr_s, s_S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); break; \
      case 1: hdiffsmag_fullfusion(s_uout, s_vout, s_uin, s_vin, s_mask, s_crlavo, s_crlavu, s_crlato, s_crlatu, s_acrlat0, s_T_sqr_s, s_S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); break; \
      case 2: hdiffsmag_partialfusion(s_uout, s_vout, s_uin, s_vin, s_mask, s_crlavo, s_crlavu, s_crlato, s_crlatu, s_acrlat0, s_T_sqr_s, s_S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); break; \
      default: hdiffsmag_openmp(s_uout, s_vout, s_uin, s_vin, s_mask, s_crlavo, s_crlavu, s_crlato, s_crlatu, s_acrlat0, s_T_sqr_s, s_S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
