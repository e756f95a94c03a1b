// ref_hadvuv.cpp -- reference harness for kernels/hadvuv.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/hadvuv.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_hadvuv_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef HADVUV_H
#include "hadvuv.h"
}  // namespace oebns_hadvuv_f64

namespace oebns_hadvuv_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef HADVUV_H
#include "hadvuv.h"
}  // namespace oebns_hadvuv_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_hadvuv_##SUF(int variant, const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M1* acrlat0, const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, const M3* uatupos, const M3* vatupos, const M3* uatvpos, const M3* vatvpos, const M3* uavg, const M3* vavg, const M3* ures, const M3* vres, T eddlat, T eddlon, int64_t n, int64_t nz) { \
    using namespace oebns_hadvuv_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_uout = OEB_S3(uout); Storage3D s_vout = OEB_S3(vout); Storage3D s_uin = OEB_S3(uin); Storage3D s_vin = OEB_S3(vin); Storage3D s_uatupos = OEB_S3(uatupos); Storage3D s_vatupos = OEB_S3(vatupos); Storage3D s_uatvpos = OEB_S3(uatvpos); Storage3D s_vatvpos = OEB_S3(vatvpos); Storage3D s_uavg = OEB_S3(uavg); Storage3D s_vavg = OEB_S3(vavg); Storage3D s_ures = OEB_S3(ures); Storage3D s_vres = OEB_S3(vres); Storage1D s_acrlat0 = OEB_S1(acrlat0); Storage1D s_acrlat1 = OEB_S1(acrlat1); Storage1D s_tgrlatda0 = OEB_S1(tgrlatda0); Storage1D s_tgrlatda1 = OEB_S1(tgrlatda1);                                                                              \
    switch (variant) {                                                                   \
      case 0: hadvuv(s_uout, s_vout, s_uin, s_vin, s_acrlat0, s_acrlat1, s_tgrlatda0, s_tgrlatda1, s_uatupos, s_vatupos, s_uatvpos, s_vatvpos, s_uavg, s_vavg, s_ures, s_vres, eddlat, eddlon); break; \
      case 1: hadvuv_fullfusion(s_uout, s_vout, s_uin, s_vin, s_acrlat0, s_acrlat1, s_tgrlatda0, s_tgrlatda1, s_uatupos, s_vatupos, s_uatvpos, s_vatvpos, s_uavg, s_vavg, s_ures, s_vres, eddlat, eddlon); break; \
      case 2: hadvuv_partialfusion(s_uout, s_vout, s_uin, s_vin, s_acrlat0, s_acrlat1, s_tgrlatda0, s_tgrlatda1, s_uatupos, s_vatupos, s_uatvpos, s_vatvpos, s_uavg, s_vavg, s_ures, s_vres, eddlat, eddlon); break; \
      default: hadvuv_openmp(s_uout, s_vout, s_uin, s_vin, s_acrlat0, s_acrlat1, s_tgrlatda0, s_tgrlatda1, s_uatupos, s_vatupos, s_uatvpos, s_vatvpos, s_uavg, s_vavg, s_ures, s_vres, eddlat, eddlon); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
