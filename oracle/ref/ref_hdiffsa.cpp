// ref_hdiffsa.cpp -- reference harness for kernels/hdiffsa.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/hdiffsa.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_hdiffsa_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef HDIFFSA_H
#include "hdiffsa.h"
}  // namespace oebns_hdiffsa_f64

namespace oebns_hdiffsa_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef HDIFFSA_H
#include "hdiffsa.h"
}  // namespace oebns_hdiffsa_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_hdiffsa_##SUF(int variant, const M3* out, const M3* in, const M3* mask, const M1* crlato, const M1* crlatu, const M3* lap, const M3* flx, const M3* fly, int64_t n, int64_t nz) { \
    using namespace oebns_hdiffsa_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_out = OEB_S3(out); Storage3D s_in = OEB_S3(in); Storage3D s_mask = OEB_S3(mask); Storage3D s_lap = OEB_S3(lap); Storage3D s_flx = OEB_S3(flx); Storage3D s_fly = OEB_S3(fly); Storage1D s_crlato = OEB_S1(crlato); Storage1D s_crlatu = OEB_S1(crlatu);                                                                              \
    switch (variant) {                                                                   \
      case 0: hdiffsa(s_out, s_in, s_mask, s_crlato, s_crlatu, s_lap, s_flx, s_fly); break; \
      case 1: hdiffsa_fullfusion(s_out, s_in, s_mask, s_crlato, s_crlatu, s_lap, s_flx, s_fly); break; \
      case 2: hdiffsa_partialfusion(s_out, s_in, s_mask, s_crlato, s_crlatu, s_lap, s_flx, s_fly); break; \
      default: hdiffsa_openmp(s_out, s_in, s_mask, s_crlato, s_crlatu, s_lap, s_flx, s_fly); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
