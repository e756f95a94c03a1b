// ref_uvbke.cpp -- reference harness for kernels/uvbke.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/uvbke.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_uvbke_f64 {
OEB_REF_GLOBALS(double)
double dt5 = 0.5 * 225.0;  // src/uvbke.cpp:11-12 (a double even when ElementType is float); set per call
#undef UTIL_H
#include "util.h"
#undef UVBKE_H
#include "uvbke.h"
}  // namespace oebns_uvbke_f64

namespace oebns_uvbke_f32 {
OEB_REF_GLOBALS(float)
double dt5 = 0.5 * 225.0;  // src/uvbke.cpp:11-12 (a double even when ElementType is float); set per call
#undef UTIL_H
#include "util.h"
#undef UVBKE_H
#include "uvbke.h"
}  // namespace oebns_uvbke_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_uvbke_##SUF(int variant, const M3* ub, const M3* vb, const M3* uc, const M3* vc, const M3* cosa, const M3* rsina, double dt5_value, int64_t n, int64_t nz) { \
    using namespace oebns_uvbke_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_ub = OEB_S3(ub); Storage3D s_vb = OEB_S3(vb); Storage3D s_uc = OEB_S3(uc); Storage3D s_vc = OEB_S3(vc); Storage3D s_cosa = OEB_S3(cosa); Storage3D s_rsina = OEB_S3(rsina); dt5 = dt5_value;                                                                              \
    switch (variant) {                                                                   \
      case 0: uvbke(s_ub, s_vb, s_uc, s_vc, s_cosa, s_rsina); break; \
      case 1: uvbke_fullfusion(s_ub, s_vb, s_uc, s_vc, s_cosa, s_rsina); break; \
      case 2: uvbke_partialfusion(s_ub, s_vb, s_uc, s_vc, s_cosa, s_rsina); break; \
      default: uvbke_openmp(s_ub, s_vb, s_uc, s_vc, s_cosa, s_rsina); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
