// ref_fvtp2d.cpp -- reference harness for kernels/fvtp2d.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/fvtp2d.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"
// src/fvtp2d.cpp:11-12 define p1/p2 as ElementType literals; here they name a per-namespace
// variable holding the same ElementType value, so that a call can set them.
#define p1 oeb_p1
#define p2 oeb_p2
namespace oebns_fvtp2d_f64 {
OEB_REF_GLOBALS(double)
ElementType oeb_p1 = ElementType(0.583333);
ElementType oeb_p2 = ElementType(0.083333);
#undef UTIL_H
#include "util.h"
#undef FVTP2D_H
#include "fvtp2d.h"
}  // namespace oebns_fvtp2d_f64

namespace oebns_fvtp2d_f32 {
OEB_REF_GLOBALS(float)
ElementType oeb_p1 = ElementType(0.583333);
ElementType oeb_p2 = ElementType(0.083333);
#undef UTIL_H
#include "util.h"
#undef FVTP2D_H
#include "fvtp2d.h"
}  // namespace oebns_fvtp2d_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_fvtp2d_##SUF(int variant, const M3* q_i, const M3* q_j, const M3* fx1, const M3* fx2, const M3* fy1, const M3* fy2, const M3* q, const M3* crx, const M3* cry, const M3* ra_x, const M3* ra_y, const M3* xfx, const M3* yfx, const M3* area, const M3* fxx, const M3* fyy, const M3* al, const M3* almq, const M3* br, const M3* b0, const M3* smt5, T p1_value, T p2_value, int64_t n, int64_t nz) { \
    using namespace oebns_fvtp2d_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_q_i = OEB_S3(q_i); Storage3D s_q_j = OEB_S3(q_j); Storage3D s_fx1 = OEB_S3(fx1); Storage3D s_fx2 = OEB_S3(fx2); Storage3D s_fy1 = OEB_S3(fy1); Storage3D s_fy2 = OEB_S3(fy2); Storage3D s_q = OEB_S3(q); Storage3D s_crx = OEB_S3(crx); Storage3D s_cry = OEB_S3(cry); Storage3D s_ra_x = OEB_S3(ra_x); Storage3D s_ra_y = OEB_S3(ra_y); Storage3D s_xfx = OEB_S3(xfx); Storage3D s_yfx = OEB_S3(yfx); Storage3D s_area = OEB_S3(area); Storage3D s_fxx = OEB_S3(fxx); Storage3D s_fyy = OEB_S3(fyy); Storage3D s_al = OEB_S3(al); Storage3D s_almq = OEB_S3(almq); Storage3D s_br = OEB_S3(br); Storage3D s_b0 = OEB_S3(b0); Storage3D s_smt5 = OEB_S3(smt5); oeb_p1 = p1_value; oeb_p2 = p2_value;                                                                              \
    switch (variant) {                                                                   \
      case 1: fvtp2d_fullfusion(s_q_i, s_q_j, s_fx1, s_fx2, s_fy1, s_fy2, s_q, s_crx, s_cry, s_ra_x, s_ra_y, s_xfx, s_yfx, s_area, s_fxx, s_fyy, s_al, s_almq, s_br, s_b0, s_smt5); break; \
      default: fvtp2d(s_q_i, s_q_j, s_fx1, s_fx2, s_fy1, s_fy2, s_q, s_crx, s_cry, s_ra_x, s_ra_y, s_xfx, s_yfx, s_area, s_fxx, s_fyy, s_al, s_almq, s_br, s_b0, s_smt5); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
