// ref_laplace.cpp -- reference harness for kernels/laplace.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/laplace.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_laplace_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef LAPLACE_H
#include "laplace.h"
}  // namespace oebns_laplace_f64

namespace oebns_laplace_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef LAPLACE_H
#include "laplace.h"
}  // namespace oebns_laplace_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_laplace_##SUF(int variant, const M3* in, const M3* out, int64_t n, int64_t nz) { \
    using namespace oebns_laplace_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_in = OEB_S3(in); Storage3D s_out = OEB_S3(out);                                                                              \
    switch (variant) {                                                                   \
      case 0: laplace(s_in, s_out); break; \
      case 1: laplace_fullfusion(s_in, s_out); break; \
      case 2: laplace_partialfusion(s_in, s_out); break; \
      default: laplace_openmp(s_in, s_out); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)

// The reference's own field initialisers (include/util.h:150-196), for golden vectors made
// with the drivers' inputs.  fillMath fills i, j over [-halo, n+halo) and k over [0, nz);
// initValue fills every cell, its k loop bounded by the global domain_height (util.h:193).
extern "C" void oeb_ref_fillmath3_f64(double a, double b, double c, double d, double e, double f,
                                      const oeb_memref3d_f64* m, int64_t n, int64_t nz, int64_t halo) {
  using namespace oebns_laplace_f64;
  halo_width = halo;
  domain_size = n;
  domain_height = nz;
  Storage3D s = OEB_S3(m);
  fillMath(a, b, c, d, e, f, s, n, nz);
}

extern "C" void oeb_ref_fillmath1_f64(double a, double b, double c, double d, double e, double f,
                                      const oeb_memref1d_f64* m, int64_t n, int64_t nz, int64_t halo) {
  using namespace oebns_laplace_f64;
  halo_width = halo;
  domain_size = n;
  domain_height = nz;
  Storage1D s = OEB_S1(m);
  fillMath(a, b, c, d, e, f, s, n, nz);
}

extern "C" void oeb_ref_initvalue3_f64(const oeb_memref3d_f64* m, double val, int64_t n, int64_t nz, int64_t halo) {
  using namespace oebns_laplace_f64;
  halo_width = halo;
  domain_size = n;
  domain_height = nz;
  Storage3D s = OEB_S3(m);
  initValue(s, val, n, nz);
}
