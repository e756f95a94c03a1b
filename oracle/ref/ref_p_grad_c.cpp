// ref_p_grad_c.cpp -- reference harness for kernels/p_grad_c.h (TEST INFRASTRUCTURE).
// Compiles the reference's own util.h and kernels/p_grad_c.h from the reference source tree;
// see ref_common.hpp.
#include "ref_common.hpp"

namespace oebns_p_grad_c_f64 {
OEB_REF_GLOBALS(double)

#undef UTIL_H
#include "util.h"
#undef P_GRAD_C_H
#include "p_grad_c.h"
}  // namespace oebns_p_grad_c_f64

namespace oebns_p_grad_c_f32 {
OEB_REF_GLOBALS(float)

#undef UTIL_H
#include "util.h"
#undef P_GRAD_C_H
#include "p_grad_c.h"
}  // namespace oebns_p_grad_c_f32

#define OEB_ENTRY(SUF, M3, M1, T)                                                        \
  extern "C" void oeb_ref_p_grad_c_##SUF(int variant, const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdxc, const M3* rdyc, const M3* delpc, const M3* gz, const M3* pkc, const M3* wk, T dt2, int64_t n, int64_t nz) { \
    using namespace oebns_p_grad_c_##SUF;                                                   \
    domain_size = n;                                                                     \
    domain_height = nz;                                                                  \
    Storage3D s_uout = OEB_S3(uout); Storage3D s_vout = OEB_S3(vout); Storage3D s_uin = OEB_S3(uin); Storage3D s_vin = OEB_S3(vin); Storage3D s_rdxc = OEB_S3(rdxc); Storage3D s_rdyc = OEB_S3(rdyc); Storage3D s_delpc = OEB_S3(delpc); Storage3D s_gz = OEB_S3(gz); Storage3D s_pkc = OEB_S3(pkc); Storage3D s_wk = OEB_S3(wk);                                                                              \
    switch (variant) {                                                                   \
      case 0: p_grad_c(s_uout, s_vout, s_uin, s_vin, s_rdxc, s_rdyc, s_delpc, s_gz, s_pkc, s_wk, dt2); break; \
      case 1: p_grad_c_fullfusion(s_uout, s_vout, s_uin, s_vin, s_rdxc, s_rdyc, s_delpc, s_gz, s_pkc, s_wk, dt2); break; \
      case 2: p_grad_c_partialfusion(s_uout, s_vout, s_uin, s_vin, s_rdxc, s_rdyc, s_delpc, s_gz, s_pkc, s_wk, dt2); break; \
      default: p_grad_c_openmp(s_uout, s_vout, s_uin, s_vin, s_rdxc, s_rdyc, s_delpc, s_gz, s_pkc, s_wk, dt2); break; \
    }                                                                                    \
  }
OEB_ENTRY(f64, oeb_memref3d_f64, oeb_memref1d_f64, double)
OEB_ENTRY(f32, oeb_memref3d_f32, oeb_memref1d_f32, float)
