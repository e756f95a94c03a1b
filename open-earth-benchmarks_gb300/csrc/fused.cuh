// fused.cuh -- the chained step's fused stages (fusion grouping OEB_FUSE_HADV_UPDATE), internal
// to the library: defined in k_pointwise.cu, called by chain.cu.
//
// hadvuv5th_update: hadvuv5th with the explicit update in its epilogue, u2 = alpha * (the
// tendency) + u1 and v2 likewise, written over the same box as the separate update kernel.
// hadvuv5th_adj_update: the hadvuv5th adjoint whose gather adds the update's transpose,
// u1b = alpha * (the gathered gradient) + (u2b inside the interior).  Each computes the bits
// of the two separate kernels: the same operations on the same operands, in the same order.
#pragma once

#include "oeb_common.cuh"

namespace oeb {

oeb_status hadvuv5th_update(const oeb_memref3d_f64* u2, const oeb_memref3d_f64* v2, const oeb_memref3d_f64* u1,
                            const oeb_memref3d_f64* v1, const oeb_memref1d_f64* acrlat0,
                            const oeb_memref1d_f64* acrlat1, const oeb_memref1d_f64* tgrlatda0,
                            const oeb_memref1d_f64* tgrlatda1, double eddlat, double eddlon, double alpha,
                            const oeb_domain* dom, void* stream);
oeb_status hadvuv5th_update(const oeb_memref3d_f32* u2, const oeb_memref3d_f32* v2, const oeb_memref3d_f32* u1,
                            const oeb_memref3d_f32* v1, const oeb_memref1d_f32* acrlat0,
                            const oeb_memref1d_f32* acrlat1, const oeb_memref1d_f32* tgrlatda0,
                            const oeb_memref1d_f32* tgrlatda1, float eddlat, float eddlon, float alpha,
                            const oeb_domain* dom, void* stream);
oeb_status hadvuv5th_adj_update(const oeb_memref3d_f64* u1b, const oeb_memref3d_f64* v1b,
                                const oeb_memref3d_f64* u1, const oeb_memref3d_f64* v1,
                                const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1,
                                const oeb_memref3d_f64* u2b, const oeb_memref3d_f64* v2b, double eddlat,
                                double eddlon, double alpha, const oeb_domain* dom, void* stream);
oeb_status hadvuv5th_adj_update(const oeb_memref3d_f32* u1b, const oeb_memref3d_f32* v1b,
                                const oeb_memref3d_f32* u1, const oeb_memref3d_f32* v1,
                                const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1,
                                const oeb_memref3d_f32* u2b, const oeb_memref3d_f32* v2b, float eddlat,
                                float eddlon, float alpha, const oeb_domain* dom, void* stream);

}  // namespace oeb
