// ref_common.hpp -- shared preamble of the reference harness (TEST INFRASTRUCTURE).
//
// Each oracle/ref/ref_<k>.cpp includes the reference's own include/util.h and
// kernels/<k>.h, straight from the reference source tree (the include path is set by
// oracle/build.py; nothing is copied), inside one namespace per element type, after the
// globals every reference driver defines before including util.h (src/<k>.cpp:4-9).
// The namespaces let the non-inline util.h definitions and the two advectionDriver
// functions (kernels/hadvuv.h:4, kernels/hadvuv5th.h:4) coexist in one shared library.
// The exported extern "C" functions take the same descriptors as the oracle plus a
// variant number (util.h:10-13: 0 default, 1 full fusion, 2 partial fusion, 3 openmp).
#pragma once

#include <sys/time.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <unordered_map>

#include "../../include/oeb_gb300.h"

namespace oeb_ref {
template <class S, class M>
S to_storage(const M* m) {
  S s;
  s.allocatedPtr = m->allocated;
  s.alignedPtr = m->aligned;
  s.offset = m->offset;
  for (size_t r = 0; r < s.sizes.size(); ++r) {
    s.sizes[r] = m->sizes[r];
    s.strides[r] = m->strides[r];
  }
  return s;
}
}  // namespace oeb_ref

// Globals of src/<k>.cpp:4-9; domain_size and domain_height are set per call.
#define OEB_REF_GLOBALS(TYPE)  \
  int64_t domain_size = 64;    \
  int64_t domain_height = 60;  \
  int64_t halo_width = 4;      \
  int64_t count = 1;           \
  typedef TYPE ElementType;

#define OEB_S3(x) oeb_ref::to_storage<Storage3D>(x)
#define OEB_S1(x) oeb_ref::to_storage<Storage1D>(x)
