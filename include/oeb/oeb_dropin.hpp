// oeb_dropin.hpp -- shared adapter of the drop-in kernel headers in include/oeb/.
//
// include/oeb/<k>.h replaces the reference's kernels/<k>.h: same function names, same
// signatures (Storage3D& / Storage1D& / ElementType), same include guards.  A driver built
// like the reference's src/<k>.cpp -- globals domain_size, domain_height, halo_width and the
// ElementType typedef defined, then util.h included, then the kernel header -- switches to
// the GB300 library by putting include/oeb/ on the include path instead of kernels/ and
// linking liboeb_gb300.so.  Nothing else in the driver changes.
//
// Each function converts its Storage descriptors field by field into oeb_memref
// descriptors (the layouts are identical, include/util.h:24-31), takes the interior
// extents from the driver's globals (domain_size x domain_size x domain_height, as the
// reference kernels do), and calls
//   * oeb_<k>_<f64|f32>       when the fields are in device memory (then synchronises the
//                             default stream, unless OEB_DROPIN_ASYNC is defined), or
//   * oeb_<k>_<f64|f32>_host  when they are in host memory (staged copies).
// The scratch arguments of the reference signatures are accepted and not touched.
//
// The reference functions return nothing and check nothing.  Here a failed call prints the
// library's status text to stderr and aborts, unless OEB_DROPIN_NOABORT is defined, in
// which case the status is left in oeb_dropin::last_status() and the call returns.
#ifndef OEB_DROPIN_HPP
#define OEB_DROPIN_HPP

#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "../oeb_gb300.h"
#include "oeb_dropin_calls.hpp"

namespace oeb_dropin {

inline int& last_status_ref() {
  static thread_local int s = 0;
  return s;
}
inline int last_status() { return last_status_ref(); }

inline void report(int status, const char* what) {
  last_status_ref() = status;
  if (status == OEB_OK) return;
#ifndef OEB_DROPIN_NOABORT
  std::fprintf(stderr, "%s: %s %s\n", what, oeb_status_string(status),
               status == OEB_ERR_CUDA ? oeb_last_cuda_error() : "");
  std::abort();
#endif
}

template <class T>
struct MemrefOf;
template <>
struct MemrefOf<double> {
  using M3 = oeb_memref3d_f64;
  using M1 = oeb_memref1d_f64;
};
template <>
struct MemrefOf<float> {
  using M3 = oeb_memref3d_f32;
  using M1 = oeb_memref1d_f32;
};

template <class S>
using ElemOf = typename std::remove_cv<typename std::remove_pointer<decltype(S::alignedPtr)>::type>::type;

// Storage<T,3> -> oeb_memref3d_{f64,f32}: the same five fields (include/util.h:24-31).
template <class S>
inline typename MemrefOf<ElemOf<S>>::M3 m3(const S& s) {
  typename MemrefOf<ElemOf<S>>::M3 m;
  m.allocated = s.allocatedPtr;
  m.aligned = s.alignedPtr;
  m.offset = s.offset;
  for (int r = 0; r < 3; ++r) {
    m.sizes[r] = s.sizes[r];
    m.strides[r] = s.strides[r];
  }
  return m;
}

// Storage<T,1> -> oeb_memref1d_{f64,f32}.
template <class S>
inline typename MemrefOf<ElemOf<S>>::M1 m1(const S& s) {
  typename MemrefOf<ElemOf<S>>::M1 m;
  m.allocated = s.allocatedPtr;
  m.aligned = s.alignedPtr;
  m.offset = s.offset;
  m.sizes[0] = s.sizes[0];
  m.strides[0] = s.strides[0];
  return m;
}

// Interior extents from the driver's globals (src/<k>.cpp:4-5).
inline oeb_domain domain(long long size, long long height) {
  oeb_domain d;
  d.nx = size;
  d.ny = size;
  d.nz = height;
  return d;
}

// Runs `call(stream, on_device)` with on_device chosen by where `probe` lives: the device
// entry point for device memory (then the default stream is synchronised, unless
// OEB_DROPIN_ASYNC is defined), the host-buffer entry point otherwise.
template <class Call>
inline void dispatch(const void* probe, const char* what, Call&& call) {
  if (oeb_is_device_pointer(probe)) {
    int st = call((void*)0, true);
#ifndef OEB_DROPIN_ASYNC
    if (st == OEB_OK) st = oeb_stream_synchronize((void*)0);
#endif
    report(st, what);
  } else {
    report(call((void*)0, false), what);
  }
}

}  // namespace oeb_dropin

#endif  // OEB_DROPIN_HPP
