// storage_compat.h -- a field type with the reference's Storage layout (include/util.h:24-31)
// and accessor (util.h:82-94), written for the drop-in driver test, which runs where the
// reference's util.h is not available.  The drop-in headers need exactly this interface:
// allocatedPtr, alignedPtr, offset, sizes[], strides[] and the globals a reference driver
// defines (domain_size, domain_height, halo_width, ElementType).
#ifndef STORAGE_COMPAT_H
#define STORAGE_COMPAT_H

#include <array>
#include <cstdint>
#include <vector>

template <class T, size_t R>
struct Storage {
  T* allocatedPtr;
  T* alignedPtr;
  int64_t offset;
  std::array<int64_t, R> sizes;
  std::array<int64_t, R> strides;
  T& at(int64_t i, int64_t j, int64_t k) { return alignedPtr[offset + strides[2] * i + strides[1] * j + strides[0] * k]; }
  T& at(int64_t j) { return alignedPtr[offset + strides[0] * j]; }
};

typedef Storage<ElementType, 1> Storage1D;
typedef Storage<ElementType, 3> Storage3D;

// The reference's allocation formula (util.h:126-141): sizes k-first, halo in every
// dimension, alignedPtr = allocatedPtr + (32 - halo).
inline Storage3D make3(int64_t n, int64_t nz, int64_t h, std::vector<ElementType>& buf) {
  Storage3D s;
  s.sizes = {nz + 2 * h, n + 2 * h, n + 2 * h};
  s.strides = {s.sizes[2] * s.sizes[1], s.sizes[2], 1};
  s.offset = h * s.strides[0] + h * s.strides[1] + h;
  buf.assign((size_t)(s.sizes[0] * s.sizes[1] * s.sizes[2] + (32 - h)), ElementType(0));
  s.allocatedPtr = buf.data();
  s.alignedPtr = buf.data() + (32 - h);
  return s;
}

inline Storage1D make1(int64_t n, int64_t h, std::vector<ElementType>& buf) {
  Storage1D s;
  s.sizes = {n + 2 * h};
  s.strides = {1};
  s.offset = h;
  buf.assign((size_t)(n + 2 * h + (32 - h)), ElementType(0));
  s.allocatedPtr = buf.data();
  s.alignedPtr = buf.data() + (32 - h);
  return s;
}

#endif
