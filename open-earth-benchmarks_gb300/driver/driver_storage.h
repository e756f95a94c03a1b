// driver_storage.h -- device-resident fields with the reference's Storage interface, for the
// GPU driver (oeb_driver).  The drop-in headers (include/oeb/<k>.h) need a Storage type with
// allocatedPtr, alignedPtr, offset, sizes[] and strides[] (include/util.h:24-31) and the
// globals a reference driver defines (domain_size, domain_height, halo_width, ElementType);
// this header gives them, with the storage on the GPU (oeb_storage3d_alloc_*), so every
// drop-in call runs the device entry point.
#ifndef OEB_DRIVER_STORAGE_H
#define OEB_DRIVER_STORAGE_H

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "oeb_gb300.h"

template <class T, size_t R>
struct Storage {
  T* allocatedPtr;
  T* alignedPtr;
  int64_t offset;
  std::array<int64_t, R> sizes;
  std::array<int64_t, R> strides;
};

namespace oeb_driver {

inline void die(const char* what, int status) {
  std::fprintf(stderr, "oeb_driver: %s: %s\n", what, oeb_status_string(status));
  std::exit(2);
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "oeb_driver: %s: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
}

// The analytic fill of the reference drivers (include/util.h:150-188), over the whole
// allocation: value(i, j, k) = k/100 + a (b + cos(pi (x + c y)) + sin(d pi (x + e y))) / f with
// x = i / (n + 2h), y = j / (n + 2h); 1-D fields use x = j / (n + 2h) and no k term.  Unlike the
// reference, the k-halo planes are filled too (the formula continued), since fastwavesuv,
// nh_p_grad and p_grad_c read k + 1 at the top level.
struct Fill {
  double a, b, c, d, e, f;
};

inline double fill_value(const Fill& p, int64_t i, int64_t j, int64_t k, int64_t n, int64_t h, bool rank1) {
  const double pi = 3.14159265358979323846;
  const double step = 1.0 / (double)(n + 2 * h);
  if (rank1) {
    const double x = step * (double)j;
    return p.a * (p.b + std::cos(pi * (p.c * x)) + std::sin(p.d * pi * (p.e * x))) / p.f;
  }
  const double x = step * (double)i, y = step * (double)j;
  return (double)k * 10e-3 + p.a * (p.b + std::cos(pi * (x + p.c * y)) + std::sin(p.d * pi * (x + p.e * y))) / p.f;
}

template <class T>
struct Alloc;
template <>
struct Alloc<double> {
  static int f3(int64_t nx, int64_t nz, int64_t h, oeb_memref3d_f64* m) { return oeb_storage3d_alloc_f64(nx, nx, nz, h, 1, m); }
  static int f1(int64_t n, int64_t h, oeb_memref1d_f64* m) { return oeb_storage1d_alloc_f64(n, h, m); }
};
template <>
struct Alloc<float> {
  static int f3(int64_t nx, int64_t nz, int64_t h, oeb_memref3d_f32* m) { return oeb_storage3d_alloc_f32(nx, nx, nz, h, 1, m); }
  static int f1(int64_t n, int64_t h, oeb_memref1d_f32* m) { return oeb_storage1d_alloc_f32(n, h, m); }
};

// A square n x n x nz field with halo h on the GPU, filled with `p` (or the constant `value`).
template <class T, class M3>
Storage<T, 3> device3(int64_t n, int64_t nz, int64_t h, const Fill* p, double value) {
  M3 m;
  const int st = Alloc<T>::f3(n, nz, h, &m);
  if (st != OEB_OK) die("allocating a field", st);
  Storage<T, 3> s;
  s.allocatedPtr = m.allocated;
  s.alignedPtr = m.aligned;
  s.offset = m.offset;
  for (int r = 0; r < 3; ++r) {
    s.sizes[r] = m.sizes[r];
    s.strides[r] = m.strides[r];
  }
  const int64_t span = (s.sizes[0] - 1) * s.strides[0] + (s.sizes[1] - 1) * s.strides[1] + s.sizes[2];
  std::vector<T> host((size_t)span, T(value));
  if (p)
    for (int64_t k = -h; k < nz + h; ++k)
      for (int64_t j = -h; j < n + h; ++j)
        for (int64_t i = -h; i < n + h; ++i)
          host[(size_t)(s.offset + k * s.strides[0] + j * s.strides[1] + i)] = T(fill_value(*p, i, j, k, n, h, false));
  cuda_check(cudaMemcpy(s.alignedPtr, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
  return s;
}

template <class T, class M1>
Storage<T, 1> device1(int64_t n, int64_t h, const Fill& p) {
  M1 m;
  const int st = Alloc<T>::f1(n, h, &m);
  if (st != OEB_OK) die("allocating a field", st);
  Storage<T, 1> s;
  s.allocatedPtr = m.allocated;
  s.alignedPtr = m.aligned;
  s.offset = m.offset;
  s.sizes[0] = m.sizes[0];
  s.strides[0] = m.strides[0];
  std::vector<T> host((size_t)s.sizes[0]);
  for (int64_t j = -h; j < n + h; ++j) host[(size_t)(s.offset + j)] = T(fill_value(p, 0, j, 0, n, h, true));
  cuda_check(cudaMemcpy(s.alignedPtr, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
  return s;
}

template <class S>
void release(S& s) {
  cudaFree(s.allocatedPtr);
  s.allocatedPtr = s.alignedPtr = nullptr;
}

// The interior cells [0, n)^2 x [0, nz) of a device field, as doubles in host memory.
template <class T>
std::vector<double> interior(const Storage<T, 3>& s, int64_t n, int64_t nz) {
  const int64_t span = (s.sizes[0] - 1) * s.strides[0] + (s.sizes[1] - 1) * s.strides[1] + s.sizes[2];
  std::vector<T> host((size_t)span);
  cuda_check(cudaMemcpy(host.data(), s.alignedPtr, host.size() * sizeof(T), cudaMemcpyDeviceToHost), "download");
  std::vector<double> out;
  out.reserve((size_t)(n * n * nz));
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i)
        out.push_back((double)host[(size_t)(s.offset + k * s.strides[0] + j * s.strides[1] + i)]);
  return out;
}

// One timed kernel run, as the reference's timer prints it plus a JSON line.
struct Result {
  const char* kernel;
  const char* variant;
  int count;
  double total_ms;
  int64_t points;
  int fields;  // 3-D inputs + semantic outputs: the algorithmic bytes are fields x points x sizeof(T)
  bool adjoint;  // each timed call was the forward variant followed by the kernel's adjoint
  // the semantic outputs' interiors after the timed calls (when asked for), for error columns
  std::vector<std::vector<double>> outputs;
};

}  // namespace oeb_driver

#endif  // OEB_DRIVER_STORAGE_H
