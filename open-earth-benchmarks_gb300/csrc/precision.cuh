// precision.cuh -- what changes between the FP64 and the FP32 stencils.
//
// FP64 (Prec<double>): the reference's own arithmetic, operation for operation, so that with
// FP contraction off the results are bit-identical to the reference's OpenMP kernels.
//
// FP32 (Prec<float>): fields stored and computed in FP32, with two safeguards:
//  * branch tests on the sign of a product -- the hdiffsa flux limiter (hdiffsa.h:106-113)
//    and the fvtp2d PPM monotonicity flag (fvtp2d.h:23) -- are decided on the exact
//    product, which is what an FP64 product of two floats gives (it is exact in FP64 and
//    cannot underflow); here without any FP64 instruction, from the operands' signs;
//  * the sums whose large terms cancel -- the flux sums of hdiffsmag (its laplacians,
//    hdiffsmag.h:239-241, 254-256) and of the advection drivers (hadvuv.h:10-24,
//    hadvuv5th.h:10-36) and the laplacian (laplace.h:39) -- are accumulated with
//    error-free transformations (TwoSum, and TwoProduct via fmaf), i.e. compensated
//    summation, so cancellation between their large terms does not cost FP32 digits;
//  * the paired products of the pressure gradients (nh_p_grad.h:126-142,
//    p_grad_c.h:90-97) are evaluated in float-float (diff_dot below).
#pragma once

#include <cuda_runtime.h>

namespace oeb {

template <class T>
struct Prec;

template <>
struct Prec<double> {
  static constexpr bool kCompensated = false;
  // reference semantics: the rounded FP64 product compared with 0 (hdiffsa.h:106, fvtp2d.h:23)
  __device__ static __forceinline__ bool prod_gt0(double a, double b) { return a * b > 0; }
  __device__ static __forceinline__ bool prod_lt0(double a, double b) { return (a * b) < 0.0; }
  __device__ static __forceinline__ double sqrt_(double x) { return sqrt(x); }
};

template <>
struct Prec<float> {
  static constexpr bool kCompensated = true;
  // sign of the exact product; NaN operands compare false, as in the FP64 test
  __device__ static __forceinline__ bool prod_gt0(float a, float b) {
    return (a > 0.f && b > 0.f) || (a < 0.f && b < 0.f);
  }
  __device__ static __forceinline__ bool prod_lt0(float a, float b) {
    return (a > 0.f && b < 0.f) || (a < 0.f && b > 0.f);
  }
  __device__ static __forceinline__ float sqrt_(float x) { return sqrtf(x); }
};

// Left-to-right sum of terms.  Plain for FP64 (the reference's order and rounding); for FP32
// a compensated sum: every addition is a TwoSum and every product a TwoProduct, the
// rounding errors are summed separately and added back at the end.
template <class T, bool C = Prec<T>::kCompensated>
struct Acc {
  T s;
  __device__ __forceinline__ explicit Acc(T x) : s(x) {}
  __device__ __forceinline__ static Acc prod(T a, T b) { return Acc(a * b); }
  __device__ __forceinline__ void add(T x) { s = s + x; }
  __device__ __forceinline__ void add_prod(T a, T b) { s = s + a * b; }
  __device__ __forceinline__ T get() const { return s; }
};

template <>
struct Acc<float, true> {
  float s, c;
  __device__ __forceinline__ explicit Acc(float x) : s(x), c(0.f) {}
  __device__ __forceinline__ static Acc prod(float a, float b) {
    Acc r(a * b);
    r.c = fmaf(a, b, -r.s);
    return r;
  }
  // TwoSum (Knuth): s + x = t + e exactly
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    const float bb = t - s;
    const float e = (s - (t - bb)) + (x - bb);
    s = t;
    c += e;
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    c += fmaf(a, b, -p);
    add(p);
  }
  __device__ __forceinline__ float get() const { return s + c; }
};

namespace detail {
// TwoSum (Knuth): a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
}  // namespace detail

// (a - b) * (c - d) + (e - f) * (g - h): the paired products of the pressure-gradient
// stencils (nh_p_grad.h:126-142, p_grad_c.h:90-97), whose two products nearly cancel.
// FP64: exactly these operations in this order, the reference's expression tree.  FP32:
// the four differences and the two products are error-free transformations (TwoSum,
// TwoProduct via fmaf), and the rounding terms are summed apart and added at the end --
// float-float evaluation -- so neither the cancellation nor the rounding of the differences
// (of values up to several times apart) costs FP32 digits.
template <class T>
__device__ __forceinline__ T diff_dot(T a, T b, T c, T d, T e, T f, T g, T h) {
  if constexpr (Prec<T>::kCompensated) {
    float x, xl, y, yl, z, zl, w, wl;
    detail::two_sum(a, -b, x, xl);
    detail::two_sum(c, -d, y, yl);
    detail::two_sum(e, -f, z, zl);
    detail::two_sum(g, -h, w, wl);
    const float p = x * y, pe = fmaf(x, y, -p);
    const float q = z * w, qe = fmaf(z, w, -q);
    float s, se;
    detail::two_sum(p, q, s, se);
    const float low = ((pe + qe) + se) + ((x * yl + xl * y) + (z * wl + zl * w));
    return s + low;
  } else {
    return ((a - b) * (c - d)) + ((e - f) * (g - h));
  }
}

}  // namespace oeb
