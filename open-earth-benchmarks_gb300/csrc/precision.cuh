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

// FP64 operations done exactly on the integer pipe.  The GB300 issues 1.6 FP64 operations
// per clock per SM and about 100 integer ones, and the FP64 stencils are bound by the FP64
// pipe; so sign tests, comparisons of non-negative values, multiplications by powers of two
// and the multiply by a 0/1 flag of fvtp2d are done on the bit patterns.  Each gives the
// result of the FP64 operation it replaces, bit for bit, and falls back to that operation
// for every input where the shortcut could differ (zeros, subnormals, infinities, NaN, a
// product that could underflow, a scaling that could leave the normal range).
namespace fp64 {
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ int exponent(long long b) { return (int)((b >> 52) & 0x7FF); }
// both operands normal and |a b| >= 2^(ea + eb - 2046) >= 2^-1074: the rounded product is
// nonzero and carries the sign of the exact one
__device__ __forceinline__ bool product_sign_known(long long ua, long long ub) {
  const int ea = exponent(ua), eb = exponent(ub);
  return ea > 0 && eb > 0 && ea < 2047 && eb < 2047 && ea + eb >= 972;
}
}  // namespace fp64

template <>
struct Prec<double> {
  static constexpr bool kCompensated = false;
  // reference semantics: the rounded FP64 product compared with 0 (hdiffsa.h:106, fvtp2d.h:23)
  __device__ static __forceinline__ bool prod_gt0(double a, double b) {
    const long long ua = fp64::bits(a), ub = fp64::bits(b);
    return fp64::product_sign_known(ua, ub) ? (ua ^ ub) >= 0 : a * b > 0;
  }
  __device__ static __forceinline__ bool prod_lt0(double a, double b) {
    const long long ua = fp64::bits(a), ub = fp64::bits(b);
    return fp64::product_sign_known(ua, ub) ? (ua ^ ub) < 0 : (a * b) < 0.0;
  }
  __device__ static __forceinline__ double sqrt_(double x) { return sqrt(x); }
  // x > 0 (false for NaN and -0)
  __device__ static __forceinline__ bool gt0(double x) {
    const long long b = fp64::bits(x);
    return b > 0 && b <= 0x7FF0000000000000LL;
  }
  // a < b for a, b >= +0 and not NaN: the bit patterns order as the values
  __device__ static __forceinline__ bool lt_nonneg(double a, double b) { return fp64::bits(a) < fp64::bits(b); }
  // x * 2^K
  template <int K>
  __device__ static __forceinline__ double scale2(double x) {
    const long long b = fp64::bits(x);
    const int e = fp64::exponent(b);
    if (e > 0 && e < 2047 && e + K > 0 && e + K < 2047) return __longlong_as_double(b + ((long long)K << 52));
    return x * (K >= 0 ? double(1LL << (K >= 0 ? K : 0)) : 1.0 / double(1LL << (K < 0 ? -K : 0)));
  }
  // q + t * (flag ? 1.0 : 0.0): t * 1 is t; t * 0 is a zero with t's sign (t finite), and
  // q + (+-0) is q except -0 + +0 = +0
  __device__ static __forceinline__ double add_flag(double q, double t, bool flag) {
    if (flag) return q + t;
    const long long bt = fp64::bits(t);
    if (fp64::exponent(bt) == 0x7FF) return q + t * 0.0;  // t infinite or NaN
    return (fp64::bits(q) == (long long)0x8000000000000000ULL && bt >= 0) ? 0.0 : q;
  }
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
  __device__ static __forceinline__ bool gt0(float x) { return x > 0.f; }
  __device__ static __forceinline__ bool lt_nonneg(float a, float b) { return a < b; }
  template <int K>
  __device__ static __forceinline__ float scale2(float x) {
    return x * (K >= 0 ? float(1LL << (K >= 0 ? K : 0)) : 1.0f / float(1LL << (K < 0 ? -K : 0)));
  }
  __device__ static __forceinline__ float add_flag(float q, float t, bool flag) { return q + t * (flag ? 1.f : 0.f); }
};

// the same operations by element type
template <class T>
__device__ __forceinline__ bool gt0(T x) {
  return Prec<T>::gt0(x);
}
template <int K, class T>
__device__ __forceinline__ T scale2(T x) {
  return Prec<T>::template scale2<K>(x);
}

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
