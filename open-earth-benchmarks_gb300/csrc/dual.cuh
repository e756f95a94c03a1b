// dual.cuh -- forward-mode dual numbers for the tangent-linear stencils.
//
// A Dual<T> carries a value and one directional derivative.  Instantiating a stencil kernel
// with Dual<T> in place of T computes, in one pass, the forward result (the value part,
// bit-identical to the T kernel: the same operations on the same values) and its
// tangent-linear image J * dx (the derivative part).  Every branch -- upwind switches, flux
// limiters, PPM flags, the Smagorinsky clamp -- compares value parts only, so the branches
// are frozen at the forward state, as the linearisation requires.
#pragma once

#include <cuda_runtime.h>

#include "precision.cuh"

namespace oeb {

template <class T>
struct Dual {
  T v, d;
  __host__ __device__ constexpr Dual() : v(0), d(0) {}
  __host__ __device__ constexpr Dual(T value) : v(value), d(0) {}  // NOLINT: constants are constant
  __host__ __device__ constexpr Dual(T value, T deriv) : v(value), d(deriv) {}
};

template <class T>
__host__ __device__ constexpr Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <class T>
__host__ __device__ constexpr Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <class T>
__host__ __device__ constexpr Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }
template <class T>
__host__ __device__ constexpr Dual<T> operator*(Dual<T> a, Dual<T> b) {
  return Dual<T>(a.v * b.v, a.v * b.d + a.d * b.v);
}
template <class T>
__host__ __device__ constexpr Dual<T> operator/(Dual<T> a, Dual<T> b) {
  return Dual<T>(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v));
}
// mixed operands: a plain number is a constant
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator*(S a, Dual<T> b) { return Dual<T>(T(a)) * b; }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator*(Dual<T> a, S b) { return a * Dual<T>(T(b)); }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator+(S a, Dual<T> b) { return Dual<T>(T(a)) + b; }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator+(Dual<T> a, S b) { return a + Dual<T>(T(b)); }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator-(S a, Dual<T> b) { return Dual<T>(T(a)) - b; }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator-(Dual<T> a, S b) { return a - Dual<T>(T(b)); }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator/(S a, Dual<T> b) { return Dual<T>(T(a)) / b; }
template <class T, class S>
__host__ __device__ constexpr Dual<T> operator/(Dual<T> a, S b) { return a / Dual<T>(T(b)); }

// comparisons look at values only (branches frozen at the forward state)
#define OEB_DUAL_CMP(OP)                                                                             \
  template <class T>                                                                                 \
  __host__ __device__ constexpr bool operator OP(Dual<T> a, Dual<T> b) { return a.v OP b.v; }        \
  template <class T, class S>                                                                        \
  __host__ __device__ constexpr bool operator OP(Dual<T> a, S b) { return a.v OP T(b); }             \
  template <class T, class S>                                                                        \
  __host__ __device__ constexpr bool operator OP(S a, Dual<T> b) { return T(a) OP b.v; }
OEB_DUAL_CMP(<)
OEB_DUAL_CMP(>)
OEB_DUAL_CMP(<=)
OEB_DUAL_CMP(>=)
#undef OEB_DUAL_CMP

template <class T>
__device__ __forceinline__ Dual<T> ld(const Dual<T>* p) {
  const T* q = reinterpret_cast<const T*>(p);
#ifdef OEB_COHERENT_LOADS  // the step kernel: see ld() in stencil_util.cuh
  return Dual<T>(__ldca(q), __ldca(q + 1));
#else
  return Dual<T>(__ldg(q), __ldg(q + 1));
#endif
}

template <class T>
struct Prec<Dual<T>> {
  static constexpr bool kCompensated = false;
  // the branch decided exactly as the T kernel decides it, on the values
  __device__ static __forceinline__ bool prod_gt0(Dual<T> a, Dual<T> b) { return Prec<T>::prod_gt0(a.v, b.v); }
  __device__ static __forceinline__ bool prod_lt0(Dual<T> a, Dual<T> b) { return Prec<T>::prod_lt0(a.v, b.v); }
  __device__ static __forceinline__ Dual<T> sqrt_(Dual<T> x) {
    const T s = Prec<T>::sqrt_(x.v);
    return Dual<T>(s, x.d / (T(2) * s));
  }
  __device__ static __forceinline__ bool gt0(Dual<T> x) { return Prec<T>::gt0(x.v); }
  __device__ static __forceinline__ bool lt_nonneg(Dual<T> a, Dual<T> b) { return Prec<T>::lt_nonneg(a.v, b.v); }
  template <int K>
  __device__ static __forceinline__ Dual<T> scale2(Dual<T> x) {
    return Dual<T>(Prec<T>::template scale2<K>(x.v), Prec<T>::template scale2<K>(x.d));
  }
  __device__ static __forceinline__ Dual<T> scale2v(Dual<T> x, int k) {
    return Dual<T>(Prec<T>::scale2v(x.v, k), Prec<T>::scale2v(x.d, k));
  }
  __device__ static __forceinline__ Dual<T> add_flag(Dual<T> q, Dual<T> t, bool flag) {
    return q + t * (flag ? T(1) : T(0));
  }
};

template <class T>
struct ValueOf {
  using type = T;
};
template <class T>
struct ValueOf<Dual<T>> {
  using type = T;
};

}  // namespace oeb
