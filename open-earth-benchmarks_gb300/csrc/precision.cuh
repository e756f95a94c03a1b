// precision.cuh -- what changes between the FP64 and the FP32 stencils.
//
// FP64 (Prec<double>): the reference's own arithmetic, operation for operation, so that with
// FP contraction off the results are bit-identical to the reference's OpenMP kernels.
//
// FP32 (Prec<float>): fields stored and computed in FP32.  Where the reference's float
// sequence is as accurate as anything cheaper-than-FP64 (measured against the FP64 oracle),
// the kernels run exactly that sequence and are bit-identical to the reference compiled for
// float: the advection drivers (hadvuv.h:10-24, hadvuv5th.h:10-36) and hdiffsmag.  Elsewhere:
//  * branch tests on the sign of a product -- the hdiffsa flux limiter (hdiffsa.h:106-113)
//    and the fvtp2d PPM monotonicity flag (fvtp2d.h:23) -- are decided on the exact
//    product, which is what an FP64 product of two floats gives (it is exact in FP64 and
//    cannot underflow); here without any FP64 instruction, from the operands' signs;
//  * the laplacian (laplace.h:39), whose centre term nearly cancels the neighbour sum, is
//    formed as a sum of neighbour differences (k_pointwise.cu);
//  * the paired products of the pressure gradients (nh_p_grad.h:126-142,
//    p_grad_c.h:90-97) are summed with Kahan's FMA algorithm over error-free
//    differences (diff_dot below);
//  * uvbke's double dt5 multiplies as a float pair (k_pointwise.cu).
// kCompensated selects these forms.
#pragma once

#include <cuda_runtime.h>

namespace oeb {

template <class T>
struct Prec;

// FP64 operations done exactly on the integer pipe.  The GB300 issues 1.6 FP64 operations
// per clock per SM and about 100 integer ones, and the FP64 stencils are bound by the FP64
// pipe; so multiplications, sign tests, comparisons of non-negative values, multiplications
// by powers of two and the multiply by a 0/1 flag of fvtp2d are done on the bit patterns.
// Each gives the result of the FP64 operation it replaces, bit for bit, and falls back to
// that operation for every input where the shortcut could differ (zeros, subnormals,
// infinities, NaN, a result that could underflow or overflow).
//
// The fallbacks are calls, not inline operations: an inline FP64 operation on a branch is
// if-converted into a predicated instruction that takes its slot in the FP64 pipe on every
// pass, taken or not, and the integer path would then save nothing.
namespace fp64 {
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ int exponent(long long b) { return (int)((b >> 52) & 0x7FF); }
// both operands normal and |a b| >= 2^(ea + eb - 2046) >= 2^-1074: the rounded product is
// nonzero and carries the sign of the exact one
__device__ __forceinline__ bool product_sign_known(long long ua, long long ub) {
  const int ea = exponent(ua), eb = exponent(ub);
  return ea > 0 && eb > 0 && ea < 2047 && eb < 2047 && ea + eb >= 972;
}

// The fallbacks of the integer-pipe operations below take and return bit patterns: their
// result then merges with the fast path's as an integer, where a merge of two doubles has
// been seen to cost an FP64 instruction on every pass.
static __device__ __noinline__ unsigned long long mul_bits(unsigned long long a, unsigned long long b) {
  return (unsigned long long)bits(__dmul_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b)));
}
static __device__ __noinline__ unsigned long long div_bits(unsigned long long a, unsigned long long b) {
  return (unsigned long long)bits(__ddiv_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b)));
}
static __device__ __noinline__ unsigned long long add_bits(unsigned long long a, unsigned long long b) {
  return (unsigned long long)bits(__dadd_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b)));
}
static __device__ __noinline__ unsigned long long sqrt_bits(unsigned long long x) {
  return (unsigned long long)bits(__dsqrt_rn(__longlong_as_double((long long)x)));
}
// q + t * 0.0, both roundings (t infinite or NaN: a NaN)
static __device__ __noinline__ unsigned long long add_mul0_bits(unsigned long long q, unsigned long long t) {
  return (unsigned long long)bits(
      __dadd_rn(__longlong_as_double((long long)q), __dmul_rn(__longlong_as_double((long long)t), 0.0)));
}

// a * b rounded to nearest even, on the integer pipe.  For normal a, b whose product is
// normal: the exact product of the two 53-bit significands (1.f, hidden bit set) has 105 or
// 106 bits; its top 53 bits are the significand of the result, the next bit is the round
// bit and the OR of the rest the sticky bit, and IEEE 754 round-to-nearest-even adds one
// ulp when round and (sticky or the last kept bit) are set.  A carry out of the significand
// moves into the exponent field by itself, which is the correct rounding up to the next
// power of two.  The 106-bit product comes from four independent 32 x 32 -> 64-bit multiplies
// of the significands split into a high part of 21 bits and a low part of 32.  Any other input --
// a zero, subnormal, infinite or NaN operand, or an exponent sum outside [1, 2045] where the
// result could be subnormal or overflow -- takes the FP64 multiply.
__device__ __forceinline__ double mul(double a, double b) {
  const unsigned long long ua = (unsigned long long)bits(a), ub = (unsigned long long)bits(b);
  const unsigned ha = (unsigned)(ua >> 32), hb = (unsigned)(ub >> 32);
  const unsigned la = (unsigned)ua, lb = (unsigned)ub;
  const unsigned ea = (ha >> 20) & 0x7FFu, eb = (hb >> 20) & 0x7FFu;
  const unsigned a1 = (ha & 0xFFFFFu) | 0x100000u, b1 = (hb & 0xFFFFFu) | 0x100000u;
  // (a1 2^32 + la)(b1 2^32 + lb) = w3:w2:w1:w0 (32-bit words), in [2^104, 2^106); the four
  // partial products are independent (a short dependency chain), the middle ones summed
  // with the carry of the lowest (below 2^55: no overflow)
  const unsigned long long p00 = (unsigned long long)la * lb;
  const unsigned long long p01 = (unsigned long long)la * b1;
  const unsigned long long p10 = (unsigned long long)a1 * lb;
  const unsigned long long p11 = (unsigned long long)a1 * b1;
  const unsigned long long mid = p01 + p10 + (p00 >> 32);
  const unsigned long long top64 = p11 + (mid >> 32);
  const unsigned w0 = (unsigned)p00, w1 = (unsigned)mid, w2 = (unsigned)top64, w3 = (unsigned)(top64 >> 32);
  const unsigned top = w3 >> 9;  // 1 if the product has 106 bits
  const unsigned sh = 20u + top;  // significand = (w3:w2:w1) >> sh, hidden bit at bit 52
  const unsigned mlo = __funnelshift_r(w1, w2, sh);
  const unsigned mhi = __funnelshift_r(w2, w3, sh);
  // the bits below the significand, left-aligned: bit 31 is the round bit; w0 joins the
  // sticky bits at bit 0 (the shift leaves at least 11 zero bits there)
  const unsigned rest = (w1 << (12u - top)) | (w0 != 0u ? 1u : 0u);
  const unsigned up = (rest + (mlo & 1u)) > 0x80000000u ? 1u : 0u;
  const int e = (int)(ea + eb) - 1023 + (int)top;  // biased exponent before rounding
  unsigned long long r = ((((unsigned long long)mhi) << 32) | mlo) + up;
  r += (unsigned long long)(unsigned)(e - 1) << 52;  // the hidden bit adds the last 1
  r |= ((unsigned long long)((ha ^ hb) & 0x80000000u)) << 32;
  const bool fast = (ea - 1u < 2046u) & (eb - 1u < 2046u) & ((unsigned)(e - 1) < 2045u);
  if (__builtin_expect(!fast, 0)) r = mul_bits(ua, ub);
  return __longlong_as_double((long long)r);
}

// FP32 reciprocal estimate (PTX rcp.approx: relative error within a few 2^-23)
__device__ __forceinline__ float rcp_estimate(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// a / b rounded to nearest even, on the integer pipe, by digit recurrence.  For normal a,
// b whose quotient is normal: with the significands ma, mb in [2^52, 2^53) and X = ma (or
// 2 ma when ma < mb, the exponent one lower) so that X / mb is in [1, 2), the result's
// significand and round bit are Q = floor(X 2^53 / mb), in [2^53, 2^54), and its sticky bit
// is (X 2^53 - Q mb != 0).  Q is found as three digits of 20, 20 and 13 bits: each digit q
// estimates P 2^s / mb for the current remainder P with a 30-bit fixed-point reciprocal R
// of mb (from the FP32 reciprocal of mb's top 24 bits), rounded to nearest, and the next
// remainder P 2^s - q mb is computed exactly in 64-bit two's complement (it is below 2 mb in
// magnitude, so the arithmetic modulo 2^64 is exact).  A digit may be off by one; the
// remainders stay signed and the last one, within (-mb, 2 mb), is brought into [0, mb) by
// one correction of Q.  Round-to-nearest-even then adds one ulp when the round bit is set
// and the remainder or the last kept bit is nonzero.  Inputs outside that case -- zeros,
// subnormals, infinities, NaN, a quotient that could be subnormal or overflow -- and any
// remainder still outside [0, mb) take the FP64 division.
__device__ __forceinline__ double div(double a, double b) {
  typedef unsigned long long u64;
  typedef long long i64;
  const u64 ua = (u64)bits(a), ub = (u64)bits(b);
  const unsigned ha = (unsigned)(ua >> 32), hb = (unsigned)(ub >> 32);
  const unsigned ea = (ha >> 20) & 0x7FFu, eb = (hb >> 20) & 0x7FFu;
  const u64 ma = (ua & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const u64 mb = (ub & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const bool lt = ma < mb;
  const u64 X = lt ? ma << 1 : ma;
  const int e = (int)ea - (int)eb + 1023 - (lt ? 1 : 0);  // biased exponent before rounding
  // R ~ 2^82 / mb, in (2^29, 2^30]: 2^29 / (mb >> 29) scaled by 2^53
  const int R = (int)(rcp_estimate((float)(int)(mb >> 29)) * 9007199254740992.0f);
  // digit q ~ P 2^s / mb = (P >> 24) R 2^(s - 58), rounded to nearest
  const int qa = (int)(((i64)(int)(X >> 24) * R + (1ll << 37)) >> 38);
  const u64 P1 = (X << 20) - (u64)((i64)qa * (i64)mb);
  const int qb = (int)(((i64)(int)((i64)P1 >> 24) * R + (1ll << 37)) >> 38);
  const u64 P2 = (P1 << 20) - (u64)((i64)qb * (i64)mb);
  const int qc = (int)(((i64)(int)((i64)P2 >> 24) * R + (1ll << 44)) >> 45);
  i64 P = (i64)((P2 << 13) - (u64)((i64)qc * (i64)mb));
  i64 Q = ((i64)qa << 33) + ((i64)qb << 13) + qc;
  if (P < 0) {
    Q -= 1;
    P += (i64)mb;
  } else if (P >= (i64)mb) {
    Q += 1;
    P -= (i64)mb;
  }
  const u64 sig = (u64)Q >> 1;  // hidden bit at bit 52
  const unsigned up = (unsigned)(Q & 1) & ((P != 0 ? 1u : 0u) | (unsigned)(sig & 1));
  u64 r = sig + up + ((u64)(unsigned)(e - 1) << 52);
  r |= ((u64)((ha ^ hb) & 0x80000000u)) << 32;
  const bool fast = (ea - 1u < 2046u) & (eb - 1u < 2046u) & ((unsigned)(e - 1) < 2045u) & (P >= 0) & (P < (i64)mb);
  if (__builtin_expect(!fast, 0)) r = div_bits(ua, ub);
  return __longlong_as_double((long long)r);
}

// a + b rounded to nearest even, on the integer pipe.  With |x| >= |y| the operands ordered
// by magnitude (their bit patterns without the sign order as the magnitudes), the 53-bit
// significands are placed at bits 62..10 of 64-bit words, so ten guard bits sit below
// them; y's is shifted right by the exponent difference with every bit shifted out ORed
// into bit 0 (the sticky bit).  The significands are added or, for opposite signs,
// subtracted (the difference is >= 0), the sum is normalised so that its leading bit is
// bit 63 (at most one place right for a sum, any number left for a difference -- a left
// shift of more than two places happens only when no bit was shifted out), and
// round-to-nearest-even on bits 10..0 gives the result, the exponent following the
// normalisation.  Exact cancellation gives +0 and y = +-0 gives x, as IEEE addition does.
// Zeros for x, subnormals, infinities, NaN and a result that could be subnormal or
// overflow take the FP64 addition.
__device__ __forceinline__ double add(double a, double b) {
  typedef unsigned long long u64;
  const u64 M = 0x7FFFFFFFFFFFFFFFull;
  const u64 ua = (u64)bits(a), ub = (u64)bits(b);
  const u64 aa = ua & M, ab = ub & M;
  const bool sw = ab > aa;
  const u64 x = sw ? ub : ua, y = sw ? ua : ub;
  const u64 ax = sw ? ab : aa, ay = sw ? aa : ab;
  const unsigned ex = (unsigned)(ax >> 52), ey = (unsigned)(ay >> 52);
  const u64 mx = ((ax & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) << 10;
  const u64 my = ((ay & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) << 10;
  const unsigned d = ex - ey;
  const unsigned dc = d < 63u ? d : 63u;
  const u64 ya = (my >> dc) | ((my & ((1ull << dc) - 1ull)) != 0ull ? 1ull : 0ull);
  const bool sub = (long long)(x ^ y) < 0;
  const u64 S = sub ? mx - ya : mx + ya;
  const int lz = __clzll((long long)S);
  const u64 N = S << (lz & 63);
  const u64 sig = N >> 11;
  const unsigned rest = (unsigned)N & 0x7FFu;
  const unsigned up = (rest + (unsigned)(sig & 1ull)) > 0x400u ? 1u : 0u;
  const int e = (int)ex + 1 - lz;  // biased exponent before rounding
  u64 r = (((u64)(unsigned)(e - 1)) << 52) + sig + up;
  r |= x & 0x8000000000000000ull;
  const bool xok = ex - 1u < 2046u;
  bool fast = xok & (ey - 1u < 2046u) & ((unsigned)(e - 1) < 2045u);
  if (S == 0ull) {
    r = 0ull;
    fast = xok;
  }
  if (ay == 0ull) {
    r = x;
    fast = xok;
  }
  if (__builtin_expect(!fast, 0)) r = add_bits(ua, ub);
  return __longlong_as_double((long long)r);
}

// FP32 reciprocal square root estimate (PTX rsqrt.approx: relative error within a few 2^-23)
__device__ __forceinline__ float rsqrt_estimate(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// sqrt(x) rounded to nearest even, on the integer pipe.  For positive normal x with
// significand m in [2^52, 2^53) and M = m (or 2 m, making the exponent even), the result's
// significand and round bit are S = floor(sqrt(M 2^54)), in [2^53, 2^54), and its sticky
// bit is (M 2^54 - S^2 != 0).  S is found in two halves of 27 bits, S = s1 2^27 + s0:
//  * s1 = floor(sqrt(M)): an estimate from the FP32 reciprocal square root y of M's top 24
//    bits, one Newton step s1 + (M - s1^2) / (2 s1) with the exact integer residual, and
//    one correction that brings r = M - s1^2 into [0, 2 s1];
//  * s0 ~ r 2^54 / (2 s1 2^27) from y, one Newton step on the residual
//    R = r 2^54 - s0 (2 s1 2^27 + s0), computed exactly in 64-bit two's complement (it stays
//    within a few multiples of 2 S), and one correction that brings R into [0, 2 S].
// Round-to-nearest-even then adds one ulp when the round bit is set and R or the last kept
// bit is nonzero (an exact tie cannot occur).  Zero, negative, subnormal, infinite and NaN
// inputs, and any residual still outside [0, 2 S], take the FP64 square root.
__device__ __forceinline__ double sqrt(double x) {
  typedef unsigned long long u64;
  typedef long long i64;
  const u64 ux = (u64)bits(x);
  const unsigned ex = (unsigned)(ux >> 52);  // with the sign: a negative x gives ex >= 2048
  const u64 m = (ux & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const unsigned odd = (ex & 1u) ^ 1u;  // the unbiased exponent of m is odd
  const u64 M = m << odd;               // [2^52, 2^54)
  const float mf = (float)(unsigned)(M >> 30);  // [2^22, 2^24), exact
  const float y = rsqrt_estimate(mf);
  unsigned s1 = (unsigned)(mf * y * 32768.0f + 0.5f);
  i64 r = (i64)(M - (u64)s1 * s1);
  s1 = (unsigned)((int)s1 + (int)rintf((float)r * (y * (1.0f / 65536.0f))));
  r = (i64)(M - (u64)s1 * s1);
  if (r < 0) {
    s1 -= 1;
    r += 2 * (i64)s1 + 1;
  } else if (r > 2 * (i64)s1) {
    r -= 2 * (i64)s1 + 1;
    s1 += 1;
  }
  int s0 = (int)rintf((float)r * (y * 2048.0f));
  const u64 t = (u64)s1 << 28;
  u64 rem = ((u64)r << 54) - (u64)(i64)s0 * (t + (u64)(i64)s0);
  s0 += (int)rintf((float)(int)((i64)rem >> 32) * (y * (1.0f / 2048.0f)));
  rem = ((u64)r << 54) - (u64)(i64)s0 * (t + (u64)(i64)s0);
  u64 S = ((u64)s1 << 27) + (u64)(i64)s0;
  i64 R = (i64)rem;
  if (R < 0) {
    R += 2 * (i64)S - 1;
    S -= 1;
  } else if (R > 2 * (i64)S) {
    R -= 2 * (i64)S + 1;
    S += 1;
  }
  const u64 sig = S >> 1;  // hidden bit at bit 52
  const unsigned up = (unsigned)(S & 1ull) & ((R != 0 ? 1u : 0u) | (unsigned)(sig & 1ull));
  const unsigned be = ((ex - odd - 1u) >> 1) + 512u;  // biased exponent of the root
  u64 res = (((u64)(be - 1u)) << 52) + sig + up;
  const bool fast = (ex - 1u < 2046u) & (R >= 0) & (R <= 2 * (i64)S);
  if (__builtin_expect(!fast, 0)) res = sqrt_bits(ux);
  return __longlong_as_double((long long)res);
}

// -x: the sign bit flipped (IEEE negation)
__device__ __forceinline__ double neg(double x) {
  return __longlong_as_double(bits(x) ^ (long long)0x8000000000000000ull);
}

// Ordered comparisons on the bit patterns: a pattern mapped to its magnitude, negated for a
// negative sign, orders as the values do (+0 and -0 both map to 0); any comparison with a
// NaN is false.
__device__ __forceinline__ long long order_key(long long b) {
  const long long m = b & 0x7FFFFFFFFFFFFFFFll;
  return b < 0 ? -m : m;
}
__device__ __forceinline__ bool unordered(long long a, long long b) {
  return ((a & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll) | ((b & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll);
}
__device__ __forceinline__ bool lt(double a, double b) {
  const long long ia = bits(a), ib = bits(b);
  return !unordered(ia, ib) && order_key(ia) < order_key(ib);
}
__device__ __forceinline__ bool le(double a, double b) {
  const long long ia = bits(a), ib = bits(b);
  return !unordered(ia, ib) && order_key(ia) <= order_key(ib);
}
__device__ __forceinline__ bool eq(double a, double b) {
  const long long ia = bits(a), ib = bits(b);
  return !unordered(ia, ib) && order_key(ia) == order_key(ib);
}
}  // namespace fp64

template <>
struct Prec<double> {
  static constexpr bool kCompensated = false;
  // reference semantics: the rounded FP64 product compared with 0 (hdiffsa.h:106, fvtp2d.h:23)
  __device__ static __forceinline__ bool prod_gt0(double a, double b) {
    const long long ua = fp64::bits(a), ub = fp64::bits(b);
    if (fp64::product_sign_known(ua, ub)) return (ua ^ ub) >= 0;
    const long long p = (long long)fp64::mul_bits((unsigned long long)ua, (unsigned long long)ub);
    return p > 0 && p <= 0x7FF0000000000000LL;  // positive, not NaN
  }
  __device__ static __forceinline__ bool prod_lt0(double a, double b) {
    const long long ua = fp64::bits(a), ub = fp64::bits(b);
    if (fp64::product_sign_known(ua, ub)) return (ua ^ ub) < 0;
    const long long p = (long long)fp64::mul_bits((unsigned long long)ua, (unsigned long long)ub);
    const long long m = p & 0x7FFFFFFFFFFFFFFFLL;
    return p < 0 && m != 0 && m <= 0x7FF0000000000000LL;  // negative, not -0, not NaN
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
    long long r = b + ((long long)K << 52);
    if (!(e > 0 && e < 2047 && e + K > 0 && e + K < 2047)) {
      const double f = K >= 0 ? double(1LL << (K >= 0 ? K : 0)) : 1.0 / double(1LL << (K < 0 ? -K : 0));
      r = (long long)fp64::mul_bits((unsigned long long)b, (unsigned long long)fp64::bits(f));
    }
    return __longlong_as_double(r);
  }
  // x * 2^k for a k chosen at run time (|k| small)
  __device__ static __forceinline__ double scale2v(double x, int k) {
    const long long b = fp64::bits(x);
    const int e = fp64::exponent(b);
    long long r = b + ((long long)k << 52);
    if (!(e > 0 && e < 2047 && e + k > 0 && e + k < 2047))
      r = (long long)fp64::mul_bits((unsigned long long)b, (unsigned long long)(1023 + k) << 52);
    return __longlong_as_double(r);
  }
  // q + t * (flag ? 1.0 : 0.0): t * 1 is t; t * 0 is a zero with t's sign (t finite), and
  // q + (+-0) is q except -0 + +0 = +0
  __device__ static __forceinline__ double add_flag(double q, double t, bool flag) {
    const long long bq = fp64::bits(q), bt = fp64::bits(t);
    long long r;
    if (flag) {
      r = fp64::bits(q + t);
    } else if (fp64::exponent(bt) == 0x7FF) {  // t infinite or NaN
      r = (long long)fp64::add_mul0_bits((unsigned long long)bq, (unsigned long long)bt);
    } else {
      r = (bq == (long long)0x8000000000000000ULL && bt >= 0) ? 0 : bq;
    }
    return __longlong_as_double(r);
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
  __device__ static __forceinline__ float scale2v(float x, int k) { return x * __int_as_float((127 + k) << 23); }
  __device__ static __forceinline__ float add_flag(float q, float t, bool flag) { return q + t * (flag ? 1.f : 0.f); }
};

// FP64 in the stencil kernels: a double whose multiplications, divisions, square roots
// (Prec<F64i>::sqrt_), negations and comparisons run on the integer pipe (fp64::mul, div,
// sqrt, neg, lt/le/eq) and whose additions and subtractions are the FP64 instruction, or
// fp64::add where a kernel asks for it with iadd/isub.  Every operation rounds exactly as
// the double operation does, so a kernel gives the same bits with F64i as with double; the
// FP64 pipe, which bounds these kernels, then carries only the additions, while the
// integer pipe does the rest beside it.  Same size and alignment as double:
// double fields are read and written as F64i in place.  launch() (launch.cuh) runs every
// kernel instantiated for double with F64i.
struct F64i {
  double v;
  F64i() = default;
  __host__ __device__ constexpr F64i(double x) : v(x) {}
};
static_assert(sizeof(F64i) == sizeof(double) && alignof(F64i) == alignof(double), "F64i must alias double");

__host__ __device__ constexpr F64i operator+(F64i a, F64i b) { return F64i(a.v + b.v); }
__host__ __device__ constexpr F64i operator-(F64i a, F64i b) { return F64i(a.v - b.v); }
// constant expressions (the kernels' folded coefficients) divide at compile time
__host__ __device__ constexpr F64i operator/(F64i a, F64i b) {
#if defined(__CUDA_ARCH__)
  if (!__builtin_is_constant_evaluated()) return F64i(fp64::div(a.v, b.v));
#endif
  return F64i(a.v / b.v);
}
__host__ __device__ constexpr F64i operator-(F64i a) {
#if defined(__CUDA_ARCH__)
  if (!__builtin_is_constant_evaluated()) return F64i(fp64::neg(a.v));
#endif
  return F64i(-a.v);
}
__device__ __forceinline__ F64i operator*(F64i a, F64i b) { return F64i(fp64::mul(a.v, b.v)); }
__device__ __forceinline__ F64i& operator+=(F64i& a, F64i b) { return a = a + b; }
__device__ __forceinline__ F64i& operator-=(F64i& a, F64i b) { return a = a - b; }
__device__ __forceinline__ F64i& operator*=(F64i& a, F64i b) { return a = a * b; }
__device__ __forceinline__ F64i& operator/=(F64i& a, F64i b) { return a = a / b; }
__device__ __forceinline__ bool operator<(F64i a, F64i b) { return fp64::lt(a.v, b.v); }
__device__ __forceinline__ bool operator>(F64i a, F64i b) { return fp64::lt(b.v, a.v); }
__device__ __forceinline__ bool operator<=(F64i a, F64i b) { return fp64::le(a.v, b.v); }
__device__ __forceinline__ bool operator>=(F64i a, F64i b) { return fp64::le(b.v, a.v); }
__device__ __forceinline__ bool operator==(F64i a, F64i b) { return fp64::eq(a.v, b.v); }
__device__ __forceinline__ bool operator!=(F64i a, F64i b) { return !fp64::eq(a.v, b.v); }
// fused multiply-add of the adjoint accumulations: the FP64 instruction (one rounding); the
// float and double overloads stay visible beside it
using ::fma;
__device__ __forceinline__ F64i fma(F64i a, F64i b, F64i c) { return F64i(::fma(a.v, b.v, c.v)); }
#ifdef OEB_COHERENT_LOADS  // the step kernel: see ld() in stencil_util.cuh
__device__ __forceinline__ F64i ld(const F64i* p) { return F64i(__ldca(reinterpret_cast<const double*>(p))); }
#else
__device__ __forceinline__ F64i ld(const F64i* p) { return F64i(__ldg(reinterpret_cast<const double*>(p))); }
#endif

template <>
struct Prec<F64i> {
  static constexpr bool kCompensated = false;
  __device__ static __forceinline__ bool prod_gt0(F64i a, F64i b) { return Prec<double>::prod_gt0(a.v, b.v); }
  __device__ static __forceinline__ bool prod_lt0(F64i a, F64i b) { return Prec<double>::prod_lt0(a.v, b.v); }
  __device__ static __forceinline__ F64i sqrt_(F64i x) { return F64i(fp64::sqrt(x.v)); }
  __device__ static __forceinline__ bool gt0(F64i x) { return Prec<double>::gt0(x.v); }
  __device__ static __forceinline__ bool lt_nonneg(F64i a, F64i b) { return Prec<double>::lt_nonneg(a.v, b.v); }
  template <int K>
  __device__ static __forceinline__ F64i scale2(F64i x) {
    return F64i(Prec<double>::template scale2<K>(x.v));
  }
  __device__ static __forceinline__ F64i scale2v(F64i x, int k) { return F64i(Prec<double>::scale2v(x.v, k)); }
  __device__ static __forceinline__ F64i add_flag(F64i q, F64i t, bool flag) {
    return F64i(Prec<double>::add_flag(q.v, t.v, flag));
  }
};

// An addition or subtraction that the FP64 kernels do on the integer pipe (fp64::add) to
// balance it against the FP64 pipe; every other element type adds as usual.  The results
// are those of + and -.
template <class T>
__device__ __forceinline__ T iadd(T a, T b) {
  return a + b;
}
template <class T>
__device__ __forceinline__ T isub(T a, T b) {
  return a - b;
}
template <>
__device__ __forceinline__ F64i iadd<F64i>(F64i a, F64i b) {
  return F64i(fp64::add(a.v, b.v));
}
template <>
__device__ __forceinline__ F64i isub<F64i>(F64i a, F64i b) {
  return F64i(fp64::add(a.v, fp64::neg(b.v)));
}

// the same operations by element type
template <class T>
__device__ __forceinline__ bool gt0(T x) {
  return Prec<T>::gt0(x);
}
template <int K, class T>
__device__ __forceinline__ T scale2(T x) {
  return Prec<T>::template scale2<K>(x);
}
// x * 2^k, k chosen at run time (|k| small)
template <class T>
__device__ __forceinline__ T scale2v(T x, int k) {
  return Prec<T>::scale2v(x, k);
}

// Left-to-right sum of terms, in the reference's order and rounding (every precision).
template <class T>
struct Acc {
  T s;
  __device__ __forceinline__ explicit Acc(T x) : s(x) {}
  __device__ __forceinline__ static Acc prod(T a, T b) { return Acc(a * b); }
  __device__ __forceinline__ void add(T x) { s = s + x; }
  __device__ __forceinline__ void add_prod(T a, T b) { s = s + a * b; }
  __device__ __forceinline__ T get() const { return s; }
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
// FP64: exactly these operations in this order, the reference's expression tree.  FP32: the
// four differences as TwoSum pairs x + xl (exact), and the sum of the products evaluated with
// Kahan's FMA algorithm -- q = z w rounded, its rounding error qe = fma(z, w, -q) exactly, then
// fma(x, y, q) -- with qe and the first-order terms of the differences' errors (x yl + xl y +
// z wl + zl w) added at the end.  The result is within a few ulp of the exact expression of
// the FP32 operands, without a branch, in 32 operations (a float-float evaluation of the same
// takes 43).
template <class T>
__device__ __forceinline__ T diff_dot(T a, T b, T c, T d, T e, T f, T g, T h) {
  if constexpr (Prec<T>::kCompensated) {
    float x, xl, y, yl, z, zl, w, wl;
    detail::two_sum(a, -b, x, xl);
    detail::two_sum(c, -d, y, yl);
    detail::two_sum(e, -f, z, zl);
    detail::two_sum(g, -h, w, wl);
    const float q = z * w;
    const float qe = fmaf(z, w, -q);
    const float m = fmaf(x, y, q);
    const float low = fmaf(x, yl, fmaf(xl, y, fmaf(z, wl, fmaf(zl, w, qe))));
    return m + low;
  } else {
    return ((a - b) * (c - d)) + ((e - f) * (g - h));
  }
}

// The same paired products for fields stored as an FP64 per-level base profile plus FP32
// perturbations: each difference is a base difference between two levels, D (FP32, formed once
// a level from the FP64 profile), plus the difference of the perturbations, a - b.  a - b is a
// TwoSum pair, D is added to it by a second TwoSum, and the two low parts join the first-order
// terms of diff_dot: (D1 + a - b)(D2 + c - d) + (D3 + e - f)(D4 + g - h).
__device__ __forceinline__ void based_diff(float D, float a, float b, float& x, float& xl) {
  float p, pl, t;
  detail::two_sum(a, -b, p, pl);
  detail::two_sum(D, p, x, t);
  xl = t + pl;
}
__device__ __forceinline__ float diff_dot_based(float D1, float a, float b, float D2, float c, float d, float D3,
                                                float e, float f, float D4, float g, float h) {
  float x, xl, y, yl, z, zl, w, wl;
  based_diff(D1, a, b, x, xl);
  based_diff(D2, c, d, y, yl);
  based_diff(D3, e, f, z, zl);
  based_diff(D4, g, h, w, wl);
  const float q = z * w;
  const float qe = fmaf(z, w, -q);
  const float m = fmaf(x, y, q);
  const float low = fmaf(x, yl, fmaf(xl, y, fmaf(z, wl, fmaf(zl, w, qe))));
  return m + low;
}

}  // namespace oeb
