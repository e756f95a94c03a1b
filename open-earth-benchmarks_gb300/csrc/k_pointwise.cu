// k_pointwise.cu -- stencils whose intermediates are used only at their own point:
// laplace, uvbke, p_grad_c, nh_p_grad, hadvuv and hadvuv5th, in FP64 and FP32.
//
// FP64: compiled with --fmad=false, every a*b+c is rounded twice, exactly as the reference
// compiled without FP contraction, and double division and square root are IEEE
// round-to-nearest on both sides, so the results are bit-identical to the reference
// OpenMP kernels.  Expression trees keep the reference's order and parenthesisation; a
// subexpression that occurs twice in the reference is computed once here (same operands,
// same value).  FP32: the same trees in float (the advection stencils are then bit-identical
// to the reference compiled for float), except where cancellation costs digits
// (precision.cuh): the laplacian as a sum of neighbour differences, and the paired products
// of the pressure-gradient stencils by Kahan's FMA algorithm over error-free differences.
//
// The adjoint kernels reproduce no reference arithmetic: their accumulations use explicit
// fma() (one rounding, half the FP64 instructions), which --fmad=false does not affect.  The
// state values that decide their branches are recomputed exactly as the forward computes them.
//
// One CTA of 32 x 8 threads covers a 32 x 32 (i, j) tile and kb k-levels; each thread
// computes 4 rows.  Neighbour reads go through L1.
#include <type_traits>

#include "precision.cuh"
#include "stage.cuh"
#include "stencil_util.cuh"
#include "tangent.cuh"
#include "fused.cuh"

// Built on its own, this file's bodies and helpers are local to it; the step kernel
// (step.cu) includes it with OEB_BODIES_ONLY and a namespace of its own instead.
#ifndef OEB_BODIES_NS
#define OEB_BODIES_NS
#endif
namespace oeb {
namespace OEB_BODIES_NS {

constexpr int kTI = 32, kTJ = 32, kRows = kTJ / kTY;

// Tile width and height (cells) of tile shape S (tuned_shape): 32 x 32, 32 x 8, 64 x 16.
template <int S>
struct TileOf {
  static constexpr int I = S == 2 ? 64 : 32;
  static constexpr int J = S == 0 ? 32 : S == 1 ? 8 : 16;
};

// Visits the points of this thread in a TI x TJ tile: TI / 32 columns 32 apart, TJ / 8 rows 8
// apart (U of them unrolled); f(o, j) with o the in-plane offset of (i, j) plus the plane
// offset of k.
template <int TI, int TJ, int U, class F>
__device__ __forceinline__ void for_points_tile(const uint3& blk, const Dims& d, int kb, F&& f) {
  const int k0 = blk.z * kb;
  const int k1 = min(k0 + kb, d.nz);
  const int sj = (int)d.sj;
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
#pragma unroll 1
    for (int c = 0; c < TI / 32; ++c) {
      const int i = blk.x * TI + 32 * c + threadIdx.x;
      if (i < d.nx) {
#pragma unroll U
        for (int r = 0; r < TJ / kTY; ++r) {
          const int j = blk.y * TJ + threadIdx.y + kTY * r;
          if (j < d.ny) f(kofs + i + j * sj, j);
        }
      }
    }
  }
}

// Visits the points of this thread: f(o, j) with o the in-plane offset of (i, j) plus the
// plane offset of k.
template <int U = kRows, class F>
__device__ __forceinline__ void for_points(const uint3& blk, const Dims& d, int kb, F&& f) {
  const int i = blk.x * kTI + threadIdx.x;
  if (i >= d.nx) return;
  const int k0 = blk.z * kb;
  const int k1 = min(k0 + kb, d.nz);
  const int sj = (int)d.sj;
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
#pragma unroll U
    for (int r = 0; r < kRows; ++r) {
      const int j = blk.y * kTJ + threadIdx.y + kTY * r;
      if (j < d.ny) f(kofs + i + j * sj, j);
    }
  }
}

// The FP32 nh_p_grad waits on its global loads (ncu: long-scoreboard stalls, DRAM under 30 %
// busy): the CTA first asks L2 for its tile of every field it reads, at each of its k-levels
// (`now`) and the level above (`up`, the fields read at k+1) -- 7 % faster at 256 x 256 x 80
// (the same made p_grad_c 7 % slower; it is not used there).  The FP64 kernels are bound by
// arithmetic and skip it.
template <class T, int N, int M>
__device__ __forceinline__ void prefetch_points(const uint3& blk, const Dims& d, int kb, const T* const (&now)[N],
                                                const T* const (&up)[M]) {
  if constexpr (std::is_same<T, float>::value) {
    const int i0 = blk.x * kTI, j0 = blk.y * kTJ, sj = (int)d.sj;
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
    for (int k = k0; k < k1; ++k) {
      prefetch_tile(now, (int64_t)k * d.sk, i0, j0, d.nx, d.ny, sj);
      prefetch_tile(up, (int64_t)(k + 1) * d.sk, i0, j0, d.nx, d.ny, sj);
    }
  }
}

// ---- laplace: kernels/laplace.h:34-43 ----------------------------------------------
template <class T>
struct laplace_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, const T* __restrict__ in, T* __restrict__ out, Dims d,
                                             int kb) {
    const int64_t sj = d.sj;
    for_points<RowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int) {
      if constexpr (Prec<T>::kCompensated) {
        // -4 in nearly cancels the neighbour sum on smooth fields.  FP32 sums the four
        // neighbour differences instead: each is exact where the neighbours lie within a factor
        // 2 (Sterbenz), and the sum then cancels no more than the differences themselves --
        // about the accuracy of a compensated five-term sum, in 7 operations instead of 30.
        const T c = ld(in + o);
        out[o] = ((ld(in + o - 1) - c) + (ld(in + o + 1) - c)) + ((ld(in + o + sj) - c) + (ld(in + o - sj) - c));
      } else {
        out[o] = -scale2<2>(ld(in + o)) + ((ld(in + o - 1) + ld(in + o + 1)) + (ld(in + o + sj) + ld(in + o - sj)));
      }
    });
  }
};

// ---- uvbke: kernels/uvbke.h:61-75 ----------------------------------------------------
// dt5 is a double in every precision (src/uvbke.cpp:11-12), so the reference compiled for
// float multiplies by it in double and rounds once.  The FP32 kernel gets dt5 as a float
// pair hi + lo (exact to 48 bits) and forms dt5 * t * rs with TwoProduct and fmaf, which
// rounds about as the reference does.
template <class T>
__device__ __forceinline__ T uvbke_scale(T t, T rs, T dt5_hi, T dt5_lo) {
  if constexpr (Prec<T>::kCompensated) {
    const T p = t * rs, pe = fmaf(t, rs, -p);  // t * rs = p + pe exactly
    return fmaf(dt5_hi, p, fmaf(dt5_hi, pe, dt5_lo * p));
  } else {
    return (dt5_hi * t) * rs;
  }
}

template <class T>
struct uvbke_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ ub, T* __restrict__ vb,
                                             const T* __restrict__ uc, const T* __restrict__ vc,
                                             const T* __restrict__ cosa, const T* __restrict__ rsina, T dt5, T dt5_lo,
                                             Dims d, int kb) {
    const int64_t sj = d.sj;
    for_points<RowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int) {
      const T su = ld(uc + o - sj) + ld(uc + o);
      const T sv = ld(vc + o - 1) + ld(vc + o);
      const T ca = ld(cosa + o);
      const T rs = ld(rsina + o);
      ub[o] = uvbke_scale(su - (sv * ca), rs, dt5, dt5_lo);
      vb[o] = uvbke_scale(sv - (su * ca), rs, dt5, dt5_lo);
    });
  }
};

// ---- p_grad_c: kernels/p_grad_c.h:80-101 ---------------------------------------------
template <class T>
struct p_grad_c_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uout, T* __restrict__ vout,
                                             const T* __restrict__ uin, const T* __restrict__ vin,
                                             const T* __restrict__ rdxc, const T* __restrict__ rdyc,
                                             const T* __restrict__ delpc, const T* __restrict__ gz,
                                             const T* __restrict__ pkc, T dt2, Dims d, int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    for_points<RowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int) {
      const T wk = ld(delpc + o);
      const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pkc + o), pk1 = ld(pkc + o + sk);
      // the two products nearly cancel (a small pressure-gradient residual): diff_dot is the
      // reference's tree in FP64 and float-float in FP32
      const T fu = diff_dot(ld(gz + o - 1 + sk), gz0, pk1, ld(pkc + o - 1), ld(gz + o - 1), gz1, ld(pkc + o - 1 + sk), pk0);
      uout[o] = (ld(uin + o) + (((dt2 * ld(rdxc + o)) / (ld(delpc + o - 1) + wk)) * fu));
      const T fv =
          diff_dot(ld(gz + o - sj + sk), gz0, pk1, ld(pkc + o - sj), ld(gz + o - sj), gz1, ld(pkc + o - sj + sk), pk0);
      vout[o] = (ld(vin + o) + (((dt2 * ld(rdyc + o)) / (ld(delpc + o - sj) + wk)) * fv));
    });
  }
};

// ---- nh_p_grad: kernels/nh_p_grad.h:116-146 --------------------------------------------
template <class T>
struct nh_p_grad_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uout, T* __restrict__ vout,
                                             const T* __restrict__ uin, const T* __restrict__ vin,
                                             const T* __restrict__ rdx, const T* __restrict__ rdy,
                                             const T* __restrict__ gz, const T* __restrict__ pp,
                                             const T* __restrict__ pk3, const T* __restrict__ wk1, T dt, Dims d,
                                             int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    const T* const now[8] = {pk3, gz, pp, wk1, uin, vin, rdx, rdy};
    const T* const up[3] = {pk3, gz, pp};
    prefetch_points(blk, d, kb, now, up);
    for_points<HeavyRowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int) {
      const T pk0 = ld(pk3 + o), pk1 = ld(pk3 + o + sk);
      const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk);
      const T pp0 = ld(pp + o), pp1 = ld(pp + o + sk);
      const T w1 = ld(wk1 + o);
      const T wk = pk1 - pk0;
      // u: neighbour i+1
      {
        const T pkx0 = ld(pk3 + o + 1), pkx1 = ld(pk3 + o + 1 + sk);
        const T wkx = pkx1 - pkx0;
        const T gx0 = ld(gz + o + 1), gx1 = ld(gz + o + 1 + sk);
        // the two products of each sum nearly cancel: diff_dot (precision.cuh)
        const T fk = diff_dot(gz1, gx0, pkx1, pk0, gz0, gx1, pk1, pkx0);
        const T fp = diff_dot(gz1, gx0, ld(pp + o + 1 + sk), pp0, gz0, gx1, pp1, ld(pp + o + 1));
        const T du = ((dt / (wk + wkx)) * fk);
        uout[o] = (((ld(uin + o) + du) + ((dt / (w1 + ld(wk1 + o + 1))) * fp)) * ld(rdx + o));
      }
      // v: neighbour j+1
      {
        const T pky0 = ld(pk3 + o + sj), pky1 = ld(pk3 + o + sj + sk);
        const T wky = pky1 - pky0;
        const T gy0 = ld(gz + o + sj), gy1 = ld(gz + o + sj + sk);
        const T fk = diff_dot(gz1, gy0, pky1, pk0, gz0, gy1, pk1, pky0);
        const T fp = diff_dot(gz1, gy0, ld(pp + o + sj + sk), pp0, gz0, gy1, pp1, ld(pp + o + sj));
        const T dv = ((dt / (wk + wky)) * fk);
        vout[o] = (((ld(vin + o) + dv) + ((dt / (w1 + ld(wk1 + o + sj))) * fp)) * ld(rdy + o));
      }
    });
  }
};

// ---- hadvuv / hadvuv5th: kernels/hadvuv.h:4-27,178-210 and kernels/hadvuv5th.h:4-39,177-201

// The upwind sums without a branch.  Both branches of the reference's drivers are one
// left-to-right sum of the same shape -- products, one plain term, products -- and differ
// only in which coefficients and neighbours fill the slots.  Each lane selects its operands
// (integer selects, no FP64 work) and then performs exactly the operation sequence of its
// branch: the FP64 results are bit-identical to the branchy form, and a warp whose lanes
// disagree on the upwind direction no longer runs both branches.  (a > 0 ? a : -a) * sum
// is the reference's `-uavg * (...)`, the negation being exact.
//
// FP32 runs the same sequence in float: it is then bit-identical to the reference compiled
// for float.  A compensated form (TwoProduct for every term, TwoSum for every addition) was
// measured as well and dropped: its largest error against the FP64 oracle was no smaller
// (2.8e-7, the same as the plain sums' on every test case) -- the upwind sum's roundings are
// not the largest term, the products and averages around it are -- and it took about four
// times the sum's operations.

// 3rd-order upwind advection along one axis (stride s): hadvuv.h:10-16 (x) and :18-24 (y).
//   a > 0:  ((c6 f[-2] + f[-1]) + ch f[0]) + c3 f[1]
//   else :  ((c3 f[-1] + ch f[0]) + f[1]) + c6 f[2]
template <class T>
__device__ __forceinline__ T adv3_axis(const T* __restrict__ f, int64_t o, int64_t s, T a) {
  constexpr T c6 = T(-1.0) / T(6.0), c3 = T(-1.0) / T(3.0);
  const bool pos = gt0(a);
  const T fa = ld(f + o + (pos ? -2 : -1) * s), fb = ld(f + o - s), f0 = ld(f + o), fc = ld(f + o + s),
          fd = ld(f + o + (pos ? 1 : 2) * s);
  // the -1/2 term: an exact scaling
  const T p0 = (pos ? c6 : c3) * fa, ph = -scale2<-1>(f0), p3 = (pos ? c3 : c6) * fd;
  return (pos ? a : -a) * (((p0 + (pos ? fb : ph)) + (pos ? ph : fc)) + p3);
}

// 5th-order upwind advection along one axis: hadvuv5th.h:10-22 (x) and :24-36 (y).
//   a > 0:  ((((c30 f[-3] + c4 f[-2]) + f[-1]) + c3 f[0]) + c2 f[1]) + c20 f[2]
//   else :  ((((c20 f[-2] + c2 f[-1]) + c3 f[0]) + f[1]) + c4 f[2]) + c30 f[3]
template <class T>
__device__ __forceinline__ T adv5_axis(const T* __restrict__ f, int64_t o, int64_t s, T a) {
  constexpr T c30 = T(1.0) / T(30.0), c3 = T(-1.0) / T(3.0), c20 = T(1.0) / T(20.0);
  const bool pos = gt0(a);
  const int64_t sh = pos ? 0 : s;  // the negative branch reads one cell further along the axis
  const T x0 = ld(f + o - 3 * s + sh), x1 = ld(f + o - 2 * s + sh), fm1 = ld(f + o - s), f0 = ld(f + o),
          fp1 = ld(f + o + s), x4 = ld(f + o + s + sh), x5 = ld(f + o + 2 * s + sh);
  // the -1/4 and -1/2 terms: exact power-of-two scalings
  const T p0 = (pos ? c30 : c20) * x0, p1 = -scale2v(x1, pos ? -2 : -1), pm = c3 * f0, p4 = -scale2v(x4, pos ? -1 : -2),
          p5 = (pos ? c20 : c30) * x5;
  return (pos ? a : -a) * (((((p0 + p1) + (pos ? fm1 : pm)) + (pos ? pm : fp1)) + p4) + p5);
}

// update != 0 fuses the chained step's explicit update into the epilogue: the outputs are
// alpha * (the tendency) + (the input), the same two roundings as the tendency stored and then
// combined by a separate kernel.
template <class T, int ORDER, int SHAPE = 0>
struct hadv_kernel {
  static constexpr int kStepOp = step_op<T>(ORDER == 5 ? kOpHadv5Fwd + SHAPE : -1);  // the step kernel's id
  static constexpr int kShape = SHAPE;
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uout, T* __restrict__ vout,
                                             const T* __restrict__ uin, const T* __restrict__ vin,
                                             const T* __restrict__ acrlat0, const T* __restrict__ acrlat1,
                                             const T* __restrict__ tgrlatda0, const T* __restrict__ tgrlatda1,
                                             int64_t s1d, T eddlat, T eddlon, Dims d, int kb, T alpha, int update) {
    const int64_t sj = d.sj;
    constexpr T third = T(1.0) / T(3.0);
    constexpr T rr = earth_radius_recip<T>();
    for_points_tile<TileOf<SHAPE>::I, TileOf<SHAPE>::J, HeavyRowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int j) {
      const int64_t jo = (int64_t)j * s1d;
      const T u0 = ld(uin + o), v0 = ld(vin + o);
      const T um = ld(uin + o - 1) + u0;  // uin(i-1)+uin(i), first pair of both averages
      // u at the u-position and v at the u-position (hadvuv.h:186-189)
      const T u_atupos = third * (um + ld(uin + o + 1));
      const T v_atupos = scale2<-2>(((ld(vin + o + 1) + ld(vin + o + 1 - sj)) + v0) + ld(vin + o - sj));
      T ua = ld(acrlat0 + jo) * u_atupos;
      T va = rr * v_atupos;
      T rx, ry;
      if (ORDER == 3) {
        rx = adv3_axis(uin, o, 1, ua);
        ry = adv3_axis(uin, o, sj, va);
      } else {
        rx = adv5_axis(uin, o, 1, ua);
        ry = adv5_axis(uin, o, sj, va);
      }
      const T ures = eddlat * rx + eddlon * ry;
      const T ut = ures + (ld(tgrlatda0 + jo) * u0) * v_atupos;
      uout[o] = update ? alpha * ut + u0 : ut;
      // u and v at the v-position (hadvuv.h:197-206)
      const T u_atvpos = scale2<-2>(((um) + ld(uin + o + sj)) + ld(uin + o - 1 + sj));
      const T v_atvpos = third * ((ld(vin + o - sj) + v0) + ld(vin + o + sj));
      ua = ld(acrlat1 + jo) * u_atvpos;
      va = rr * v_atvpos;
      if (ORDER == 3) {
        rx = adv3_axis(vin, o, 1, ua);
        ry = adv3_axis(vin, o, sj, va);
      } else {
        rx = adv5_axis(vin, o, 1, ua);
        ry = adv5_axis(vin, o, sj, va);
      }
      const T vres = eddlat * rx + eddlon * ry;
      const T vt = vres - (ld(tgrlatda1 + jo) * u_atvpos) * u_atvpos;
      vout[o] = update ? alpha * vt + v0 : vt;
    });
  }
};

constexpr int kKB = 1;  // k-levels per CTA (one: the most CTAs, which hides FP64 and load latency best)

// ---- FP32 forms staged through shared memory (stage.cuh) -----------------------------
// laplace and nh_p_grad: a CTA owns a 32 x 32 tile and the k-levels [k0, k0+kb); the input
// boxes read at neighbouring points are copied level by level into a ring of NB shared-memory
// buffers by cp.async, ahead of the level being computed.  nh_p_grad reads level k+1 as well,
// so it computes level k once levels k and k+1 are resident, with one more level in flight;
// laplace keeps two levels in flight.  Measured at 256 x 256 x 80 (each stencil alone, average
// over back-to-back launches): laplace 0.38 -> 0.49 of the HBM copy rate, nh_p_grad 0.32 ->
// 0.42.  uvbke and p_grad_c measured faster as the plain kernels above (0.69 and 0.60 against
// 0.62 and 0.48 staged) and keep them: their loads are all independent, and eight CTAs an SM
// of plain loads keep more bytes in flight than the two or four CTAs their staged rings allowed.

// Marches the levels of a staged CTA: issue(k) copies level k (or commits an empty group),
// compute(k) reads the resident levels k .. k+LEAD; NB - 1 - LEAD levels are in flight while
// level k is computed.
template <int NB, int LEAD, class Issue, class Compute>
__device__ __forceinline__ void staged_march(int k0, int k1, Issue&& issue, Compute&& compute) {
  static_assert(NB >= LEAD + 2, "at least one level in flight beyond those a level reads");
#pragma unroll 1
  for (int t = 0; t < NB - 1; ++t) issue(k0 + t);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    issue(k + NB - 1);  // into the buffer level k-1 left
    cp_async_wait<NB - 1 - LEAD>();  // every level up to k + LEAD has landed
    __syncthreads();
    compute(k);
    __syncthreads();  // the buffer of level k is refilled next
  }
}

// laplace.h:39, FP32: one 34 x 34 box of `in` a level, summed in the difference form of
// laplace_kernel above.
struct laplace_staged_f32 {
  static constexpr int NB = 3;
  static constexpr int kCtasPerSm = 8;
  using B = RowBox<34, 34>;
  struct Smem {
    float in[NB][B::N];
  };
  static __device__ __forceinline__ void run(const uint3& blk, const float* __restrict__ in, float* __restrict__ out,
                                             Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    const int i0 = blk.x * kTI, j0 = blk.y * kTJ;
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
    const int ie = min(i0 + kTI, d.nx), je = min(j0 + kTJ, d.ny);
    auto issue = [&](int k) {
      if (k < k1)
        stage_rows<34, 34>(s.in[k % NB], in, (int64_t)k * d.sk, i0 - 1, j0 - 1, d.sj, i0 - 1, ie + 1, j0 - 1, je + 1);
      cp_async_commit();
    };
    staged_march<NB, 0>(k0, k1, issue, [&](int k) {
      const int64_t kofs = (int64_t)k * d.sk;
      const RowMis mis = row_mis(in, kofs, i0 - 1, j0 - 1, d.sj);
      const float* t = s.in[k % NB];
      const int a = threadIdx.x, i = i0 + a;
      if (i >= ie) return;
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        const int b = threadIdx.y + kTY * r, j = j0 + b;
        if (j < je) {
          const float* up = t + b * B::SW + mis(b) + a;  // row j-1 from cell i-1
          const float* mid = t + (b + 1) * B::SW + mis(b + 1) + a;
          const float* dn = t + (b + 2) * B::SW + mis(b + 2) + a;
          const float c = mid[1];
          out[kofs + i + (int64_t)j * d.sj] = ((mid[0] - c) + (mid[2] - c)) + ((dn[1] - c) + (up[1] - c));
        }
      }
    });
  }
};

// The four fields a staged nh_p_grad thread reads at its own points only, loaded into registers
// one level ahead of the level it computes (the loads of level k+1 are in flight while level k
// is computed).
struct PointRegs {
  float v[4][kRows];
  __device__ __forceinline__ void fetch(const float* __restrict__ f0, const float* __restrict__ f1,
                                        const float* __restrict__ f2, const float* __restrict__ f3, int64_t kofs,
                                        int i, int j0, int je, int64_t sj) {
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      const int j = j0 + (int)threadIdx.y + kTY * r;
      const bool ok = j < je;
      const int64_t o = kofs + i + (int64_t)(ok ? j : j0) * sj;
      v[0][r] = ok ? ld(f0 + o) : 0.f;
      v[1][r] = ok ? ld(f1 + o) : 0.f;
      v[2][r] = ok ? ld(f2 + o) : 0.f;
      v[3][r] = ok ? ld(f3 + o) : 0.f;
    }
  }
};

// nh_p_grad.h:121-141, FP32: gz, pp, pk3 staged on 33 x 33 from (i0, j0) at k and k+1, wk1 at
// k; uin, vin, rdx, rdy in registers a level ahead.
struct nh_p_grad_staged_f32 {
  static constexpr int NB = 3;
  static constexpr int kCtasPerSm = 3;
  static constexpr int kMinCtas = 3;  // registers for three CTAs an SM
  using Q = RowBox<33, 33>;
  struct Level {
    float gz[Q::N], pp[Q::N], pk[Q::N], w1[Q::N];
  };
  struct Smem {
    Level l[NB];
  };
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uout, float* __restrict__ vout,
                                             const float* __restrict__ uin, const float* __restrict__ vin,
                                             const float* __restrict__ rdx, const float* __restrict__ rdy,
                                             const float* __restrict__ gz, const float* __restrict__ pp,
                                             const float* __restrict__ pk3, const float* __restrict__ wk1, float dt,
                                             Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    const int i0 = blk.x * kTI, j0 = blk.y * kTJ;
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
    const int ie = min(i0 + kTI, d.nx), je = min(j0 + kTJ, d.ny);
    const int a = threadIdx.x, i = i0 + a;
    const int ic = i < ie ? i : i0;  // a column of the tile for the register loads
    auto issue = [&](int k) {
      if (k <= k1) {  // level k1 only for the fields read at k+1
        const int64_t ko = (int64_t)k * d.sk;
        Level& L = s.l[k % NB];
        if (k < k1) stage_rows<33, 33>(L.w1, wk1, ko, i0, j0, d.sj, i0, ie + 1, j0, je + 1);
        stage_rows<33, 33>(L.gz, gz, ko, i0, j0, d.sj, i0, ie + 1, j0, je + 1);
        stage_rows<33, 33>(L.pp, pp, ko, i0, j0, d.sj, i0, ie + 1, j0, je + 1);
        stage_rows<33, 33>(L.pk, pk3, ko, i0, j0, d.sj, i0, ie + 1, j0, je + 1);
      }
      cp_async_commit();
    };
    PointRegs cur;
    cur.fetch(uin, vin, rdx, rdy, (int64_t)k0 * d.sk, ic, j0, je, d.sj);
    staged_march<NB, 1>(k0, k1, issue, [&](int k) {
      PointRegs nxt;
      if (k + 1 < k1) nxt.fetch(uin, vin, rdx, rdy, (int64_t)(k + 1) * d.sk, ic, j0, je, d.sj);
      const int64_t kofs = (int64_t)k * d.sk, kofs1 = kofs + d.sk;
      const Level& C = s.l[k % NB];
      const Level& N = s.l[(k + 1) % NB];
      const RowMis mw = row_mis(wk1, kofs, i0, j0, d.sj);
      const RowMis mg0 = row_mis(gz, kofs, i0, j0, d.sj), mg1 = row_mis(gz, kofs1, i0, j0, d.sj);
      const RowMis mq0 = row_mis(pp, kofs, i0, j0, d.sj), mq1 = row_mis(pp, kofs1, i0, j0, d.sj);
      const RowMis mp0 = row_mis(pk3, kofs, i0, j0, d.sj), mp1 = row_mis(pk3, kofs1, i0, j0, d.sj);
      if (i < ie) {
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
          const int b = threadIdx.y + kTY * r, j = j0 + b;
          if (j < je) {
            // rows j (box row b) and j+1 (box row b+1); cell i is a in them
            const float* wc = C.w1 + b * Q::SW + mw(b) + a;
            const float* wn = C.w1 + (b + 1) * Q::SW + mw(b + 1) + a;
            const float* g0c = C.gz + b * Q::SW + mg0(b) + a;
            const float* g0n = C.gz + (b + 1) * Q::SW + mg0(b + 1) + a;
            const float* g1c = N.gz + b * Q::SW + mg1(b) + a;
            const float* g1n = N.gz + (b + 1) * Q::SW + mg1(b + 1) + a;
            const float* q0c = C.pp + b * Q::SW + mq0(b) + a;
            const float* q0n = C.pp + (b + 1) * Q::SW + mq0(b + 1) + a;
            const float* q1c = N.pp + b * Q::SW + mq1(b) + a;
            const float* q1n = N.pp + (b + 1) * Q::SW + mq1(b + 1) + a;
            const float* p0c = C.pk + b * Q::SW + mp0(b) + a;
            const float* p0n = C.pk + (b + 1) * Q::SW + mp0(b + 1) + a;
            const float* p1c = N.pk + b * Q::SW + mp1(b) + a;
            const float* p1n = N.pk + (b + 1) * Q::SW + mp1(b + 1) + a;
            const float pk0 = p0c[0], pk1 = p1c[0], gz0 = g0c[0], gz1 = g1c[0], pp0 = q0c[0], pp1 = q1c[0];
            const float w1 = wc[0];
            const float wk = pk1 - pk0;
            const int64_t o = kofs + i + (int64_t)j * d.sj;
            {  // u: neighbour i+1
              const float pkx0 = p0c[1], pkx1 = p1c[1];
              const float wkx = pkx1 - pkx0;
              const float gx0 = g0c[1], gx1 = g1c[1];
              const float fk = diff_dot(gz1, gx0, pkx1, pk0, gz0, gx1, pk1, pkx0);
              const float fp = diff_dot(gz1, gx0, q1c[1], pp0, gz0, gx1, pp1, q0c[1]);
              const float du = ((dt / (wk + wkx)) * fk);
              uout[o] = (((cur.v[0][r] + du) + ((dt / (w1 + wc[1])) * fp)) * cur.v[2][r]);
            }
            {  // v: neighbour j+1
              const float pky0 = p0n[0], pky1 = p1n[0];
              const float wky = pky1 - pky0;
              const float gy0 = g0n[0], gy1 = g1n[0];
              const float fk = diff_dot(gz1, gy0, pky1, pk0, gz0, gy1, pk1, pky0);
              const float fp = diff_dot(gz1, gy0, q1n[0], pp0, gz0, gy1, pp1, q0n[0]);
              const float dv = ((dt / (wk + wky)) * fk);
              vout[o] = (((cur.v[1][r] + dv) + ((dt / (w1 + wn[0])) * fp)) * cur.v[3][r]);
            }
          }
        }
      }
      cur = nxt;
    });
  }
};

// Grid and k-levels a CTA of a staged body: about one wave of CTAs (stage.cuh).
template <class S>
void staged_launch_shape(const oeb_domain& dom, dim3* grid, int* kb) {
  const int tiles = (int)(((dom.nx + kTI - 1) / kTI) * ((dom.ny + kTJ - 1) / kTJ));
  *kb = tuned_kb(staged_kb(tiles, (int)dom.nz, S::kCtasPerSm));
  *grid = tile_grid((int)dom.nx, (int)dom.ny, (int)dom.nz, kTI, kTJ, *kb);
}

template <class T>
Dims make_dims(const oeb_domain& dom, const Grid<T>& g) {
  return Dims{(int)dom.nx, (int)dom.ny, (int)dom.nz, g.sj, g.sk};
}

dim3 grid_for(const oeb_domain& dom, int kb) { return tile_grid((int)dom.nx, (int)dom.ny, (int)dom.nz, kTI, kTJ, kb); }

// ------------------------------ entry points -----------------------------------------

template <class T, class M3>
oeb_status laplace_entry(const M3* in, const M3* out, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gin, gout;
  OEB_TRY((check_field3<T>(in, *dom, Reach{1, 1, 1, 1, 0, 0}, &gin)));
  OEB_TRY((check_field3<T>(out, *dom, kInterior, &gout)));
  OEB_TRY(check_same_strides<T>({&gin, &gout}));
  OEB_TRY(check_no_alias({gout.lo, gout.hi}, {gin.lo, gin.hi}));
  OEB_RETURN_IF_VALIDATING();
  if constexpr (std::is_same<T, float>::value) if (!fields_in_host_memory()) {
    dim3 grid;
    int kb;
    staged_launch_shape<laplace_staged_f32>(*dom, &grid, &kb);
    return launch<laplace_staged_f32>(grid, sizeof(laplace_staged_f32::Smem), (cudaStream_t)stream, gin.origin,
                                      gout.origin, make_dims(*dom, gin), kb);
  }
  const int kb = tuned_kb(kKB);
  return launch<laplace_kernel<T>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, gin.origin, gout.origin,
                                   make_dims(*dom, gin), kb);
}

template <class T, class M3>
oeb_status uvbke_entry(const M3* ub, const M3* vb, const M3* uc, const M3* vc, const M3* cosa, const M3* rsina,
                       double dt5, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gub, gvb, guc, gvc, gca, grs;
  OEB_TRY((check_field3<T>(ub, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<T>(vb, *dom, kInterior, &gvb)));
  OEB_TRY((check_field3<T>(uc, *dom, Reach{0, 0, 1, 0, 0, 0}, &guc)));
  OEB_TRY((check_field3<T>(vc, *dom, Reach{1, 0, 0, 0, 0, 0}, &gvc)));
  OEB_TRY((check_field3<T>(cosa, *dom, kInterior, &gca)));
  OEB_TRY((check_field3<T>(rsina, *dom, kInterior, &grs)));
  OEB_TRY(check_same_strides<T>({&gub, &gvb, &guc, &gvc, &gca, &grs}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi},
                         {guc.lo, guc.hi, gvc.lo, gvc.hi, gca.lo, gca.hi, grs.lo, grs.hi}));
  OEB_RETURN_IF_VALIDATING();
  const T dt5_hi = T(dt5), dt5_lo = T(dt5 - (double)dt5_hi);  // dt5_lo = 0 for FP64
  const int kb = tuned_kb(kKB);
  return launch<uvbke_kernel<T>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, gub.origin, gvb.origin, guc.origin,
                                 gvc.origin, gca.origin, grs.origin, dt5_hi, dt5_lo, make_dims(*dom, gub), kb);
}

// The descriptors' checks of p_grad_c (g: uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc).
template <class T, class M3>
oeb_status p_grad_c_check(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdxc,
                          const M3* rdyc, const M3* delpc, const M3* gz, const M3* pkc, const oeb_domain* dom,
                          Grid<T> (&g)[9]) {
  OEB_TRY(check_domain(dom));
  const M3* f[9] = {uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc};
  const Reach reach[9] = {kInterior, kInterior, kInterior, kInterior, kInterior, kInterior,
                          Reach{1, 0, 1, 0, 0, 0}, Reach{1, 0, 1, 0, 0, 1}, Reach{1, 0, 1, 0, 0, 1}};
  for (int q = 0; q < 9; ++q) OEB_TRY((check_field3<T>(f[q], *dom, reach[q], &g[q])));
  OEB_TRY(check_same_strides<T>({&g[0], &g[1], &g[2], &g[3], &g[4], &g[5], &g[6], &g[7], &g[8]}));
  return check_no_alias({g[0].lo, g[0].hi, g[1].lo, g[1].hi},
                        {g[2].lo, g[2].hi, g[3].lo, g[3].hi, g[4].lo, g[4].hi, g[5].lo, g[5].hi, g[6].lo, g[6].hi,
                         g[7].lo, g[7].hi, g[8].lo, g[8].hi});
}

template <class T, class M3>
oeb_status p_grad_c_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdxc,
                          const M3* rdyc, const M3* delpc, const M3* gz, const M3* pkc, T dt2,
                          const oeb_domain* dom, void* stream) {
  Grid<T> g[9];
  OEB_TRY(p_grad_c_check<T>(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, dom, g));
  OEB_RETURN_IF_VALIDATING();
  const int kb = tuned_kb(kKB);
  return launch<p_grad_c_kernel<T>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, g[0].origin, g[1].origin,
                                    g[2].origin, g[3].origin, g[4].origin, g[5].origin, g[6].origin, g[7].origin,
                                    g[8].origin, dt2, make_dims(*dom, g[0]), kb);
}

// The descriptors' checks of nh_p_grad (g: uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1).
template <class T, class M3>
oeb_status nh_p_grad_check(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdx,
                           const M3* rdy, const M3* gz, const M3* pp, const M3* pk3, const M3* wk1,
                           const oeb_domain* dom, Grid<T> (&g)[10]) {
  OEB_TRY(check_domain(dom));
  const M3* f[10] = {uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1};
  const Reach r11 = Reach{0, 1, 0, 1, 0, 1};
  const Reach reach[10] = {kInterior, kInterior, kInterior, kInterior, kInterior, kInterior, r11, r11, r11,
                           Reach{0, 1, 0, 1, 0, 0}};
  for (int q = 0; q < 10; ++q) OEB_TRY((check_field3<T>(f[q], *dom, reach[q], &g[q])));
  OEB_TRY(check_same_strides<T>({&g[0], &g[1], &g[2], &g[3], &g[4], &g[5], &g[6], &g[7], &g[8], &g[9]}));
  return check_no_alias({g[0].lo, g[0].hi, g[1].lo, g[1].hi},
                        {g[2].lo, g[2].hi, g[3].lo, g[3].hi, g[4].lo, g[4].hi, g[5].lo, g[5].hi, g[6].lo, g[6].hi,
                         g[7].lo, g[7].hi, g[8].lo, g[8].hi, g[9].lo, g[9].hi});
}

template <class T, class M3>
oeb_status nh_p_grad_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdx,
                           const M3* rdy, const M3* gz, const M3* pp, const M3* pk3, const M3* wk1, T dt,
                           const oeb_domain* dom, void* stream) {
  Grid<T> g[10];
  OEB_TRY(nh_p_grad_check<T>(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, dom, g));
  OEB_RETURN_IF_VALIDATING();
  if constexpr (std::is_same<T, float>::value) if (!fields_in_host_memory()) {
    dim3 grid;
    int kb;
    staged_launch_shape<nh_p_grad_staged_f32>(*dom, &grid, &kb);
    return launch<nh_p_grad_staged_f32>(grid, sizeof(nh_p_grad_staged_f32::Smem), (cudaStream_t)stream, g[0].origin,
                                        g[1].origin, g[2].origin, g[3].origin, g[4].origin, g[5].origin, g[6].origin,
                                        g[7].origin, g[8].origin, g[9].origin, dt, make_dims(*dom, g[0]), kb);
  }
  const int kb = tuned_kb(kKB);
  return launch<nh_p_grad_kernel<T>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, g[0].origin, g[1].origin,
                                     g[2].origin, g[3].origin, g[4].origin, g[5].origin, g[6].origin, g[7].origin,
                                     g[8].origin, g[9].origin, dt, make_dims(*dom, g[0]), kb);
}

// ---- FP32 pressure gradients on profile-relative fields ---------------------------------
// The pressure, geopotential and Exner fields of these stencils are a per-level profile plus
// a small perturbation, and the stencils difference them between neighbouring points and
// levels, where the profile nearly cancels: stored in FP32, their rounding (2^-24 of values
// about 100 times the perturbations) then dominates the outputs' error.  These forms take the
// fields as FP32 perturbations from an FP64 base profile b(k) (one value a level): a
// difference between levels k + 1 and k is the base difference b(k+1) - b(k) (formed once a
// level in FP64, rounded once to FP32) plus the perturbations' difference, and one between
// points of a level is the perturbations' difference alone.  Same expression trees as
// p_grad_c_kernel / nh_p_grad_kernel in FP32, with diff_dot_based for the paired products.

// Visits this thread's points of the CTA's 32 x 32 tile at its levels [k0, k1); f(o, D) gets
// D[q] = float(base_q[k+1] - base_q[k]) of the point's level k.  FP64 is a narrow pipe on this
// GPU, so the differences are formed once a CTA or a warp, not a thread, in one of two ways
// (measured at 256 x 256 x 80, one level a CTA):
// * SMEM: before each chunk of up to kLevelChunk levels, NB x chunk threads write them to
//   shared memory between two barriers (p_grad_c 59-63 us, 65 us by shuffles);
// * shuffles: a warp is one row of 32 threads, all at the same level; lane q < NB forms D[q]
//   and the warp shares it by __shfl_sync, with no barrier (nh_p_grad 101 us, 119 us in
//   shared memory).
// Every thread of the CTA reaches each barrier and shuffle: the chunk and level loops depend
// on blk only, and threads outside the tile skip the work, not the loops.
constexpr int kLevelChunk = 32;
template <int NB, int U, bool SMEM, class F>
__device__ __forceinline__ void for_points_profiled(const uint3& blk, const Dims& d, int kb,
                                                    const double* const (&base)[NB], F&& f) {
  static_assert(NB * kLevelChunk <= kThreads && kTX == 32, "a warp is one row of threads");
  const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  const int lane = threadIdx.x;
  const int i = blk.x * kTI + lane;
  const int sj = (int)d.sj;
  auto rows = [&](int k, const float (&D)[NB]) {
    if (i >= d.nx) return;
    const int64_t kofs = (int64_t)k * d.sk;
#pragma unroll U
    for (int r = 0; r < kRows; ++r) {
      const int j = blk.y * kTJ + threadIdx.y + kTY * r;
      if (j < d.ny) f(kofs + i + j * sj, D);
    }
  };
  // base[q] for a run-time q, by constant indices (no local-memory copy of base)
  auto pick = [&](int q) {
    const double* b = base[0];
#pragma unroll
    for (int p = 1; p < NB; ++p)
      if (q == p) b = base[p];
    return b;
  };
  if constexpr (SMEM) {
    __shared__ float lv[NB][kLevelChunk];
    const int t = threadIdx.y * kTX + lane;
    for (int c0 = k0; c0 < k1; c0 += kLevelChunk) {
      const int c1 = min(c0 + kLevelChunk, k1);
      __syncthreads();  // the previous chunk's readers are done with lv
      if (t < NB * kLevelChunk) {
        const int q = t / kLevelChunk, k = c0 + t % kLevelChunk;
        const double* bq = pick(q);
        if (k < c1) lv[q][k - c0] = (float)(ld(bq + k + 1) - ld(bq + k));
      }
      __syncthreads();
#pragma unroll 1
      for (int k = c0; k < c1; ++k) {
        float D[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) D[q] = lv[q][k - c0];
        rows(k, D);
      }
    }
  } else {
    const double* bl = pick(lane);
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const float mine = lane < NB ? (float)(ld(bl + k + 1) - ld(bl + k)) : 0.0f;
      float D[NB];
#pragma unroll
      for (int q = 0; q < NB; ++q) D[q] = __shfl_sync(0xffffffffu, mine, q);
      rows(k, D);
    }
  }
}

struct p_grad_c_profiled_f32 {
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uout, float* __restrict__ vout,
                                             const float* __restrict__ uin, const float* __restrict__ vin,
                                             const float* __restrict__ rdxc, const float* __restrict__ rdyc,
                                             const float* __restrict__ delpc, const float* __restrict__ gz,
                                             const float* __restrict__ pkc, const double* __restrict__ gz_base,
                                             const double* __restrict__ pkc_base, float dt2, Dims d, int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    const double* const base[2] = {gz_base, pkc_base};
    for_points_profiled<2, RowUnroll<float>::value, true>(blk, d, kb, base, [&](int64_t o, const float (&D)[2]) {
      const float G = D[0], K = D[1];
      const float wk = ld(delpc + o);
      const float gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pkc + o), pk1 = ld(pkc + o + sk);
      // gz(p-s,k+1) - gz0, pk1 - pkc(p-s), gz(p-s) - gz1, pkc(p-s,k+1) - pk0 (p_grad_c.h:90-97)
      const float fu = diff_dot_based(G, ld(gz + o - 1 + sk), gz0, K, pk1, ld(pkc + o - 1), -G, ld(gz + o - 1), gz1,
                                      K, ld(pkc + o - 1 + sk), pk0);
      uout[o] = (ld(uin + o) + (((dt2 * ld(rdxc + o)) / (ld(delpc + o - 1) + wk)) * fu));
      const float fv = diff_dot_based(G, ld(gz + o - sj + sk), gz0, K, pk1, ld(pkc + o - sj), -G, ld(gz + o - sj), gz1,
                                      K, ld(pkc + o - sj + sk), pk0);
      vout[o] = (ld(vin + o) + (((dt2 * ld(rdyc + o)) / (ld(delpc + o - sj) + wk)) * fv));
    });
  }
};

struct nh_p_grad_profiled_f32 {
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uout, float* __restrict__ vout,
                                             const float* __restrict__ uin, const float* __restrict__ vin,
                                             const float* __restrict__ rdx, const float* __restrict__ rdy,
                                             const float* __restrict__ gz, const float* __restrict__ pp,
                                             const float* __restrict__ pk3, const float* __restrict__ wk1,
                                             const double* __restrict__ gz_base, const double* __restrict__ pp_base,
                                             const double* __restrict__ pk3_base, float dt, Dims d, int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    const double* const base[3] = {gz_base, pp_base, pk3_base};
    for_points_profiled<3, kRows, false>(blk, d, kb, base, [&](int64_t o, const float (&D)[3]) {
      const float G = D[0], P = D[1], K = D[2];
      const float pk0 = ld(pk3 + o), pk1 = ld(pk3 + o + sk);
      const float gz0 = ld(gz + o), gz1 = ld(gz + o + sk);
      const float pp0 = ld(pp + o), pp1 = ld(pp + o + sk);
      const float w1 = ld(wk1 + o);
      const float wk = K + (pk1 - pk0);  // pk3(k+1) - pk3(k)
      // u: neighbour i+1 (nh_p_grad.h:121-131)
      {
        const float pkx0 = ld(pk3 + o + 1), pkx1 = ld(pk3 + o + 1 + sk);
        const float wkx = K + (pkx1 - pkx0);
        const float gx0 = ld(gz + o + 1), gx1 = ld(gz + o + 1 + sk);
        const float fk = diff_dot_based(G, gz1, gx0, K, pkx1, pk0, -G, gz0, gx1, K, pk1, pkx0);
        const float fp = diff_dot_based(G, gz1, gx0, P, ld(pp + o + 1 + sk), pp0, -G, gz0, gx1, P, pp1, ld(pp + o + 1));
        const float du = ((dt / (wk + wkx)) * fk);
        uout[o] = (((ld(uin + o) + du) + ((dt / (w1 + ld(wk1 + o + 1))) * fp)) * ld(rdx + o));
      }
      // v: neighbour j+1 (nh_p_grad.h:132-142)
      {
        const float pky0 = ld(pk3 + o + sj), pky1 = ld(pk3 + o + sj + sk);
        const float wky = K + (pky1 - pky0);
        const float gy0 = ld(gz + o + sj), gy1 = ld(gz + o + sj + sk);
        const float fk = diff_dot_based(G, gz1, gy0, K, pky1, pk0, -G, gz0, gy1, K, pk1, pky0);
        const float fp =
            diff_dot_based(G, gz1, gy0, P, ld(pp + o + sj + sk), pp0, -G, gz0, gy1, P, pp1, ld(pp + o + sj));
        const float dv = ((dt / (wk + wky)) * fk);
        vout[o] = (((ld(vin + o) + dv) + ((dt / (w1 + ld(wk1 + o + sj))) * fp)) * ld(rdy + o));
      }
    });
  }
};

template <class T, int ORDER, class M3, class M1>
oeb_status hadv_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M1* acrlat0,
                      const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, T eddlat, T eddlon,
                      const oeb_domain* dom, void* stream, T alpha = T(0), int update = 0) {
  OEB_TRY(check_domain(dom));
  const int h = ORDER == 3 ? 2 : 3;
  Grid<T> gu, gv, gui, gvi;
  Line<T> a0, a1, t0, t1;
  OEB_TRY((check_field3<T>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<T>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<T>(uin, *dom, Reach{h, h, h, h, 0, 0}, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, Reach{h, h, h, h, 0, 0}, &gvi)));
  OEB_TRY((check_field1<T>(acrlat0, *dom, 0, 0, &a0)));
  OEB_TRY((check_field1<T>(acrlat1, *dom, 0, 0, &a1)));
  OEB_TRY((check_field1<T>(tgrlatda0, *dom, 0, 0, &t0)));
  OEB_TRY((check_field1<T>(tgrlatda1, *dom, 0, 0, &t1)));
  // The four 1-D fields share one stride in the kernel.
  if (a1.s != a0.s || t0.s != a0.s || t1.s != a0.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<T>({&gu, &gv, &gui, &gvi}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi}, {gui.lo, gui.hi, gvi.lo, gvi.hi, a0.lo, a0.hi, a1.lo, a1.hi,
                                                        t0.lo, t0.hi, t1.lo, t1.hi}));
  OEB_RETURN_IF_VALIDATING();
  const int kb = tuned_kb(kKB);
  auto go = [&](auto body, int shape) {
    using B = decltype(body);
    constexpr int S = B::kShape;
    (void)shape;
    return launch<B>(tile_grid((int)dom->nx, (int)dom->ny, (int)dom->nz, TileOf<S>::I, TileOf<S>::J, kb), 0,
                     (cudaStream_t)stream, gu.origin, gv.origin, gui.origin, gvi.origin, a0.origin, a1.origin,
                     t0.origin, t1.origin, a0.s, eddlat, eddlon, make_dims(*dom, gu), kb, alpha, update);
  };
  switch (tuned_shape()) {
    case 1: return go(hadv_kernel<T, ORDER, 1>{}, 1);
    case 2: return go(hadv_kernel<T, ORDER, 2>{}, 2);
    default: return go(hadv_kernel<T, ORDER, 0>{}, 0);
  }
}

// Tangent-linear hadvuv / hadvuv5th: d(uout, vout) = J(uin, vin) d(uin, vin), on Dual<T>.
template <class T, int ORDER, class M3, class M1>
oeb_status hadv_tl_entry(const M3* duout, const M3* dvout, const M3* uin, const M3* vin, const M1* acrlat0,
                         const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, const M3* duin, const M3* dvin,
                         T eddlat, T eddlon, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY((hadv_entry<T, ORDER>(duout, dvout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom,
                                  stream)));
    OEB_TRY((hadv_entry<T, ORDER>(duout, dvout, duin, dvin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon,
                                  dom, stream)));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *u, *v, *a0, *a1, *t0, *t1, *ou, *ov;
  OEB_TRY(arr.pack(uin, duin, &u));
  OEB_TRY(arr.pack(vin, dvin, &v));
  OEB_TRY(arr.pack(acrlat0, (const M1*)nullptr, &a0));
  OEB_TRY(arr.pack(acrlat1, (const M1*)nullptr, &a1));
  OEB_TRY(arr.pack(tgrlatda0, (const M1*)nullptr, &t0));
  OEB_TRY(arr.pack(tgrlatda1, (const M1*)nullptr, &t1));
  OEB_TRY(arr.alloc(duout, &ou));
  OEB_TRY(arr.alloc(dvout, &ov));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, uin->strides[1], uin->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY((launch<hadv_kernel<D, ORDER>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, ou, ov, u, v, a0, a1, t0, t1,
                                         acrlat0->strides[0], D(eddlat), D(eddlon), d, kb, D(0), 0)));
  OEB_TRY(arr.unpack(duout->aligned + duout->offset, ou, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dvout->aligned + dvout->offset, ov, *dom, kInterior, d.sj, d.sk);
}

// ============================== hadvuv / hadvuv5th adjoint ==========================
// With Ax = acrlat0 ua, Ay = R^-1 va, Bx = acrlat1 ub, By = R^-1 vb (the u/v averages of
// hadvuv.h:186-201) and the signed upwind sums Px, Py (of u) and Qx, Qy (of v) -- r = A P --
//   uout = eddlat Ax Px + eddlon Ay Py + tgr0 u va
//   vout = eddlat Bx Qx + eddlon By Qy - tgr1 ub^2
// the transpose for ybar = (uoutb, voutb), branches frozen, is a gather of per-point terms:
//   ax = eddlat Ax uoutb          -> ubar(i+m)  with the x upwind weights of point i
//   ay = eddlon Ay uoutb          -> ubar(j+m)  with the y upwind weights
//   bx = eddlat Px acrlat0 uoutb/3 -> ubar(i-1), ubar(i), ubar(i+1)
//   by = (eddlon Py R^-1 + tgr0 u) uoutb/4 -> vbar at the 4 points of va
//   dd = tgr0 va uoutb            -> ubar(i)
//   gx = eddlat Bx voutb, gy = eddlon By voutb -> vbar along the v upwind stencils
//   ex = (eddlat Qx acrlat1 - 2 tgr1 ub) voutb/4 -> ubar at the 4 points of ub
//   ey = eddlon Qy R^-1 voutb/3   -> vbar(j-1), vbar(j), vbar(j+1)
// Pass 1 writes the nine terms and the four branch flags of every interior point to
// scratch; pass 2 makes each input cell gather the terms of the points that read it.

template <class T>
struct HadvTerms {
  T *ax, *ay, *bx, *by, *dd, *gx, *gy, *ex, *ey;
  unsigned char* fl;  // bit 0: Ax > 0, 1: Ay > 0, 2: Bx > 0, 3: By > 0
};

// Upwind weights of the advection drivers as the weight of field(i + m) in the signed sum
// (branch B carries the leading minus of hadvuv.h:14 / hadvuv5th.h:17).
template <class T, int ORDER>
__device__ __forceinline__ T upwind_weight(bool pos, int m) {
  if (ORDER == 3) {
    constexpr T c6 = T(-1.0) / T(6.0), c3 = T(-1.0) / T(3.0), ch = T(-0.5);
    if (pos) return m == -2 ? c6 : m == -1 ? T(1) : m == 0 ? ch : m == 1 ? c3 : T(0);
    return m == -1 ? -c3 : m == 0 ? -ch : m == 1 ? T(-1) : m == 2 ? -c6 : T(0);
  } else {
    constexpr T c30 = T(1.0) / T(30.0), c4 = T(-1.0) / T(4.0), c3 = T(-1.0) / T(3.0), c2 = T(-1.0) / T(2.0),
                c20 = T(1.0) / T(20.0);
    if (pos)
      return m == -3 ? c30 : m == -2 ? c4 : m == -1 ? T(1) : m == 0 ? c3 : m == 1 ? c2 : m == 2 ? c20 : T(0);
    return m == -2 ? -c20 : m == -1 ? -c2 : m == 0 ? -c3 : m == 1 ? T(-1) : m == 2 ? -c4 : m == 3 ? -c30 : T(0);
  }
}

// signed upwind sum: r = a * adv_sum(...)
template <class T, int ORDER>
__device__ __forceinline__ T adv_sum(const T* __restrict__ f, int64_t o, int64_t s, bool pos) {
  constexpr int lo = ORDER == 3 ? -2 : -3;
  T acc = T(0);
#pragma unroll
  for (int m = lo; m <= -lo; ++m) {
    const T w = upwind_weight<T, ORDER>(pos, m);
    if (w != T(0)) acc = fma(w, ld(f + o + m * s), acc);  // adjoint coefficients: one rounding
  }
  return acc;
}

template <class T, int ORDER, int SHAPE = 0>
struct hadv_adj_terms_kernel {
  static constexpr int kStepOp = step_op<T>(ORDER == 5 ? kOpHadv5AdjTerms + SHAPE : -1);  // the step kernel's id
  // Three CTAs per SM: FP64 80 registers instead of 94 (the hadvuv5th adjoint 4 % faster; the
  // same bound on the hdiffsmag and fastwavesuv adjoints was slower), FP32 80 instead of 128
  // (the FP32 hadvuv5th adjoint 0.268 -> 0.229 ms at 256 x 256 x 80, hadvuv 0.258 -> 0.248)
  static constexpr int kMinCtas = 3;
  static constexpr int kShape = SHAPE;
  static __device__ __forceinline__ void run(const uint3& blk, HadvTerms<T> tm, const T* __restrict__ uin,
                                             const T* __restrict__ vin, const T* __restrict__ acrlat0,
                                             const T* __restrict__ acrlat1, const T* __restrict__ tgrlatda0,
                                             const T* __restrict__ tgrlatda1, int64_t s1d,
                                             const T* __restrict__ uoutb, const T* __restrict__ voutb, T eddlat,
                                             T eddlon, Dims d, int kb) {
    const int64_t sj = d.sj;
    constexpr T third = T(1.0) / T(3.0);
    constexpr T rr = earth_radius_recip<T>();
    for_points_tile<TileOf<SHAPE>::I, TileOf<SHAPE>::J, RowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int j) {
      const int64_t jo = (int64_t)j * s1d;
      const T u0 = ld(uin + o), v0 = ld(vin + o);
      const T um = ld(uin + o - 1) + u0;
      const T ua = third * (um + ld(uin + o + 1));
      const T va = T(0.25) * (((ld(vin + o + 1) + ld(vin + o + 1 - sj)) + v0) + ld(vin + o - sj));
      const T ub = T(0.25) * ((um + ld(uin + o + sj)) + ld(uin + o - 1 + sj));
      const T vb = third * ((ld(vin + o - sj) + v0) + ld(vin + o + sj));
      const T a0 = ld(acrlat0 + jo), a1 = ld(acrlat1 + jo), t0 = ld(tgrlatda0 + jo), t1 = ld(tgrlatda1 + jo);
      const T Ax = a0 * ua, Ay = rr * va, Bx = a1 * ub, By = rr * vb;
      const bool px = Ax > 0, py = Ay > 0, qx = Bx > 0, qy = By > 0;
      const T Px = adv_sum<T, ORDER>(uin, o, 1, px), Py = adv_sum<T, ORDER>(uin, o, sj, py);
      const T Qx = adv_sum<T, ORDER>(vin, o, 1, qx), Qy = adv_sum<T, ORDER>(vin, o, sj, qy);
      const T yu = ld(uoutb + o), yv = ld(voutb + o);
      tm.ax[o] = (eddlat * Ax) * yu;
      tm.ay[o] = (eddlon * Ay) * yu;
      tm.bx[o] = ((eddlat * Px) * a0) * (third * yu);
      tm.by[o] = ((eddlon * Py) * rr + t0 * u0) * (T(0.25) * yu);
      tm.dd[o] = (t0 * va) * yu;
      tm.gx[o] = (eddlat * Bx) * yv;
      tm.gy[o] = (eddlon * By) * yv;
      tm.ex[o] = ((eddlat * Qx) * a1 - (T(2) * t1) * ub) * (T(0.25) * yv);
      tm.ey[o] = ((eddlon * Qy) * rr) * (third * yv);
      tm.fl[o] = (unsigned char)((px ? 1 : 0) | (py ? 2 : 0) | (qx ? 4 : 0) | (qy ? 8 : 0));
    });
  }
};

// Visits every cell of the box [-h, nx+h) x [-h, ny+h) x [0, nz) owned by this thread.
template <class F>
__device__ __forceinline__ void for_box_points(const uint3& blk, const Dims& d, int h, int kb, F&& f) {
  const int i = -h + (int)(blk.x * kTI + threadIdx.x);
  if (i >= d.nx + h) return;
  const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  const int sj = (int)d.sj;
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const int64_t kofs = (int64_t)k * d.sk;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      const int j = -h + (int)(blk.y * kTJ + threadIdx.y) + kTY * r;
      if (j < d.ny + h) f(kofs + i + j * sj, i, j);
    }
  }
}

// update != 0 fuses the transpose of the chained step's update: the outputs are alpha * (the
// gathered gradient), plus the seeds (yu, yv) inside the interior -- the same two roundings as
// the gradient stored and then combined by a separate kernel.
template <class T, int ORDER>
struct hadv_adj_gather_kernel {
  static constexpr int kStepOp = step_op<T>(ORDER == 5 ? kOpHadv5AdjGather : -1);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uinb, T* __restrict__ vinb,
                                             HadvTerms<T> tm, Dims d, int kb, const T* __restrict__ yu,
                                             const T* __restrict__ yv, T alpha, int update) {
    constexpr int h = ORDER == 3 ? 2 : 3;
    const int64_t sj = d.sj;
    for_box_points(blk, d, h, kb, [&](int64_t o, int a, int b) {
      auto in = [&](int i, int j) { return i >= 0 && i < d.nx && j >= 0 && j < d.ny; };
      T ub = T(0), vb = T(0);
      // upwind stencils: point (a - m, b) reads (a, b) with offset m, and likewise in j
  #pragma unroll
      for (int m = -h; m <= h; ++m) {
        if (in(a - m, b)) {
          const int64_t q = o - m;
          const unsigned char f = tm.fl[q];
          ub = fma(upwind_weight<T, ORDER>(f & 1, m), tm.ax[q], ub);
          vb = fma(upwind_weight<T, ORDER>(f & 4, m), tm.gx[q], vb);
        }
        if (in(a, b - m)) {
          const int64_t q = o - m * sj;
          const unsigned char f = tm.fl[q];
          ub = fma(upwind_weight<T, ORDER>(f & 2, m), tm.ay[q], ub);
          vb = fma(upwind_weight<T, ORDER>(f & 8, m), tm.gy[q], vb);
        }
      }
      // u average of point i (i-1, i, i+1) and the ub average (i-1..i, j..j+1)
      if (in(a - 1, b)) ub = ub + tm.bx[o - 1];
      if (in(a, b)) ub = (ub + tm.bx[o]) + (tm.dd[o] + tm.ex[o]);
      if (in(a + 1, b)) ub = (ub + tm.bx[o + 1]) + tm.ex[o + 1];
      if (in(a, b - 1)) ub = ub + tm.ex[o - sj];
      if (in(a + 1, b - 1)) ub = ub + tm.ex[o + 1 - sj];
      // v average va of point (i, j): (i+1, j), (i+1, j-1), (i, j), (i, j-1); vb: (i, j-1..j+1)
      if (in(a - 1, b)) vb = vb + tm.by[o - 1];
      if (in(a - 1, b + 1)) vb = vb + tm.by[o - 1 + sj];
      if (in(a, b)) vb = (vb + tm.by[o]) + tm.ey[o];
      if (in(a, b + 1)) vb = (vb + tm.by[o + sj]) + tm.ey[o + sj];
      if (in(a, b - 1)) vb = vb + tm.ey[o - sj];
      if (update) {
        const T au = alpha * ub, av = alpha * vb;
        const bool inside = in(a, b);
        uinb[o] = inside ? au + yu[o] : au;
        vinb[o] = inside ? av + yv[o] : av;
      } else {
        uinb[o] = ub;
        vinb[o] = vb;
      }
    });
  }
};

// ---- FP32 hadvuv / hadvuv5th adjoint in one tiled launch ----------------------------
// A CTA owns a 32 x 32 tile of the gradient box [-h, n+h)^2 and a chunk of k-levels.  At each
// level it forms, in shared memory, the terms and flags of every interior point its cells
// gather from -- the tile widened by h on each side -- with the terms pass's expressions
// (hadv_adj_terms_kernel), then each cell gathers them as hadv_adj_gather_kernel does: the
// same operations on the same operands in the same order, so the same bits.  The apron
// recomputes (32 + 2h)^2 / 32^2 - 1 = 41 % more terms (h = 3), and the 37 bytes a point of
// term scratch are neither written nor read back.
template <int ORDER>
struct HadvAdjF32Smem {
  static constexpr int kH = ORDER == 3 ? 2 : 3;
  static constexpr int kAW = 32 + 2 * kH;  // term region edge
  float t[9][kAW][kAW];                     // ax ay bx by dd gx gy ex ey
  unsigned char fl[kAW][kAW];
};

template <int ORDER>
struct hadv_adj_f32 {
  static constexpr int kStepOp = step_op<float>(ORDER == 5 ? kOpHadv5AdjTiled : -1);  // the step kernel's id
  static constexpr int kMinCtas = 3;
  using Smem = HadvAdjF32Smem<ORDER>;
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uinb, float* __restrict__ vinb,
                                             const float* __restrict__ uin, const float* __restrict__ vin,
                                             const float* __restrict__ acrlat0, const float* __restrict__ acrlat1,
                                             const float* __restrict__ tgrlatda0, const float* __restrict__ tgrlatda1,
                                             int64_t s1d, const float* __restrict__ uoutb,
                                             const float* __restrict__ voutb, float eddlat, float eddlon, Dims d,
                                             int kb, float alpha, int update) {
    using T = float;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    constexpr int h = Smem::kH, W = Smem::kAW;
    enum { AX, AY, BX, BY, DD, GX, GY, EX, EY };
    const int64_t sj = d.sj;
    constexpr T third = T(1.0) / T(3.0);
    constexpr T rr = earth_radius_recip<T>();
    const int ci0 = -h + (int)blk.x * 32, cj0 = -h + (int)blk.y * 32;  // the tile's first cell
    const int pi0 = ci0 - h, pj0 = cj0 - h;                            // its term region's first point
    const int k0 = (int)blk.z * kb, k1 = min(k0 + kb, d.nz);
    const int tid = threadIdx.y * kTX + threadIdx.x;
    auto in = [&](int i, int j) { return i >= 0 && i < d.nx && j >= 0 && j < d.ny; };
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      // the terms (hadv_adj_terms_kernel) of the interior points of the region
      for (int e = tid; e < W * W; e += kThreads) {
        const int li = e % W, lj = e / W;
        const int i = pi0 + li, j = pj0 + lj;
        if (!in(i, j)) continue;
        const int64_t o = kofs + i + (int64_t)j * sj;
        const int64_t jo = (int64_t)j * s1d;
        const T u0 = ld(uin + o), v0 = ld(vin + o);
        const T um = ld(uin + o - 1) + u0;
        const T ua = third * (um + ld(uin + o + 1));
        const T va = T(0.25) * (((ld(vin + o + 1) + ld(vin + o + 1 - sj)) + v0) + ld(vin + o - sj));
        const T ub = T(0.25) * ((um + ld(uin + o + sj)) + ld(uin + o - 1 + sj));
        const T vb = third * ((ld(vin + o - sj) + v0) + ld(vin + o + sj));
        const T a0 = ld(acrlat0 + jo), a1 = ld(acrlat1 + jo), t0 = ld(tgrlatda0 + jo), t1 = ld(tgrlatda1 + jo);
        const T Ax = a0 * ua, Ay = rr * va, Bx = a1 * ub, By = rr * vb;
        const bool px = Ax > 0, py = Ay > 0, qx = Bx > 0, qy = By > 0;
        const T Px = adv_sum<T, ORDER>(uin, o, 1, px), Py = adv_sum<T, ORDER>(uin, o, sj, py);
        const T Qx = adv_sum<T, ORDER>(vin, o, 1, qx), Qy = adv_sum<T, ORDER>(vin, o, sj, qy);
        const T yu = ld(uoutb + o), yv = ld(voutb + o);
        s.t[AX][lj][li] = (eddlat * Ax) * yu;
        s.t[AY][lj][li] = (eddlon * Ay) * yu;
        s.t[BX][lj][li] = ((eddlat * Px) * a0) * (third * yu);
        s.t[BY][lj][li] = ((eddlon * Py) * rr + t0 * u0) * (T(0.25) * yu);
        s.t[DD][lj][li] = (t0 * va) * yu;
        s.t[GX][lj][li] = (eddlat * Bx) * yv;
        s.t[GY][lj][li] = (eddlon * By) * yv;
        s.t[EX][lj][li] = ((eddlat * Qx) * a1 - (T(2) * t1) * ub) * (T(0.25) * yv);
        s.t[EY][lj][li] = ((eddlon * Qy) * rr) * (third * yv);
        s.fl[lj][li] = (unsigned char)((px ? 1 : 0) | (py ? 2 : 0) | (qx ? 4 : 0) | (qy ? 8 : 0));
      }
      __syncthreads();
      // the gather (hadv_adj_gather_kernel) of the tile's cells, four rows a thread
#pragma unroll 1
      for (int r = 0; r < 4; ++r) {
        const int a = ci0 + (int)threadIdx.x, b = cj0 + (int)threadIdx.y + 8 * r;
        if (a >= d.nx + h || b >= d.ny + h) continue;
        const int li = a - pi0, lj = b - pj0;
        auto tm = [&](int q, int di, int dj) { return s.t[q][lj + dj][li + di]; };
        T ub = T(0), vb = T(0);
#pragma unroll
        for (int m = -h; m <= h; ++m) {
          if (in(a - m, b)) {
            const unsigned char f = s.fl[lj][li - m];
            ub = fma(upwind_weight<T, ORDER>(f & 1, m), tm(AX, -m, 0), ub);
            vb = fma(upwind_weight<T, ORDER>(f & 4, m), tm(GX, -m, 0), vb);
          }
          if (in(a, b - m)) {
            const unsigned char f = s.fl[lj - m][li];
            ub = fma(upwind_weight<T, ORDER>(f & 2, m), tm(AY, 0, -m), ub);
            vb = fma(upwind_weight<T, ORDER>(f & 8, m), tm(GY, 0, -m), vb);
          }
        }
        if (in(a - 1, b)) ub = ub + tm(BX, -1, 0);
        if (in(a, b)) ub = (ub + tm(BX, 0, 0)) + (tm(DD, 0, 0) + tm(EX, 0, 0));
        if (in(a + 1, b)) ub = (ub + tm(BX, 1, 0)) + tm(EX, 1, 0);
        if (in(a, b - 1)) ub = ub + tm(EX, 0, -1);
        if (in(a + 1, b - 1)) ub = ub + tm(EX, 1, -1);
        if (in(a - 1, b)) vb = vb + tm(BY, -1, 0);
        if (in(a - 1, b + 1)) vb = vb + tm(BY, -1, 1);
        if (in(a, b)) vb = (vb + tm(BY, 0, 0)) + tm(EY, 0, 0);
        if (in(a, b + 1)) vb = (vb + tm(BY, 0, 1)) + tm(EY, 0, 1);
        if (in(a, b - 1)) vb = vb + tm(EY, 0, -1);
        const int64_t o = kofs + a + (int64_t)b * sj;
        if (update) {
          const T au = alpha * ub, av = alpha * vb;
          const bool inside = in(a, b);
          uinb[o] = inside ? au + uoutb[o] : au;
          vinb[o] = inside ? av + voutb[o] : av;
        } else {
          uinb[o] = ub;
          vinb[o] = vb;
        }
      }
      __syncthreads();  // the next level's terms replace these
    }
  }
};

template <class T, int ORDER, class M3, class M1>
oeb_status hadv_adj_entry(const M3* uinb, const M3* vinb, const M3* uin, const M3* vin, const M1* acrlat0,
                          const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, const M3* uoutb,
                          const M3* voutb, T eddlat, T eddlon, const oeb_domain* dom, void* stream,
                          T alpha = T(0), int update = 0) {
  {
    ValidateOnly guard;
    OEB_TRY((hadv_entry<T, ORDER>(uoutb, voutb, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon,
                                  dom, stream)));
  }
  const int h = ORDER == 3 ? 2 : 3;
  Grid<T> gub, gvb, gui, gvi, guo, gvo;
  OEB_TRY((check_field3<T>(uinb, *dom, Reach{h, h, h, h, 0, 0}, &gub)));
  OEB_TRY((check_field3<T>(vinb, *dom, Reach{h, h, h, h, 0, 0}, &gvb)));
  OEB_TRY((check_field3<T>(uin, *dom, Reach{h, h, h, h, 0, 0}, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, Reach{h, h, h, h, 0, 0}, &gvi)));
  OEB_TRY((check_field3<T>(uoutb, *dom, kInterior, &guo)));
  OEB_TRY((check_field3<T>(voutb, *dom, kInterior, &gvo)));
  OEB_TRY(check_same_strides<T>({&gub, &gvb, &gui, &gvi, &guo, &gvo}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi},
                         {gui.lo, gui.hi, gvi.lo, gvi.hi, guo.lo, guo.hi, gvo.lo, gvo.hi}));
  OEB_RETURN_IF_VALIDATING();
  cudaStream_t st = (cudaStream_t)stream;
  if constexpr (std::is_same<T, float>::value) {
    if (adjoint_tiles()) {  // one tiled launch, no scratch
      const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
      const int kb = tuned_kb(kKB);
      return launch<hadv_adj_f32<ORDER>>(
          tile_grid(d.nx + 2 * h, d.ny + 2 * h, d.nz, kTI, kTJ, kb), sizeof(HadvAdjF32Smem<ORDER>), st, gub.origin,
          gvb.origin, gui.origin, gvi.origin, (const T*)acrlat0->aligned + acrlat0->offset,
          (const T*)acrlat1->aligned + acrlat1->offset, (const T*)tgrlatda0->aligned + tgrlatda0->offset,
          (const T*)tgrlatda1->aligned + tgrlatda1->offset, acrlat0->strides[0], guo.origin, gvo.origin, eddlat, eddlon,
          d, kb, alpha, update);
    }
  }
  // scratch: nine term fields and the flags, in uin's layout (terms are read at interior points only)
  const T* start = (uin->allocated && uin->allocated <= uin->aligned) ? uin->allocated : uin->aligned;
  const int64_t last = (uin->sizes[0] - 1) * uin->strides[0] + (uin->sizes[1] - 1) * uin->strides[1] +
                       (uin->sizes[2] - 1) * uin->strides[2];
  const int64_t n = (int64_t)(uin->aligned - start) + last + 1;
  const int64_t org = (int64_t)(uin->aligned - start) + uin->offset;
  void* buf = nullptr;
  OEB_TRY(scratch_alloc(&buf, (size_t)n * (9 * sizeof(T) + 1), st));
  HadvTerms<T> tm;
  T* base = static_cast<T*>(buf);
  T** fields[9] = {&tm.ax, &tm.ay, &tm.bx, &tm.by, &tm.dd, &tm.gx, &tm.gy, &tm.ex, &tm.ey};
  for (int q = 0; q < 9; ++q) *fields[q] = base + q * n + org;
  tm.fl = reinterpret_cast<unsigned char*>(base + 9 * n) + org;
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
  const int kb = tuned_kb(kKB);
  auto terms = [&](auto body) {
    using B = decltype(body);
    constexpr int S = B::kShape;
    return launch<B>(tile_grid(d.nx, d.ny, d.nz, TileOf<S>::I, TileOf<S>::J, kb), 0, st, tm, gui.origin, gvi.origin,
                     (const T*)acrlat0->aligned + acrlat0->offset, (const T*)acrlat1->aligned + acrlat1->offset,
                     (const T*)tgrlatda0->aligned + tgrlatda0->offset, (const T*)tgrlatda1->aligned + tgrlatda1->offset,
                     acrlat0->strides[0], guo.origin, gvo.origin, eddlat, eddlon, d, kb);
  };
  oeb_status stt;
  switch (tuned_shape()) {
    case 1: stt = terms(hadv_adj_terms_kernel<T, ORDER, 1>{}); break;
    case 2: stt = terms(hadv_adj_terms_kernel<T, ORDER, 2>{}); break;
    default: stt = terms(hadv_adj_terms_kernel<T, ORDER, 0>{}); break;
  }
  if (stt == OEB_OK)
    stt = launch<hadv_adj_gather_kernel<T, ORDER>>(tile_grid(d.nx + 2 * h, d.ny + 2 * h, d.nz, kTI, kTJ, kb), 0, st,
                                                   gub.origin, gvb.origin, tm, d, kb, update ? guo.origin : nullptr,
                                                   update ? gvo.origin : nullptr, alpha, update);
  scratch_free(buf, st);
  return stt;
}


// ============================== shared pieces of the adjoints below ==================
// Scratch term fields of an adjoint, each laid out like `like` (the terms are written and read
// at interior points only): cells per field and the offset of the interior origin.
struct TermLayout {
  int64_t n, org;
};
template <class M3>
TermLayout term_layout(const M3* like) {
  const auto* start = (like->allocated && like->allocated <= like->aligned) ? like->allocated : like->aligned;
  const int64_t last = (like->sizes[0] - 1) * like->strides[0] + (like->sizes[1] - 1) * like->strides[1] +
                       (like->sizes[2] - 1) * like->strides[2];
  return TermLayout{(int64_t)(like->aligned - start) + last + 1, (int64_t)(like->aligned - start) + like->offset};
}

__device__ __forceinline__ bool inside(const Dims& d, int i, int j, int k) {
  return i >= 0 && i < d.nx && j >= 0 && j < d.ny && k >= 0 && k < d.nz;
}

// ============================== laplace: tangent-linear and adjoint ==================
// laplace.h:39 is linear: out = -4 in + (in(i-1) + in(i+1)) + (in(j+1) + in(j-1)).  Its
// transpose for outb gathers, at every cell c of in's reach box [-1, N+1)^2 x [0, Nz):
//   inb(c) = -4 outb(c) + outb(c-i) + outb(c+i) + outb(c-j) + outb(c+j)   (interior terms only)
template <class T>
struct laplace_adj_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ inb, const T* __restrict__ outb,
                                             Dims d, int kb) {
    const int64_t sj = d.sj;
    for_box_k<RowUnroll<T>::value>(blk, d.sj, d.sk, -1, -1, d.nx + 2, d.ny + 2, d.nz, kb,
                                   [&](int64_t o, int i, int j, int k) {
      T v = inside(d, i, j, k) ? T(-4.0) * ld(outb + o) : T(0);
      if (inside(d, i - 1, j, k)) v = v + ld(outb + o - 1);
      if (inside(d, i + 1, j, k)) v = v + ld(outb + o + 1);
      if (inside(d, i, j - 1, k)) v = v + ld(outb + o - sj);
      if (inside(d, i, j + 1, k)) v = v + ld(outb + o + sj);
      inb[o] = v;
    });
  }
};

template <class T, class M3>
oeb_status laplace_tl_entry(const M3* dout, const M3* in, const M3* din, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(laplace_entry<T>(in, dout, dom, stream));
    OEB_TRY(laplace_entry<T>(din, dout, dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *x, *y;
  OEB_TRY(arr.pack(in, din, &x));
  OEB_TRY(arr.alloc(dout, &y));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, in->strides[1], in->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<laplace_kernel<D>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, x, y, d, kb));
  return arr.unpack(dout->aligned + dout->offset, y, *dom, kInterior, d.sj, d.sk);
}

template <class T, class M3>
oeb_status laplace_adj_entry(const M3* inb, const M3* in, const M3* outb, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(laplace_entry<T>(in, outb, dom, stream));
  }
  Grid<T> gib, gin, gob;
  OEB_TRY((check_field3<T>(inb, *dom, Reach{1, 1, 1, 1, 0, 0}, &gib)));
  OEB_TRY((check_field3<T>(in, *dom, Reach{1, 1, 1, 1, 0, 0}, &gin)));
  OEB_TRY((check_field3<T>(outb, *dom, kInterior, &gob)));
  OEB_TRY(check_same_strides<T>({&gib, &gin, &gob}));
  OEB_TRY(check_no_alias({gib.lo, gib.hi}, {gin.lo, gin.hi, gob.lo, gob.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gob.sj, gob.sk};
  const int kb = tuned_kb(kKB);
  return launch<laplace_adj_kernel<T>>(tile_grid(d.nx + 2, d.ny + 2, d.nz, kTI, kTJ, kb), 0, (cudaStream_t)stream,
                                       gib.origin, gob.origin, d, kb);
}

// ============================== uvbke: tangent-linear and adjoint =====================
// uvbke.h:66-71 is linear in (uc, vc) with su = uc(j-1) + uc and sv = vc(i-1) + vc:
//   ub = dt5 (su - sv cosa) rsina,  vb = dt5 (sv - su cosa) rsina.
// Its transpose for (ubb, vbb): at each interior point
//   sub = dt5 rsina (ubb - cosa vbb),  svb = dt5 rsina (vbb - cosa ubb),
// and each cell gathers ucb(c) = sub(c) + sub(c+j) (on [0,N) x [-1,N)) and
// vcb(c) = svb(c) + svb(c+i) (on [-1,N) x [0,N)), interior points only.
template <class T>
__device__ __forceinline__ T uvbke_sub(const T* ubb, const T* vbb, const T* cosa, const T* rsina, int64_t o, T dt5) {
  return (dt5 * ld(rsina + o)) * (ld(ubb + o) - ld(cosa + o) * ld(vbb + o));
}
template <class T>
__device__ __forceinline__ T uvbke_svb(const T* ubb, const T* vbb, const T* cosa, const T* rsina, int64_t o, T dt5) {
  return (dt5 * ld(rsina + o)) * (ld(vbb + o) - ld(cosa + o) * ld(ubb + o));
}

template <class T>
struct uvbke_adj_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ ucb, T* __restrict__ vcb,
                                             const T* __restrict__ cosa, const T* __restrict__ rsina,
                                             const T* __restrict__ ubb, const T* __restrict__ vbb, T dt5, Dims d,
                                             int kb) {
    const int64_t sj = d.sj;
    for_box_k<RowUnroll<T>::value>(blk, d.sj, d.sk, -1, -1, d.nx + 1, d.ny + 1, d.nz, kb,
                                   [&](int64_t o, int i, int j, int k) {
      const bool here = inside(d, i, j, k);
      const T su = here ? uvbke_sub(ubb, vbb, cosa, rsina, o, dt5) : T(0);
      const T sv = here ? uvbke_svb(ubb, vbb, cosa, rsina, o, dt5) : T(0);
      if (i >= 0) ucb[o] = inside(d, i, j + 1, k) ? su + uvbke_sub(ubb, vbb, cosa, rsina, o + sj, dt5) : su;
      if (j >= 0) vcb[o] = inside(d, i + 1, j, k) ? sv + uvbke_svb(ubb, vbb, cosa, rsina, o + 1, dt5) : sv;
    });
  }
};

template <class T, class M3>
oeb_status uvbke_tl_entry(const M3* dub, const M3* dvb, const M3* uc, const M3* vc, const M3* cosa, const M3* rsina,
                          const M3* duc, const M3* dvc, double dt5, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(uvbke_entry<T>(dub, dvb, uc, vc, cosa, rsina, dt5, dom, stream));
    OEB_TRY(uvbke_entry<T>(dub, dvb, duc, dvc, cosa, rsina, dt5, dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *u, *v, *ca, *rs, *ou, *ov;
  OEB_TRY(arr.pack(uc, duc, &u));
  OEB_TRY(arr.pack(vc, dvc, &v));
  OEB_TRY(arr.pack(cosa, (const M3*)nullptr, &ca));
  OEB_TRY(arr.pack(rsina, (const M3*)nullptr, &rs));
  OEB_TRY(arr.alloc(dub, &ou));
  OEB_TRY(arr.alloc(dvb, &ov));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, uc->strides[1], uc->strides[0]};
  const T dt5_hi = T(dt5), dt5_lo = T(dt5 - (double)dt5_hi);
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<uvbke_kernel<D>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, ou, ov, u, v, ca, rs, D(dt5_hi),
                                  D(dt5_lo), d, kb));
  OEB_TRY(arr.unpack(dub->aligned + dub->offset, ou, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dvb->aligned + dvb->offset, ov, *dom, kInterior, d.sj, d.sk);
}

template <class T, class M3>
oeb_status uvbke_adj_entry(const M3* ucb, const M3* vcb, const M3* uc, const M3* vc, const M3* cosa, const M3* rsina,
                           const M3* ubb, const M3* vbb, double dt5, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(uvbke_entry<T>(ubb, vbb, uc, vc, cosa, rsina, dt5, dom, stream));
  }
  Grid<T> gucb, gvcb, gca, grs, gub, gvb;
  OEB_TRY((check_field3<T>(ucb, *dom, Reach{0, 0, 1, 0, 0, 0}, &gucb)));
  OEB_TRY((check_field3<T>(vcb, *dom, Reach{1, 0, 0, 0, 0, 0}, &gvcb)));
  OEB_TRY((check_field3<T>(cosa, *dom, kInterior, &gca)));
  OEB_TRY((check_field3<T>(rsina, *dom, kInterior, &grs)));
  OEB_TRY((check_field3<T>(ubb, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<T>(vbb, *dom, kInterior, &gvb)));
  OEB_TRY(check_same_strides<T>({&gucb, &gvcb, &gca, &grs, &gub, &gvb}));
  OEB_TRY(check_no_alias({gucb.lo, gucb.hi, gvcb.lo, gvcb.hi},
                         {gca.lo, gca.hi, grs.lo, grs.hi, gub.lo, gub.hi, gvb.lo, gvb.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gub.sj, gub.sk};
  const int kb = tuned_kb(kKB);
  return launch<uvbke_adj_kernel<T>>(tile_grid(d.nx + 1, d.ny + 1, d.nz, kTI, kTJ, kb), 0, (cudaStream_t)stream,
                                     gucb.origin, gvcb.origin, gca.origin, grs.origin, gub.origin, gvb.origin, T(dt5),
                                     d, kb);
}

// ============================== p_grad_c: tangent-linear and adjoint ==================
// p_grad_c.h:90-97 at point p, along the axis of stride s (i for uout, j for vout):
//   out = in + c f,  c = dt2 rd / (delpc(p-s) + delpc(p)),
//   f = A1 B1 + A2 B2,  A1 = gz(p-s,k+1) - gz(p),  B1 = pkc(p,k+1) - pkc(p-s),
//                       A2 = gz(p-s) - gz(p,k+1),  B2 = pkc(p-s,k+1) - pkc(p).
// Active inputs: uin, vin, delpc, gz, pkc (rdxc, rdyc, dt2 are parameters).  The transpose
// for outb, with fb = outb c and sb = -fb f / (delpc(p-s) + delpc(p)):
//   inb += outb;  delpcb(p-s), delpcb(p) += sb;
//   gzb(p-s,k+1) += fb B1, gzb(p) -= fb B1, gzb(p-s) += fb B2, gzb(p,k+1) -= fb B2;
//   pkcb(p,k+1) += fb A1, pkcb(p-s) -= fb A1, pkcb(p-s,k+1) += fb A2, pkcb(p) -= fb A2.
// Pass 1 writes uinb, vinb and the five terms (sb, fb B1, fb B2, fb A1, fb A2) of each axis at
// every interior point; pass 2 makes every cell of the reach boxes gather them.
template <class T>
struct PgcTerms {
  T* t[10];  // per axis (u: 0-4, v: 5-9): sb, fb B1, fb B2, fb A1, fb A2
};

// The five terms of point o along the axis of stride s (both forms of the adjoint use these
// expressions).
template <class T>
__device__ __forceinline__ void pgc_adj_terms(T (&t)[5], const T* __restrict__ gz, const T* __restrict__ pkc,
                                              const T* __restrict__ delpc, int64_t o, int64_t s, int64_t sk, T gz0,
                                              T gz1, T pk0, T pk1, T wk, T coef, T y) {
  const T A1 = ld(gz + o - s + sk) - gz0, B1 = pk1 - ld(pkc + o - s);
  const T A2 = ld(gz + o - s) - gz1, B2 = ld(pkc + o - s + sk) - pk0;
  const T f = A1 * B1 + A2 * B2;
  const T r = T(1) / (ld(delpc + o - s) + wk);
  const T fb = (y * coef) * r;
  t[0] = -(fb * f) * r;
  t[1] = fb * B1;
  t[2] = fb * B2;
  t[3] = fb * A1;
  t[4] = fb * A2;
}

template <class T>
__device__ __forceinline__ void pgc_adj_axis(T* const* t, const T* __restrict__ gz, const T* __restrict__ pkc,
                                             const T* __restrict__ delpc, int64_t o, int64_t s, int64_t sk, T gz0,
                                             T gz1, T pk0, T pk1, T wk, T coef, T y) {
  T v[5];
  pgc_adj_terms(v, gz, pkc, delpc, o, s, sk, gz0, gz1, pk0, pk1, wk, coef, y);
#pragma unroll
  for (int q = 0; q < 5; ++q) t[q][o] = v[q];
}

template <class T>
struct p_grad_c_adj_terms_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, PgcTerms<T> tm, T* __restrict__ uinb,
                                             T* __restrict__ vinb, const T* __restrict__ rdxc,
                                             const T* __restrict__ rdyc, const T* __restrict__ delpc,
                                             const T* __restrict__ gz, const T* __restrict__ pkc,
                                             const T* __restrict__ uoutb, const T* __restrict__ voutb, T dt2, Dims d,
                                             int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    for_points<RowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int) {
      const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pkc + o), pk1 = ld(pkc + o + sk);
      const T wk = ld(delpc + o);
      const T yu = ld(uoutb + o), yv = ld(voutb + o);
      uinb[o] = yu;
      vinb[o] = yv;
      pgc_adj_axis(tm.t, gz, pkc, delpc, o, 1, sk, gz0, gz1, pk0, pk1, wk, dt2 * ld(rdxc + o), yu);
      pgc_adj_axis(tm.t + 5, gz, pkc, delpc, o, sj, sk, gz0, gz1, pk0, pk1, wk, dt2 * ld(rdyc + o), yv);
    });
  }
};

// Every cell c of [-1, N) x [-1, N) x [0, Nz] (delpcb only below Nz) gathers the terms of the
// interior points that read it: along axis s, the points c, c+s, c-k and c+s-k.
template <class T>
struct p_grad_c_adj_gather_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ delpcb, T* __restrict__ gzb,
                                             T* __restrict__ pkcb, PgcTerms<T> tm, Dims d, int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    for_box_k<RowUnroll<T>::value>(blk, sj, sk, -1, -1, d.nx + 1, d.ny + 1, d.nz + 1, kb,
                                   [&](int64_t o, int i, int j, int k) {
      T db = T(0), gb = T(0), pb = T(0);
  #pragma unroll
      for (int ax = 0; ax < 2; ++ax) {
        T* const* t = tm.t + 5 * ax;
        const int di = ax == 0 ? 1 : 0, dj = 1 - di;
        const int64_t s = ax == 0 ? 1 : sj;
        if (inside(d, i, j, k)) {  // p = c
          db = db + t[0][o];
          gb = gb - t[1][o];
          pb = pb - t[4][o];
        }
        if (inside(d, i + di, j + dj, k)) {  // p = c + s
          db = db + t[0][o + s];
          gb = gb + t[2][o + s];
          pb = pb - t[3][o + s];
        }
        if (inside(d, i, j, k - 1)) {  // p = c - k
          gb = gb - t[2][o - sk];
          pb = pb + t[3][o - sk];
        }
        if (inside(d, i + di, j + dj, k - 1)) {  // p = c + s - k
          gb = gb + t[1][o + s - sk];
          pb = pb + t[4][o + s - sk];
        }
      }
      if (k < d.nz) delpcb[o] = db;
      gzb[o] = gb;
      pkcb[o] = pb;
    });
  }
};

// ---- FP32 p_grad_c adjoint in one tiled launch -----------------------------------------
// A CTA owns a 32 x 16 tile of the gather box [-1, N)^2 and a chunk of its levels [0, Nz], and
// marches k.  At each level it forms the terms (pgc_adj_terms, as the terms pass) of the
// interior points its cells read -- for the x axis the tile and one more column, for the y
// axis the tile and one more row -- into a two-level ring in shared memory, and its cells
// gather the terms of levels k and k-1 in the gather pass's order: the same bits as the two
// passes, without the 40 bytes a point of term scratch.  A chunk first forms the level below
// its first one.
constexpr int kPgcTJ = 16;  // rows of a tile
struct PgcAdjF32Smem {
  float tx[2][5][kPgcTJ][33];      // x-axis terms: rows cj0 .., columns ci0 .. ci0 + 32
  float ty[2][5][kPgcTJ + 1][32];  // y-axis terms: rows cj0 .. cj0 + 16, columns ci0 ..
};

struct p_grad_c_adj_f32 {
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uinb, float* __restrict__ vinb,
                                             float* __restrict__ delpcb, float* __restrict__ gzb,
                                             float* __restrict__ pkcb, const float* __restrict__ rdxc,
                                             const float* __restrict__ rdyc, const float* __restrict__ delpc,
                                             const float* __restrict__ gz, const float* __restrict__ pkc,
                                             const float* __restrict__ uoutb, const float* __restrict__ voutb,
                                             float dt2, Dims d, int kb) {
    using T = float;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PgcAdjF32Smem& s = *reinterpret_cast<PgcAdjF32Smem*>(smem_raw);
    const int64_t sj = d.sj, sk = d.sk;
    const int ci0 = -1 + (int)blk.x * 32, cj0 = -1 + (int)blk.y * kPgcTJ;  // the tile's first cell
    const int kz0 = (int)blk.z * kb, kz1 = min(kz0 + kb, d.nz + 1);       // its levels of [0, nz]
    const int tid = threadIdx.y * kTX + threadIdx.x;
    // the terms of level k into ring slot k & 1, and (own = true) uinb, vinb of the points this
    // tile owns
    auto terms = [&](int k, bool own) {
      const int slot = k & 1;
      const int64_t kofs = (int64_t)k * sk;
      for (int e = tid; e < 33 * (kPgcTJ + 1); e += kThreads) {
        const int a = e % 33, b = e / 33;
        const int i = ci0 + a, j = cj0 + b;
        const bool xs = b < kPgcTJ, ys = a < 32;  // in the x-axis / y-axis region
        if (!(xs || ys) || !inside(d, i, j, k)) continue;
        const int64_t o = kofs + i + (int64_t)j * sj;
        const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pkc + o), pk1 = ld(pkc + o + sk);
        const T wk = ld(delpc + o);
        const T yu = ld(uoutb + o), yv = ld(voutb + o);
        if (own && xs && ys) {  // the tile's own cells
          uinb[o] = yu;
          vinb[o] = yv;
        }
        T v[5];
        if (xs) {
          pgc_adj_terms(v, gz, pkc, delpc, o, 1, sk, gz0, gz1, pk0, pk1, wk, dt2 * ld(rdxc + o), yu);
#pragma unroll
          for (int q = 0; q < 5; ++q) s.tx[slot][q][b][a] = v[q];
        }
        if (ys) {
          pgc_adj_terms(v, gz, pkc, delpc, o, sj, sk, gz0, gz1, pk0, pk1, wk, dt2 * ld(rdyc + o), yv);
#pragma unroll
          for (int q = 0; q < 5; ++q) s.ty[slot][q][b][a] = v[q];
        }
      }
    };
    if (kz0 >= 1) terms(kz0 - 1, false);  // the level below the chunk's first (its cells read it)
#pragma unroll 1
    for (int k = kz0; k < kz1; ++k) {
      if (k < d.nz) terms(k, true);
      __syncthreads();
      const int cur = k & 1, prev = (k - 1) & 1;
      const int64_t kofs = (int64_t)k * sk;
#pragma unroll
      for (int r = 0; r < kPgcTJ / kTY; ++r) {
        const int a = threadIdx.x, b = threadIdx.y + kTY * r;
        const int i = ci0 + a, j = cj0 + b;
        if (i >= d.nx || j >= d.ny) continue;  // the gather box is [-1, N)^2
        T db = T(0), gb = T(0), pb = T(0);
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
          const int di = ax == 0 ? 1 : 0, dj = 1 - di;
          // term q of axis ax at the point (i + ei, j + ej) of level slot sl
          auto t = [&](int sl, int q, int ei, int ej) {
            return ax == 0 ? s.tx[sl][q][b + ej][a + ei] : s.ty[sl][q][b + ej][a + ei];
          };
          if (inside(d, i, j, k)) {  // p = c
            db = db + t(cur, 0, 0, 0);
            gb = gb - t(cur, 1, 0, 0);
            pb = pb - t(cur, 4, 0, 0);
          }
          if (inside(d, i + di, j + dj, k)) {  // p = c + s
            db = db + t(cur, 0, di, dj);
            gb = gb + t(cur, 2, di, dj);
            pb = pb - t(cur, 3, di, dj);
          }
          if (inside(d, i, j, k - 1)) {  // p = c - k
            gb = gb - t(prev, 2, 0, 0);
            pb = pb + t(prev, 3, 0, 0);
          }
          if (inside(d, i + di, j + dj, k - 1)) {  // p = c + s - k
            gb = gb + t(prev, 1, di, dj);
            pb = pb + t(prev, 4, di, dj);
          }
        }
        const int64_t o = kofs + i + (int64_t)j * sj;
        if (k < d.nz) delpcb[o] = db;
        gzb[o] = gb;
        pkcb[o] = pb;
      }
      __syncthreads();  // level k + 1's terms replace level k - 1's
    }
  }
};

template <class T, class M3>
oeb_status p_grad_c_tl_entry(const M3* duout, const M3* dvout, const M3* uin, const M3* vin, const M3* rdxc,
                             const M3* rdyc, const M3* delpc, const M3* gz, const M3* pkc, const M3* duin,
                             const M3* dvin, const M3* ddelpc, const M3* dgz, const M3* dpkc, T dt2,
                             const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(p_grad_c_entry<T>(duout, dvout, uin, vin, rdxc, rdyc, delpc, gz, pkc, dt2, dom, stream));
    OEB_TRY(p_grad_c_entry<T>(duout, dvout, duin, dvin, rdxc, rdyc, ddelpc, dgz, dpkc, dt2, dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *u, *v, *rx, *ry, *dp, *g, *pk, *ou, *ov;
  OEB_TRY(arr.pack(uin, duin, &u));
  OEB_TRY(arr.pack(vin, dvin, &v));
  OEB_TRY(arr.pack(rdxc, (const M3*)nullptr, &rx));
  OEB_TRY(arr.pack(rdyc, (const M3*)nullptr, &ry));
  OEB_TRY(arr.pack(delpc, ddelpc, &dp));
  OEB_TRY(arr.pack(gz, dgz, &g));
  OEB_TRY(arr.pack(pkc, dpkc, &pk));
  OEB_TRY(arr.alloc(duout, &ou));
  OEB_TRY(arr.alloc(dvout, &ov));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, uin->strides[1], uin->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<p_grad_c_kernel<D>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, ou, ov, u, v, rx, ry, dp, g, pk,
                                     D(dt2), d, kb));
  OEB_TRY(arr.unpack(duout->aligned + duout->offset, ou, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dvout->aligned + dvout->offset, ov, *dom, kInterior, d.sj, d.sk);
}

template <class T, class M3>
oeb_status p_grad_c_adj_entry(const M3* uinb, const M3* vinb, const M3* delpcb, const M3* gzb, const M3* pkcb,
                              const M3* uin, const M3* vin, const M3* rdxc, const M3* rdyc, const M3* delpc,
                              const M3* gz, const M3* pkc, const M3* uoutb, const M3* voutb, T dt2,
                              const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(p_grad_c_entry<T>(uoutb, voutb, uin, vin, rdxc, rdyc, delpc, gz, pkc, dt2, dom, stream));
  }
  Grid<T> gub, gvb, gdb, ggb, gpb, grx, gry, gdp, ggz, gpk, guo, gvo;
  const Reach rk{1, 0, 1, 0, 0, 1};
  OEB_TRY((check_field3<T>(uinb, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<T>(vinb, *dom, kInterior, &gvb)));
  OEB_TRY((check_field3<T>(delpcb, *dom, Reach{1, 0, 1, 0, 0, 0}, &gdb)));
  OEB_TRY((check_field3<T>(gzb, *dom, rk, &ggb)));
  OEB_TRY((check_field3<T>(pkcb, *dom, rk, &gpb)));
  OEB_TRY((check_field3<T>(rdxc, *dom, kInterior, &grx)));
  OEB_TRY((check_field3<T>(rdyc, *dom, kInterior, &gry)));
  OEB_TRY((check_field3<T>(delpc, *dom, Reach{1, 0, 1, 0, 0, 0}, &gdp)));
  OEB_TRY((check_field3<T>(gz, *dom, rk, &ggz)));
  OEB_TRY((check_field3<T>(pkc, *dom, rk, &gpk)));
  OEB_TRY((check_field3<T>(uoutb, *dom, kInterior, &guo)));
  OEB_TRY((check_field3<T>(voutb, *dom, kInterior, &gvo)));
  OEB_TRY(check_same_strides<T>({&gub, &gvb, &gdb, &ggb, &gpb, &grx, &gry, &gdp, &ggz, &gpk, &guo, &gvo}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi, gdb.lo, gdb.hi, ggb.lo, ggb.hi, gpb.lo, gpb.hi},
                         {grx.lo, grx.hi, gry.lo, gry.hi, gdp.lo, gdp.hi, ggz.lo, ggz.hi, gpk.lo, gpk.hi, guo.lo,
                          guo.hi, gvo.lo, gvo.hi}));
  OEB_RETURN_IF_VALIDATING();
  cudaStream_t st = (cudaStream_t)stream;
  if constexpr (std::is_same<T, float>::value) {
    if (adjoint_tiles()) {  // one tiled launch, no scratch
      const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, guo.sj, guo.sk};
      // 4 levels a chunk: measured against 2-24 at 256 x 256 x 80 (0.139 ms, against 0.172 for
      // the fewest chunks that fill one wave, 27 levels)
      const int kb = tuned_kb(4);
      return launch<p_grad_c_adj_f32>(tile_grid(d.nx + 1, d.ny + 1, d.nz + 1, 32, kPgcTJ, kb),
                                      sizeof(PgcAdjF32Smem), st, gub.origin, gvb.origin, gdb.origin, ggb.origin,
                                      gpb.origin, grx.origin, gry.origin, gdp.origin, ggz.origin, gpk.origin,
                                      guo.origin, gvo.origin, dt2, d, kb);
    }
  }
  const TermLayout lay = term_layout(uoutb);
  void* buf = nullptr;
  OEB_TRY(scratch_alloc(&buf, (size_t)lay.n * 10 * sizeof(T), st));
  PgcTerms<T> tm;
  for (int q = 0; q < 10; ++q) tm.t[q] = static_cast<T*>(buf) + q * lay.n + lay.org;
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, guo.sj, guo.sk};
  const int kb = tuned_kb(kKB);
  oeb_status stt = launch<p_grad_c_adj_terms_kernel<T>>(grid_for(*dom, kb), 0, st, tm, gub.origin, gvb.origin,
                                                        grx.origin, gry.origin, gdp.origin, ggz.origin, gpk.origin,
                                                        guo.origin, gvo.origin, dt2, d, kb);
  if (stt == OEB_OK)
    stt = launch<p_grad_c_adj_gather_kernel<T>>(tile_grid(d.nx + 1, d.ny + 1, d.nz + 1, kTI, kTJ, kb), 0, st,
                                                gdb.origin, ggb.origin, gpb.origin, tm, d, kb);
  scratch_free(buf, st);
  return stt;
}

// ============================== nh_p_grad: tangent-linear and adjoint =================
// nh_p_grad.h:121-141 at point p along the axis of stride s (i+1 for uout, j+1 for vout),
// with X0 = X(p), X1 = X(p,k+1) and x0, x1 the same at p+s:
//   out = (in + c1 fk + c2 fp) rd,  c1 = dt / ((pk1 - pk0) + (pkx1 - pkx0)),  c2 = dt / (w1 + w1x),
//   fk = A1 B1 + A2 B2,  fp = A1 P1 + A2 P2,
//   A1 = gz1 - gx0, A2 = gz0 - gx1, B1 = pkx1 - pk0, B2 = pk1 - pkx0, P1 = ppx1 - pp0, P2 = pp1 - ppx0.
// Active inputs: uin, vin, gz, pp, pk3, wk1 (rdx, rdy, dt are parameters).  With U = outb rd,
// fkb = U c1, fpb = U c2, sb = -fkb fk / (wk + wkx) and wb = -fpb fp / (w1 + w1x), the
// transpose is: inb += U;
//   gz:  a1 = fkb B1 + fpb P1 -> gz1 += a1, gx0 -= a1;  a2 = fkb B2 + fpb P2 -> gz0 += a2, gx1 -= a2
//   pk3: c1 = fkb A1 + sb -> pkx1 += c1, pk0 -= c1;     c2 = fkb A2 + sb -> pk1 += c2, pkx0 -= c2
//   pp:  e1 = fpb A1 -> ppx1 += e1, pp0 -= e1;          e2 = fpb A2 -> pp1 += e2, ppx0 -= e2
//   wk1: w1 += wb, w1x += wb.
// Pass 1 writes uinb, vinb and the seven terms of each axis; pass 2 gathers them.
template <class T>
struct NhpTerms {
  T* t[14];  // per axis (u: 0-6, v: 7-13): a1, a2, c1, c2, e1, e2, wb
};

// The seven terms of point o along the axis of stride s (both forms of the adjoint use these
// expressions).
template <class T>
__device__ __forceinline__ void nhp_adj_terms(T (&t)[7], const T* __restrict__ gz, const T* __restrict__ pp,
                                              const T* __restrict__ pk3, const T* __restrict__ wk1, int64_t o,
                                              int64_t s, int64_t sk, T gz0, T gz1, T pk0, T pk1, T pp0, T pp1, T w1,
                                              T dt, T U) {
  const T gx0 = ld(gz + o + s), gx1 = ld(gz + o + s + sk);
  const T pkx0 = ld(pk3 + o + s), pkx1 = ld(pk3 + o + s + sk);
  const T ppx0 = ld(pp + o + s), ppx1 = ld(pp + o + s + sk);
  const T A1 = gz1 - gx0, A2 = gz0 - gx1;
  const T B1 = pkx1 - pk0, B2 = pk1 - pkx0;
  const T P1 = ppx1 - pp0, P2 = pp1 - ppx0;
  const T fk = A1 * B1 + A2 * B2, fp = A1 * P1 + A2 * P2;
  const T rs = T(1) / ((pk1 - pk0) + (pkx1 - pkx0));
  const T rw = T(1) / (w1 + ld(wk1 + o + s));
  const T Ud = U * dt;
  const T fkb = Ud * rs, fpb = Ud * rw;
  const T sb = -(fkb * fk) * rs;
  t[0] = fkb * B1 + fpb * P1;
  t[1] = fkb * B2 + fpb * P2;
  t[2] = fkb * A1 + sb;
  t[3] = fkb * A2 + sb;
  t[4] = fpb * A1;
  t[5] = fpb * A2;
  t[6] = -(fpb * fp) * rw;
}

template <class T>
__device__ __forceinline__ void nhp_adj_axis(T* const* t, const T* __restrict__ gz, const T* __restrict__ pp,
                                             const T* __restrict__ pk3, const T* __restrict__ wk1, int64_t o,
                                             int64_t s, int64_t sk, T gz0, T gz1, T pk0, T pk1, T pp0, T pp1, T w1,
                                             T dt, T U) {
  T v[7];
  nhp_adj_terms(v, gz, pp, pk3, wk1, o, s, sk, gz0, gz1, pk0, pk1, pp0, pp1, w1, dt, U);
#pragma unroll
  for (int q = 0; q < 7; ++q) t[q][o] = v[q];
}

template <class T>
struct nh_p_grad_adj_terms_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, NhpTerms<T> tm, T* __restrict__ uinb,
                                             T* __restrict__ vinb, const T* __restrict__ rdx,
                                             const T* __restrict__ rdy, const T* __restrict__ gz,
                                             const T* __restrict__ pp, const T* __restrict__ pk3,
                                             const T* __restrict__ wk1, const T* __restrict__ uoutb,
                                             const T* __restrict__ voutb, T dt, Dims d, int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    for_points<RowUnroll<T>::value>(blk, d, kb, [&](int64_t o, int) {
      const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pk3 + o), pk1 = ld(pk3 + o + sk);
      const T pp0 = ld(pp + o), pp1 = ld(pp + o + sk), w1 = ld(wk1 + o);
      const T U = ld(uoutb + o) * ld(rdx + o), V = ld(voutb + o) * ld(rdy + o);
      uinb[o] = U;
      vinb[o] = V;
      nhp_adj_axis(tm.t, gz, pp, pk3, wk1, o, 1, sk, gz0, gz1, pk0, pk1, pp0, pp1, w1, dt, U);
      nhp_adj_axis(tm.t + 7, gz, pp, pk3, wk1, o, sj, sk, gz0, gz1, pk0, pk1, pp0, pp1, w1, dt, V);
    });
  }
};

// Every cell c of [0, N] x [0, N] x [0, Nz] (wk1b only below Nz) gathers, along axis s, the
// terms of the interior points c, c-s, c-k and c-s-k.
template <class T>
struct nh_p_grad_adj_gather_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ gzb, T* __restrict__ ppb,
                                             T* __restrict__ pk3b, T* __restrict__ wk1b, NhpTerms<T> tm, Dims d,
                                             int kb) {
    const int64_t sj = d.sj, sk = d.sk;
    for_box_k<RowUnroll<T>::value>(blk, sj, sk, 0, 0, d.nx + 1, d.ny + 1, d.nz + 1, kb,
                                   [&](int64_t o, int i, int j, int k) {
      T gb = T(0), pb = T(0), kb3 = T(0), wb = T(0);
  #pragma unroll
      for (int ax = 0; ax < 2; ++ax) {
        T* const* t = tm.t + 7 * ax;
        const int di = ax == 0 ? 1 : 0, dj = 1 - di;
        const int64_t s = ax == 0 ? 1 : sj;
        if (inside(d, i, j, k)) {  // p = c
          gb = gb + t[1][o];
          kb3 = kb3 - t[2][o];
          pb = pb - t[4][o];
          wb = wb + t[6][o];
        }
        if (inside(d, i - di, j - dj, k)) {  // p = c - s
          gb = gb - t[0][o - s];
          kb3 = kb3 - t[3][o - s];
          pb = pb - t[5][o - s];
          wb = wb + t[6][o - s];
        }
        if (inside(d, i, j, k - 1)) {  // p = c - k
          gb = gb + t[0][o - sk];
          kb3 = kb3 + t[3][o - sk];
          pb = pb + t[5][o - sk];
        }
        if (inside(d, i - di, j - dj, k - 1)) {  // p = c - s - k
          gb = gb - t[1][o - s - sk];
          kb3 = kb3 + t[2][o - s - sk];
          pb = pb + t[4][o - s - sk];
        }
      }
      gzb[o] = gb;
      ppb[o] = pb;
      pk3b[o] = kb3;
      if (k < d.nz) wk1b[o] = wb;
    });
  }
};

// ---- FP32 nh_p_grad adjoint in one tiled launch ------------------------------------------
// As p_grad_c_adj_f32: a CTA owns a 32 x 16 tile of the gather box [0, N]^2 and a chunk of its
// levels [0, Nz], and marches k with the terms (nhp_adj_terms) of levels k and k-1 in a
// two-level shared-memory ring; here a cell reads the points c and c - s, so the x-axis terms
// cover the tile and one more column on its left, the y-axis terms one more row below.
struct NhpAdjF32Smem {
  float tx[2][7][kPgcTJ][33];      // x-axis terms: rows cj0 .., columns ci0 - 1 .. ci0 + 31
  float ty[2][7][kPgcTJ + 1][32];  // y-axis terms: rows cj0 - 1 .. cj0 + 15, columns ci0 ..
};

struct nh_p_grad_adj_f32 {
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uinb, float* __restrict__ vinb,
                                             float* __restrict__ gzb, float* __restrict__ ppb,
                                             float* __restrict__ pk3b, float* __restrict__ wk1b,
                                             const float* __restrict__ rdx, const float* __restrict__ rdy,
                                             const float* __restrict__ gz, const float* __restrict__ pp,
                                             const float* __restrict__ pk3, const float* __restrict__ wk1,
                                             const float* __restrict__ uoutb, const float* __restrict__ voutb,
                                             float dt, Dims d, int kb) {
    using T = float;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    NhpAdjF32Smem& s = *reinterpret_cast<NhpAdjF32Smem*>(smem_raw);
    const int64_t sj = d.sj, sk = d.sk;
    const int ci0 = (int)blk.x * 32, cj0 = (int)blk.y * kPgcTJ;     // the tile's first cell
    const int kz0 = (int)blk.z * kb, kz1 = min(kz0 + kb, d.nz + 1);  // its levels of [0, nz]
    const int tid = threadIdx.y * kTX + threadIdx.x;
    auto terms = [&](int k, bool own) {
      const int slot = k & 1;
      const int64_t kofs = (int64_t)k * sk;
      for (int e = tid; e < 33 * (kPgcTJ + 1); e += kThreads) {
        const int a = e % 33, b = e / 33;            // point (ci0 - 1 + a, cj0 - 1 + b)
        const int i = ci0 - 1 + a, j = cj0 - 1 + b;
        const bool xs = b >= 1, ys = a >= 1;          // in the x-axis / y-axis region
        if (!(xs || ys) || !inside(d, i, j, k)) continue;
        const int64_t o = kofs + i + (int64_t)j * sj;
        const T gz0 = ld(gz + o), gz1 = ld(gz + o + sk), pk0 = ld(pk3 + o), pk1 = ld(pk3 + o + sk);
        const T pp0 = ld(pp + o), pp1 = ld(pp + o + sk), w1 = ld(wk1 + o);
        const T U = ld(uoutb + o) * ld(rdx + o), V = ld(voutb + o) * ld(rdy + o);
        if (own && xs && ys) {  // the tile's own cells
          uinb[o] = U;
          vinb[o] = V;
        }
        T v[7];
        if (xs) {
          nhp_adj_terms(v, gz, pp, pk3, wk1, o, 1, sk, gz0, gz1, pk0, pk1, pp0, pp1, w1, dt, U);
#pragma unroll
          for (int q = 0; q < 7; ++q) s.tx[slot][q][b - 1][a] = v[q];
        }
        if (ys) {
          nhp_adj_terms(v, gz, pp, pk3, wk1, o, sj, sk, gz0, gz1, pk0, pk1, pp0, pp1, w1, dt, V);
#pragma unroll
          for (int q = 0; q < 7; ++q) s.ty[slot][q][b][a - 1] = v[q];
        }
      }
    };
    if (kz0 >= 1) terms(kz0 - 1, false);  // the level below the chunk's first (its cells read it)
#pragma unroll 1
    for (int k = kz0; k < kz1; ++k) {
      if (k < d.nz) terms(k, true);
      __syncthreads();
      const int cur = k & 1, prev = (k - 1) & 1;
      const int64_t kofs = (int64_t)k * sk;
#pragma unroll
      for (int r = 0; r < kPgcTJ / kTY; ++r) {
        const int ta = threadIdx.x, tb = threadIdx.y + kTY * r;
        const int i = ci0 + ta, j = cj0 + tb;
        if (i > d.nx || j > d.ny) continue;  // the gather box is [0, N]^2
        T gb = T(0), pb = T(0), kb3 = T(0), wb = T(0);
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
          const int di = ax == 0 ? 1 : 0, dj = 1 - di;
          // term q of axis ax at the point c (back = 0) or c - s (back = 1) of ring slot sl
          auto t = [&](int sl, int q, int back) {
            return ax == 0 ? s.tx[sl][q][tb][ta + 1 - back] : s.ty[sl][q][tb + 1 - back][ta];
          };
          if (inside(d, i, j, k)) {  // p = c
            gb = gb + t(cur, 1, 0);
            kb3 = kb3 - t(cur, 2, 0);
            pb = pb - t(cur, 4, 0);
            wb = wb + t(cur, 6, 0);
          }
          if (inside(d, i - di, j - dj, k)) {  // p = c - s
            gb = gb - t(cur, 0, 1);
            kb3 = kb3 - t(cur, 3, 1);
            pb = pb - t(cur, 5, 1);
            wb = wb + t(cur, 6, 1);
          }
          if (inside(d, i, j, k - 1)) {  // p = c - k
            gb = gb + t(prev, 0, 0);
            kb3 = kb3 + t(prev, 3, 0);
            pb = pb + t(prev, 5, 0);
          }
          if (inside(d, i - di, j - dj, k - 1)) {  // p = c - s - k
            gb = gb - t(prev, 1, 1);
            kb3 = kb3 + t(prev, 2, 1);
            pb = pb + t(prev, 4, 1);
          }
        }
        const int64_t o = kofs + i + (int64_t)j * sj;
        gzb[o] = gb;
        ppb[o] = pb;
        pk3b[o] = kb3;
        if (k < d.nz) wk1b[o] = wb;
      }
      __syncthreads();  // level k + 1's terms replace level k - 1's
    }
  }
};

template <class T, class M3>
oeb_status nh_p_grad_tl_entry(const M3* duout, const M3* dvout, const M3* uin, const M3* vin, const M3* rdx,
                              const M3* rdy, const M3* gz, const M3* pp, const M3* pk3, const M3* wk1,
                              const M3* duin, const M3* dvin, const M3* dgz, const M3* dpp, const M3* dpk3,
                              const M3* dwk1, T dt, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(nh_p_grad_entry<T>(duout, dvout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, dt, dom, stream));
    OEB_TRY(nh_p_grad_entry<T>(duout, dvout, duin, dvin, rdx, rdy, dgz, dpp, dpk3, dwk1, dt, dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *u, *v, *rx, *ry, *g, *p, *pk, *w, *ou, *ov;
  OEB_TRY(arr.pack(uin, duin, &u));
  OEB_TRY(arr.pack(vin, dvin, &v));
  OEB_TRY(arr.pack(rdx, (const M3*)nullptr, &rx));
  OEB_TRY(arr.pack(rdy, (const M3*)nullptr, &ry));
  OEB_TRY(arr.pack(gz, dgz, &g));
  OEB_TRY(arr.pack(pp, dpp, &p));
  OEB_TRY(arr.pack(pk3, dpk3, &pk));
  OEB_TRY(arr.pack(wk1, dwk1, &w));
  OEB_TRY(arr.alloc(duout, &ou));
  OEB_TRY(arr.alloc(dvout, &ov));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, uin->strides[1], uin->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<nh_p_grad_kernel<D>>(grid_for(*dom, kb), 0, (cudaStream_t)stream, ou, ov, u, v, rx, ry, g, p, pk, w,
                                      D(dt), d, kb));
  OEB_TRY(arr.unpack(duout->aligned + duout->offset, ou, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dvout->aligned + dvout->offset, ov, *dom, kInterior, d.sj, d.sk);
}

template <class T, class M3>
oeb_status nh_p_grad_adj_entry(const M3* uinb, const M3* vinb, const M3* gzb, const M3* ppb, const M3* pk3b,
                               const M3* wk1b, const M3* uin, const M3* vin, const M3* rdx, const M3* rdy,
                               const M3* gz, const M3* pp, const M3* pk3, const M3* wk1, const M3* uoutb,
                               const M3* voutb, T dt, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(nh_p_grad_entry<T>(uoutb, voutb, uin, vin, rdx, rdy, gz, pp, pk3, wk1, dt, dom, stream));
  }
  Grid<T> gub, gvb, ggb, gpb, gkb, gwb, grx, gry, ggz, gpp, gpk, gw1, guo, gvo;
  const Reach r11{0, 1, 0, 1, 0, 1}, r10{0, 1, 0, 1, 0, 0};
  OEB_TRY((check_field3<T>(uinb, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<T>(vinb, *dom, kInterior, &gvb)));
  OEB_TRY((check_field3<T>(gzb, *dom, r11, &ggb)));
  OEB_TRY((check_field3<T>(ppb, *dom, r11, &gpb)));
  OEB_TRY((check_field3<T>(pk3b, *dom, r11, &gkb)));
  OEB_TRY((check_field3<T>(wk1b, *dom, r10, &gwb)));
  OEB_TRY((check_field3<T>(rdx, *dom, kInterior, &grx)));
  OEB_TRY((check_field3<T>(rdy, *dom, kInterior, &gry)));
  OEB_TRY((check_field3<T>(gz, *dom, r11, &ggz)));
  OEB_TRY((check_field3<T>(pp, *dom, r11, &gpp)));
  OEB_TRY((check_field3<T>(pk3, *dom, r11, &gpk)));
  OEB_TRY((check_field3<T>(wk1, *dom, r10, &gw1)));
  OEB_TRY((check_field3<T>(uoutb, *dom, kInterior, &guo)));
  OEB_TRY((check_field3<T>(voutb, *dom, kInterior, &gvo)));
  OEB_TRY(check_same_strides<T>(
      {&gub, &gvb, &ggb, &gpb, &gkb, &gwb, &grx, &gry, &ggz, &gpp, &gpk, &gw1, &guo, &gvo}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi, ggb.lo, ggb.hi, gpb.lo, gpb.hi, gkb.lo, gkb.hi, gwb.lo,
                          gwb.hi},
                         {grx.lo, grx.hi, gry.lo, gry.hi, ggz.lo, ggz.hi, gpp.lo, gpp.hi, gpk.lo, gpk.hi, gw1.lo,
                          gw1.hi, guo.lo, guo.hi, gvo.lo, gvo.hi}));
  OEB_RETURN_IF_VALIDATING();
  cudaStream_t st = (cudaStream_t)stream;
  if constexpr (std::is_same<T, float>::value) {
    if (adjoint_tiles()) {  // one tiled launch, no scratch
      const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, guo.sj, guo.sk};
      // 6 levels a chunk: measured against 2-24 at 256 x 256 x 80 (0.165 ms, against 0.218 for
      // the fewest chunks that fill one wave, 41 levels)
      const int kb = tuned_kb(6);
      return launch<nh_p_grad_adj_f32>(tile_grid(d.nx + 1, d.ny + 1, d.nz + 1, 32, kPgcTJ, kb),
                                       sizeof(NhpAdjF32Smem), st, gub.origin, gvb.origin, ggb.origin, gpb.origin,
                                       gkb.origin, gwb.origin, grx.origin, gry.origin, ggz.origin, gpp.origin,
                                       gpk.origin, gw1.origin, guo.origin, gvo.origin, dt, d, kb);
    }
  }
  const TermLayout lay = term_layout(uoutb);
  void* buf = nullptr;
  OEB_TRY(scratch_alloc(&buf, (size_t)lay.n * 14 * sizeof(T), st));
  NhpTerms<T> tm;
  for (int q = 0; q < 14; ++q) tm.t[q] = static_cast<T*>(buf) + q * lay.n + lay.org;
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, guo.sj, guo.sk};
  const int kb = tuned_kb(kKB);
  oeb_status stt = launch<nh_p_grad_adj_terms_kernel<T>>(grid_for(*dom, kb), 0, st, tm, gub.origin, gvb.origin,
                                                         grx.origin, gry.origin, ggz.origin, gpp.origin, gpk.origin,
                                                         gw1.origin, guo.origin, gvo.origin, dt, d, kb);
  if (stt == OEB_OK)
    stt = launch<nh_p_grad_adj_gather_kernel<T>>(tile_grid(d.nx + 1, d.ny + 1, d.nz + 1, kTI, kTJ, kb), 0, st,
                                                 ggb.origin, gpb.origin, gkb.origin, gwb.origin, tm, d, kb);
  scratch_free(buf, st);
  return stt;
}

}  // namespace
}  // namespace oeb

#ifndef OEB_BODIES_ONLY  // the entry points

using namespace oeb;

#define OEB_M3(S) oeb_memref3d_##S
#define OEB_M1(S) oeb_memref1d_##S

#define OEB_POINTWISE_ENTRIES(S, T)                                                                                \
  extern "C" oeb_status oeb_laplace_##S(const OEB_M3(S) * in, const OEB_M3(S) * out, const oeb_domain* dom,        \
                                        void* stream) {                                                            \
    return laplace_entry<T>(in, out, dom, stream);                                                                 \
  }                                                                                                                \
  extern "C" oeb_status oeb_uvbke_##S(const OEB_M3(S) * ub, const OEB_M3(S) * vb, const OEB_M3(S) * uc,            \
                                      const OEB_M3(S) * vc, const OEB_M3(S) * cosa, const OEB_M3(S) * rsina,       \
                                      double dt5, const oeb_domain* dom, void* stream) {                           \
    return uvbke_entry<T>(ub, vb, uc, vc, cosa, rsina, dt5, dom, stream);                                          \
  }                                                                                                                \
  extern "C" oeb_status oeb_p_grad_c_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,    \
                                         const OEB_M3(S) * vin, const OEB_M3(S) * rdxc, const OEB_M3(S) * rdyc,    \
                                         const OEB_M3(S) * delpc, const OEB_M3(S) * gz, const OEB_M3(S) * pkc,     \
                                         T dt2, const oeb_domain* dom, void* stream) {                             \
    return p_grad_c_entry<T>(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, dt2, dom, stream);                  \
  }                                                                                                                \
  extern "C" oeb_status oeb_nh_p_grad_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,   \
                                          const OEB_M3(S) * vin, const OEB_M3(S) * rdx, const OEB_M3(S) * rdy,     \
                                          const OEB_M3(S) * gz, const OEB_M3(S) * pp, const OEB_M3(S) * pk3,       \
                                          const OEB_M3(S) * wk1, T dt, const oeb_domain* dom, void* stream) {      \
    return nh_p_grad_entry<T>(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, dt, dom, stream);                  \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,      \
                                       const OEB_M3(S) * vin, const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1, \
                                       const OEB_M1(S) * tgrlatda0, const OEB_M1(S) * tgrlatda1, T eddlat,         \
                                       T eddlon, const oeb_domain* dom, void* stream) {                            \
    return hadv_entry<T, 3>(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom,     \
                            stream);                                                                               \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv5th_##S(const OEB_M3(S) * uout, const OEB_M3(S) * vout, const OEB_M3(S) * uin,   \
                                          const OEB_M3(S) * vin, const OEB_M1(S) * acrlat0,                        \
                                          const OEB_M1(S) * acrlat1, const OEB_M1(S) * tgrlatda0,                  \
                                          const OEB_M1(S) * tgrlatda1, T eddlat, T eddlon, const oeb_domain* dom,  \
                                          void* stream) {                                                          \
    return hadv_entry<T, 5>(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom,     \
                            stream);                                                                               \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv_tl_##S(const OEB_M3(S) * duout, const OEB_M3(S) * dvout, const OEB_M3(S) * uin, \
                                          const OEB_M3(S) * vin, const OEB_M1(S) * acrlat0,                        \
                                          const OEB_M1(S) * acrlat1, const OEB_M1(S) * tgrlatda0,                  \
                                          const OEB_M1(S) * tgrlatda1, const OEB_M3(S) * duin,                     \
                                          const OEB_M3(S) * dvin, T eddlat, T eddlon, const oeb_domain* dom,       \
                                          void* stream) {                                                          \
    return hadv_tl_entry<T, 3>(duout, dvout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, duin, dvin, eddlat, \
                               eddlon, dom, stream);                                                               \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv5th_tl_##S(                                                                      \
      const OEB_M3(S) * duout, const OEB_M3(S) * dvout, const OEB_M3(S) * uin, const OEB_M3(S) * vin,               \
      const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1, const OEB_M1(S) * tgrlatda0,                           \
      const OEB_M1(S) * tgrlatda1, const OEB_M3(S) * duin, const OEB_M3(S) * dvin, T eddlat, T eddlon,             \
      const oeb_domain* dom, void* stream) {                                                                       \
    return hadv_tl_entry<T, 5>(duout, dvout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, duin, dvin, eddlat, \
                               eddlon, dom, stream);                                                               \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv_adj_##S(                                                                        \
      const OEB_M3(S) * uinb, const OEB_M3(S) * vinb, const OEB_M3(S) * uin, const OEB_M3(S) * vin,                 \
      const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1, const OEB_M1(S) * tgrlatda0,                           \
      const OEB_M1(S) * tgrlatda1, const OEB_M3(S) * uoutb, const OEB_M3(S) * voutb, T eddlat, T eddlon,           \
      const oeb_domain* dom, void* stream) {                                                                       \
    return hadv_adj_entry<T, 3>(uinb, vinb, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, uoutb, voutb,       \
                                eddlat, eddlon, dom, stream);                                                      \
  }                                                                                                                \
  extern "C" oeb_status oeb_hadvuv5th_adj_##S(                                                                     \
      const OEB_M3(S) * uinb, const OEB_M3(S) * vinb, const OEB_M3(S) * uin, const OEB_M3(S) * vin,                 \
      const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1, const OEB_M1(S) * tgrlatda0,                           \
      const OEB_M1(S) * tgrlatda1, const OEB_M3(S) * uoutb, const OEB_M3(S) * voutb, T eddlat, T eddlon,           \
      const oeb_domain* dom, void* stream) {                                                                       \
    return hadv_adj_entry<T, 5>(uinb, vinb, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1, uoutb, voutb,       \
                                eddlat, eddlon, dom, stream);                                                      \
  }

#define OEB_POINTWISE_DIFF_ENTRIES(S, T)                                                                           \
  extern "C" oeb_status oeb_laplace_tl_##S(const OEB_M3(S) * dout, const OEB_M3(S) * in, const OEB_M3(S) * din,     \
                                           const oeb_domain* dom, void* stream) {                                  \
    return laplace_tl_entry<T>(dout, in, din, dom, stream);                                                        \
  }                                                                                                                \
  extern "C" oeb_status oeb_laplace_adj_##S(const OEB_M3(S) * inb, const OEB_M3(S) * in, const OEB_M3(S) * outb,    \
                                            const oeb_domain* dom, void* stream) {                                 \
    return laplace_adj_entry<T>(inb, in, outb, dom, stream);                                                       \
  }                                                                                                                \
  extern "C" oeb_status oeb_uvbke_tl_##S(const OEB_M3(S) * dub, const OEB_M3(S) * dvb, const OEB_M3(S) * uc,        \
                                         const OEB_M3(S) * vc, const OEB_M3(S) * cosa, const OEB_M3(S) * rsina,     \
                                         const OEB_M3(S) * duc, const OEB_M3(S) * dvc, double dt5,                 \
                                         const oeb_domain* dom, void* stream) {                                    \
    return uvbke_tl_entry<T>(dub, dvb, uc, vc, cosa, rsina, duc, dvc, dt5, dom, stream);                           \
  }                                                                                                                \
  extern "C" oeb_status oeb_uvbke_adj_##S(const OEB_M3(S) * ucb, const OEB_M3(S) * vcb, const OEB_M3(S) * uc,       \
                                          const OEB_M3(S) * vc, const OEB_M3(S) * cosa, const OEB_M3(S) * rsina,    \
                                          const OEB_M3(S) * ubb, const OEB_M3(S) * vbb, double dt5,                \
                                          const oeb_domain* dom, void* stream) {                                   \
    return uvbke_adj_entry<T>(ucb, vcb, uc, vc, cosa, rsina, ubb, vbb, dt5, dom, stream);                          \
  }                                                                                                                \
  extern "C" oeb_status oeb_p_grad_c_tl_##S(                                                                       \
      const OEB_M3(S) * duout, const OEB_M3(S) * dvout, const OEB_M3(S) * uin, const OEB_M3(S) * vin,               \
      const OEB_M3(S) * rdxc, const OEB_M3(S) * rdyc, const OEB_M3(S) * delpc, const OEB_M3(S) * gz,                \
      const OEB_M3(S) * pkc, const OEB_M3(S) * duin, const OEB_M3(S) * dvin, const OEB_M3(S) * ddelpc,             \
      const OEB_M3(S) * dgz, const OEB_M3(S) * dpkc, T dt2, const oeb_domain* dom, void* stream) {                 \
    return p_grad_c_tl_entry<T>(duout, dvout, uin, vin, rdxc, rdyc, delpc, gz, pkc, duin, dvin, ddelpc, dgz, dpkc, \
                                dt2, dom, stream);                                                                 \
  }                                                                                                                \
  extern "C" oeb_status oeb_p_grad_c_adj_##S(                                                                      \
      const OEB_M3(S) * uinb, const OEB_M3(S) * vinb, const OEB_M3(S) * delpcb, const OEB_M3(S) * gzb,              \
      const OEB_M3(S) * pkcb, const OEB_M3(S) * uin, const OEB_M3(S) * vin, const OEB_M3(S) * rdxc,                 \
      const OEB_M3(S) * rdyc, const OEB_M3(S) * delpc, const OEB_M3(S) * gz, const OEB_M3(S) * pkc,                 \
      const OEB_M3(S) * uoutb, const OEB_M3(S) * voutb, T dt2, const oeb_domain* dom, void* stream) {              \
    return p_grad_c_adj_entry<T>(uinb, vinb, delpcb, gzb, pkcb, uin, vin, rdxc, rdyc, delpc, gz, pkc, uoutb,       \
                                 voutb, dt2, dom, stream);                                                         \
  }                                                                                                                \
  extern "C" oeb_status oeb_nh_p_grad_tl_##S(                                                                      \
      const OEB_M3(S) * duout, const OEB_M3(S) * dvout, const OEB_M3(S) * uin, const OEB_M3(S) * vin,               \
      const OEB_M3(S) * rdx, const OEB_M3(S) * rdy, const OEB_M3(S) * gz, const OEB_M3(S) * pp,                     \
      const OEB_M3(S) * pk3, const OEB_M3(S) * wk1, const OEB_M3(S) * duin, const OEB_M3(S) * dvin,                 \
      const OEB_M3(S) * dgz, const OEB_M3(S) * dpp, const OEB_M3(S) * dpk3, const OEB_M3(S) * dwk1, T dt,           \
      const oeb_domain* dom, void* stream) {                                                                       \
    return nh_p_grad_tl_entry<T>(duout, dvout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, duin, dvin, dgz, dpp, dpk3,   \
                                 dwk1, dt, dom, stream);                                                           \
  }                                                                                                                \
  extern "C" oeb_status oeb_nh_p_grad_adj_##S(                                                                     \
      const OEB_M3(S) * uinb, const OEB_M3(S) * vinb, const OEB_M3(S) * gzb, const OEB_M3(S) * ppb,                 \
      const OEB_M3(S) * pk3b, const OEB_M3(S) * wk1b, const OEB_M3(S) * uin, const OEB_M3(S) * vin,                 \
      const OEB_M3(S) * rdx, const OEB_M3(S) * rdy, const OEB_M3(S) * gz, const OEB_M3(S) * pp,                     \
      const OEB_M3(S) * pk3, const OEB_M3(S) * wk1, const OEB_M3(S) * uoutb, const OEB_M3(S) * voutb, T dt,         \
      const oeb_domain* dom, void* stream) {                                                                       \
    return nh_p_grad_adj_entry<T>(uinb, vinb, gzb, ppb, pk3b, wk1b, uin, vin, rdx, rdy, gz, pp, pk3, wk1, uoutb,   \
                                  voutb, dt, dom, stream);                                                         \
  }

OEB_POINTWISE_ENTRIES(f64, double)
OEB_POINTWISE_ENTRIES(f32, float)
OEB_POINTWISE_DIFF_ENTRIES(f64, double)
OEB_POINTWISE_DIFF_ENTRIES(f32, float)

// The chained step's fused stages (fused.cuh).
static oeb_status p_grad_c_profiled_entry(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                   const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                   const oeb_memref3d_f32* rdxc, const oeb_memref3d_f32* rdyc,
                                   const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz,
                                   const oeb_memref3d_f32* pkc, const double* gz_base, const double* pkc_base,
                                   float dt2, const oeb_domain* dom, void* stream) {
  Grid<float> g[9];
  OEB_TRY(p_grad_c_check<float>(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, dom, g));
  if (!gz_base || !pkc_base) return OEB_ERR_NULL;
  OEB_RETURN_IF_VALIDATING();
  const int kb = tuned_kb(kKB);
  return launch<p_grad_c_profiled_f32>(grid_for(*dom, kb), 0, (cudaStream_t)stream, g[0].origin, g[1].origin,
                                       g[2].origin, g[3].origin, g[4].origin, g[5].origin, g[6].origin, g[7].origin,
                                       g[8].origin, gz_base, pkc_base, dt2, make_dims(*dom, g[0]), kb);
}

static oeb_status nh_p_grad_profiled_entry(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                    const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                    const oeb_memref3d_f32* rdx, const oeb_memref3d_f32* rdy,
                                    const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp,
                                    const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1, const double* gz_base,
                                    const double* pp_base, const double* pk3_base, float dt,
                                    const oeb_domain* dom, void* stream) {
  Grid<float> g[10];
  OEB_TRY(nh_p_grad_check<float>(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, dom, g));
  if (!gz_base || !pp_base || !pk3_base) return OEB_ERR_NULL;
  OEB_RETURN_IF_VALIDATING();
  const int kb = tuned_kb(kKB);
  return launch<nh_p_grad_profiled_f32>(grid_for(*dom, kb), 0, (cudaStream_t)stream, g[0].origin, g[1].origin,
                                        g[2].origin, g[3].origin, g[4].origin, g[5].origin, g[6].origin,
                                        g[7].origin, g[8].origin, g[9].origin, gz_base, pp_base, pk3_base, dt,
                                        make_dims(*dom, g[0]), kb);
}

extern "C" oeb_status oeb_p_grad_c_f32_profiled(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                             const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                             const oeb_memref3d_f32* rdxc, const oeb_memref3d_f32* rdyc,
                                             const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz,
                                             const oeb_memref3d_f32* pkc, const double* gz_base,
                                             const double* pkc_base, float dt2, const oeb_domain* dom,
                                             void* stream) {
  return p_grad_c_profiled_entry(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, gz_base, pkc_base, dt2, dom,
                                 stream);
}
extern "C" oeb_status oeb_nh_p_grad_f32_profiled(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                              const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                              const oeb_memref3d_f32* rdx, const oeb_memref3d_f32* rdy,
                                              const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp,
                                              const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1,
                                              const double* gz_base, const double* pp_base,
                                              const double* pk3_base, float dt, const oeb_domain* dom,
                                              void* stream) {
  return nh_p_grad_profiled_entry(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, gz_base, pp_base, pk3_base, dt,
                                  dom, stream);
}

#define OEB_FUSED_ENTRIES(S, T)                                                                                    \
  oeb_status oeb::hadvuv5th_update(const OEB_M3(S) * u2, const OEB_M3(S) * v2, const OEB_M3(S) * u1,               \
                                   const OEB_M3(S) * v1, const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1,     \
                                   const OEB_M1(S) * tgrlatda0, const OEB_M1(S) * tgrlatda1, T eddlat, T eddlon,   \
                                   T alpha, const oeb_domain* dom, void* stream) {                                 \
    return hadv_entry<T, 5>(u2, v2, u1, v1, acrlat0, acrlat1, tgrlatda0, tgrlatda1, eddlat, eddlon, dom, stream,   \
                            alpha, 1);                                                                             \
  }                                                                                                                \
  oeb_status oeb::hadvuv5th_adj_update(const OEB_M3(S) * u1b, const OEB_M3(S) * v1b, const OEB_M3(S) * u1,         \
                                       const OEB_M3(S) * v1, const OEB_M1(S) * acrlat0, const OEB_M1(S) * acrlat1, \
                                       const OEB_M1(S) * tgrlatda0, const OEB_M1(S) * tgrlatda1,                   \
                                       const OEB_M3(S) * u2b, const OEB_M3(S) * v2b, T eddlat, T eddlon, T alpha,  \
                                       const oeb_domain* dom, void* stream) {                                      \
    return hadv_adj_entry<T, 5>(u1b, v1b, u1, v1, acrlat0, acrlat1, tgrlatda0, tgrlatda1, u2b, v2b, eddlat, eddlon, \
                                dom, stream, alpha, 1);                                                            \
  }

OEB_FUSED_ENTRIES(f64, double)
OEB_FUSED_ENTRIES(f32, float)

#endif  // OEB_BODIES_ONLY
