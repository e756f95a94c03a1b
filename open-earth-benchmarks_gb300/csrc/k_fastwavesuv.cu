// k_fastwavesuv.cu -- fastwavesuv (kernels/fastwavesuv.h:154-191) in FP64 and FP32.
//
// The OpenMP variant evaluates ppgk = wgtfac*ppuv + (1-wgtfac)*ppuv(k-1) six times per point
// ((i,j),(i+1,j),(i,j+1) at k and k+1).  Here each CTA marches upward through kb k-levels
// of a 32 x 32 tile: at level k every point of the tile plus a one-cell apron in i and j
// computes ppgk(k+1) once, keeps it in a register for level k+1, and publishes
// ppgc = ppgk(k+1) - ppgk(k) and the hhl sum and difference of its column through shared
// memory; the output pass then reads its i+1 and j+1 neighbours from there.
//
// Compiled with --fmad=false (see k_pointwise.cu).
#include <type_traits>

#include "precision.cuh"
#include "stencil_util.cuh"
#include "tangent.cuh"

// Built on its own, this file's bodies and helpers are local to it; the step kernel
// (step.cu) includes it with OEB_BODIES_ONLY and a namespace of its own instead.
#ifndef OEB_BODIES_NS
#define OEB_BODIES_NS
#endif
namespace oeb {
namespace OEB_BODIES_NS {

constexpr int kT = 32;
constexpr int kR = kT + 1;                                // apron of one cell in i and j
constexpr int kOwned = (kR * kR + kThreads - 1) / kThreads;  // region points per thread

template <class T>
struct FastwavesSmem {
  T ppgc[kR][kR];
  T hs[kR][kR];  // hhl(k+1) + hhl(k)
  T hd[kR][kR];  // hhl(k+1) - hhl(k)
  T fx2[kT];     // 2 * fx(j)
};

template <class T>
struct fastwavesuv_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFwsFwd);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uout, T* __restrict__ vout,
                                             const T* __restrict__ uin, const T* __restrict__ vin,
                                             const T* __restrict__ utens, const T* __restrict__ vtens,
                                             const T* __restrict__ wgtfac, const T* __restrict__ ppuv,
                                             const T* __restrict__ hhl, const T* __restrict__ rho,
                                             const T* __restrict__ fx, int64_t s1d, T ed2, T dt, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FastwavesSmem<T>& s = *reinterpret_cast<FastwavesSmem<T>*>(smem_raw);
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int sj = (int)d.sj;
    const int64_t sk = d.sk;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    if (tid < kT) {
      const int j = j0 + tid;
      s.fx2[tid] = (j < d.ny) ? T(2.0) * ld(fx + (int64_t)j * s1d) : T(0);
    }
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);

    // Region points owned by this thread, and ppgk at the current level for each.
    int own_off[kOwned];
    bool own_ok[kOwned];
    T ppgk_cur[kOwned];
  #pragma unroll
    for (int t = 0; t < kOwned; ++t) {
      const int e = tid + t * kThreads;
      const int b = e / kR, a = e - (e / kR) * kR;
      const int i = i0 + a, j = j0 + b;
      own_ok[t] = e < kR * kR && i < d.nx + 1 && j < d.ny + 1;
      own_off[t] = i + j * sj;
      ppgk_cur[t] = T(0);
      if (own_ok[t]) {
        const int64_t o = (int64_t)k0 * sk + own_off[t];
        const T w = ld(wgtfac + o);
        ppgk_cur[t] = w * ld(ppuv + o) + (T(1.0) - w) * ld(ppuv + o - sk);  // fastwavesuv.h:162
      }
    }

  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * sk;
      const T* const late[6] = {ppuv, rho, uin, utens, vin, vtens};  // read in the last phase
      prefetch_tile(late, kofs, i0, j0, d.nx, d.ny, sj);
  #pragma unroll
      for (int t = 0; t < kOwned; ++t) {
        const int e = tid + t * kThreads;
        if (e < kR * kR) {
          const int b = e / kR, a = e - b * kR;
          T pc = T(0), hsum = T(0), hdif = T(0);
          if (own_ok[t]) {
            const int64_t o = kofs + own_off[t];
            const T w1 = ld(wgtfac + o + sk);
            const T next = w1 * ld(ppuv + o + sk) + (T(1.0) - w1) * ld(ppuv + o);  // ppgk at k+1
            pc = next - ppgk_cur[t];
            ppgk_cur[t] = next;
            const T h1 = ld(hhl + o + sk), h0 = ld(hhl + o);
            hsum = h1 + h0;
            hdif = h1 - h0;
          }
          s.ppgc[b][a] = pc;
          s.hs[b][a] = hsum;
          s.hd[b][a] = hdif;
        }
      }
      __syncthreads();
      for_region<kT, kT>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        if (i < d.nx && j < d.ny) {
          const int64_t o = kofs + i + j * sj;
          const T p0 = ld(ppuv + o);
          const T r0 = ld(rho + o);
          // fastwavesuv.h:172-175
          const T ppgu = (ld(ppuv + o + 1) - p0) + (scale2<-1>(s.ppgc[b][a + 1] + s.ppgc[b][a]) *
                                                        (s.hs[b][a] - s.hs[b][a + 1])) /
                                                           (s.hd[b][a] + s.hd[b][a + 1]);
          // fastwavesuv.h:177-180
          const T ppgv = (ld(ppuv + o + sj) - p0) + (scale2<-1>(s.ppgc[b + 1][a] + s.ppgc[b][a]) *
                                                         (s.hs[b][a] - s.hs[b + 1][a])) /
                                                            (s.hd[b][a] + s.hd[b + 1][a]);
          // fastwavesuv.h:182-186
          uout[o] = ld(uin + o) + dt * (ld(utens + o) - ppgu * (s.fx2[b] / (ld(rho + o + 1) + r0)));
          vout[o] = ld(vin + o) + dt * (ld(vtens + o) - ppgv * (ed2 / (ld(rho + o + sj) + r0)));
        }
      });
      __syncthreads();
    }
  }
};

constexpr int kKB = 1;     // k-levels per CTA by default (the most CTAs hide latency best)
// the adjoint march's k-levels per CTA (measured at 128 x 128 x 80: FP64 best at 3, FP32 at
// 2; a block of kb levels reads the coefficients of kb + 2)
template <class T>
constexpr int adj_kb() {
  return sizeof(T) == 4 ? 2 : 3;
}
// the same for the FP32 march that forms its coefficients itself (each level's are formed
// (kb + 2) / kb times)
constexpr int kAdjFusedKB = 4;

template <class T, class M3, class M1>
oeb_status fastwavesuv_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* utens,
                             const M3* vtens, const M3* wgtfac, const M3* ppuv, const M3* hhl, const M3* rho,
                             const M1* fx, T edadlat, T dt, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gu, gv, gui, gvi, gut, gvt, gw, gp, gh, gr;
  Line<T> lfx;
  OEB_TRY((check_field3<T>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<T>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<T>(uin, *dom, kInterior, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, kInterior, &gvi)));
  OEB_TRY((check_field3<T>(utens, *dom, kInterior, &gut)));
  OEB_TRY((check_field3<T>(vtens, *dom, kInterior, &gvt)));
  OEB_TRY((check_field3<T>(wgtfac, *dom, Reach{0, 1, 0, 1, 0, 1}, &gw)));
  OEB_TRY((check_field3<T>(ppuv, *dom, Reach{0, 1, 0, 1, 1, 1}, &gp)));
  OEB_TRY((check_field3<T>(hhl, *dom, Reach{0, 1, 0, 1, 0, 1}, &gh)));
  OEB_TRY((check_field3<T>(rho, *dom, Reach{0, 1, 0, 1, 0, 0}, &gr)));
  OEB_TRY((check_field1<T>(fx, *dom, 0, 0, &lfx)));
  OEB_TRY(check_same_strides<T>({&gu, &gv, &gui, &gvi, &gut, &gvt, &gw, &gp, &gh, &gr}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi},
                         {gui.lo, gui.hi, gvi.lo, gvi.hi, gut.lo, gut.hi, gvt.lo, gvt.hi, gw.lo, gw.hi, gp.lo, gp.hi,
                          gh.lo, gh.hi, gr.lo, gr.hi, lfx.lo, lfx.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gu.sj, gu.sk};
  const T ed2 = T(2.0) * edadlat;  // ElementType(2.0) * edadlat, fastwavesuv.h:186
  const int kb = tuned_kb(kKB);
  return launch<fastwavesuv_kernel<T>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(FastwavesSmem<T>),
                                       (cudaStream_t)stream, gu.origin, gv.origin, gui.origin, gvi.origin, gut.origin,
                                       gvt.origin, gw.origin, gp.origin, gh.origin, gr.origin, lfx.origin, lfx.s, ed2,
                                       dt, d, kb);
}

// Tangent-linear fastwavesuv with respect to (uin, vin, utens, vtens, ppuv); wgtfac, hhl,
// rho and fx are parameters.  The map is linear in these inputs, so this is also the
// forward stencil applied to the perturbation; it runs on Dual<T> like the others.
template <class T, class M3, class M1>
oeb_status fastwavesuv_tl_entry(const M3* duout, const M3* dvout, const M3* uin, const M3* vin, const M3* utens,
                                const M3* vtens, const M3* wgtfac, const M3* ppuv, const M3* hhl, const M3* rho,
                                const M1* fx, const M3* duin, const M3* dvin, const M3* dutens, const M3* dvtens,
                                const M3* dppuv, T edadlat, T dt, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(fastwavesuv_entry<T>(duout, dvout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, edadlat, dt, dom,
                                 stream));
    OEB_TRY(fastwavesuv_entry<T>(duout, dvout, duin, dvin, dutens, dvtens, wgtfac, dppuv, hhl, rho, fx, edadlat, dt,
                                 dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *u, *v, *ut, *vt, *w, *p, *h, *r, *f, *ou, *ov;
  OEB_TRY(arr.pack(uin, duin, &u));
  OEB_TRY(arr.pack(vin, dvin, &v));
  OEB_TRY(arr.pack(utens, dutens, &ut));
  OEB_TRY(arr.pack(vtens, dvtens, &vt));
  OEB_TRY(arr.pack(wgtfac, (const M3*)nullptr, &w));
  OEB_TRY(arr.pack(ppuv, dppuv, &p));
  OEB_TRY(arr.pack(hhl, (const M3*)nullptr, &h));
  OEB_TRY(arr.pack(rho, (const M3*)nullptr, &r));
  OEB_TRY(arr.pack(fx, (const M1*)nullptr, &f));
  OEB_TRY(arr.alloc(duout, &ou));
  OEB_TRY(arr.alloc(dvout, &ov));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, uin->strides[1], uin->strides[0]};
  const D ed2 = D(T(2.0) * edadlat);
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<fastwavesuv_kernel<D>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(FastwavesSmem<D>),
                                        (cudaStream_t)stream, ou, ov, u, v, ut, vt, w, p, h, r, f, fx->strides[0], ed2,
                                        D(dt), d, kb));
  OEB_TRY(arr.unpack(duout->aligned + duout->offset, ou, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dvout->aligned + dvout->offset, ov, *dom, kInterior, d.sj, d.sk);
}

// ============================== adjoint ===========================================
// fastwavesuv is linear in x = (uin, vin, utens, vtens, ppuv) for fixed wgtfac, hhl, rho, fx:
//   uout = uin + dt (utens - ppgu qx),  qx = 2 fx(j) / (rho(i+1) + rho(i))
//   ppgu = (ppuv(i+1) - ppuv(i)) + (ppgc(i+1) + ppgc(i)) gx,  gx = 0.5 Hs / Hd   (fastwavesuv.h:172-175)
//   ppgc(k) = ppgk(k+1) - ppgk(k),  ppgk(k) = w(k) ppuv(k) + (1 - w(k)) ppuv(k-1)
// and likewise in j.  Its transpose, written as gathers (no atomics), for ybar = (uoutb, voutb):
//   uinb = uoutb, utensb = dt uoutb (and v), and with au = -dt qx uoutb, av = -dt qy voutb,
//   cb(i,j,k)  = au(i) gx(i) + au(i-1) gx(i-1) + av(j) gy(j) + av(j-1) gy(j-1)     (ppgc adjoint)
//   kb(k)      = cb(k-1) - cb(k)                                                   (ppgk adjoint)
//   ppuvb(k)   = w(k) kb(k) + (1 - w(k+1)) kb(k+1) + au(i-1) - au(i) + av(j-1) - av(j)
// with every coefficient zero off the interior.  ppuvb covers i in [0,N], j in [0,N],
// k in [-1,N_z] (the reach of ppuv).  One CTA marches a 32 x 32 tile of that box through a
// chunk of k-levels, keeping cb at three levels in registers.
// The adjoint's coefficients at every interior point, once (pass 1): au = -dt qx uoutb and
// au gx, av = -dt qy voutb and av gy (each division once; the g-weighted term is 0 where a
// is).  The march (pass 2) reads them at the kb + 2 levels of its k-block instead of
// recomputing them there.
template <class T>
struct FastwavesAdjTerms {
  T *au, *ax, *av, *ay;  // in the layout of the state fields, 0 outside the interior unread
};

// What the terms are formed from, for a march that forms them itself (FP32: see
// fastwavesuv_adj_kernel).
template <class T>
struct FastwavesAdjState {
  const T *hhl, *rho, *fx;
  int64_t s1d;
  T ed2;
};

// The coefficients au = -dt qx uoutb and au gx at interior point o (fastwavesuv_adj_terms_kernel's
// expressions), and av, av gy with dir = sj.
template <class T, bool U>
__device__ __forceinline__ T fastwaves_adj_coef(const FastwavesAdjState<T>& st, const T* __restrict__ yb, int64_t o,
                                                int j, int64_t sj, int64_t sk, T dt, T* ag) {
  const int64_t s = U ? 1 : sj;
  const T q = U ? (T(2.0) * ld(st.fx + (int64_t)j * st.s1d)) / (ld(st.rho + o + 1) + ld(st.rho + o))
                : st.ed2 / (ld(st.rho + o + sj) + ld(st.rho + o));
  const T a = -(dt * q) * ld(yb + o);
  T g = T(0);
  if (a != T(0)) {
    const T hs0 = ld(st.hhl + o + sk) + ld(st.hhl + o), hs1 = ld(st.hhl + o + s + sk) + ld(st.hhl + o + s);
    const T hd0 = ld(st.hhl + o + sk) - ld(st.hhl + o), hd1 = ld(st.hhl + o + s + sk) - ld(st.hhl + o + s);
    g = a * ((T(0.5) * (hs0 - hs1)) / (hd0 + hd1));
  }
  *ag = g;
  return a;
}

template <class T>
struct fastwavesuv_adj_terms_kernel {
  static constexpr int kStepOp = step_op<T>(kOpFwsAdjTerms);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, FastwavesAdjTerms<T> tm, FastwavesAdjState<T> st,
                                             const T* __restrict__ uoutb, const T* __restrict__ voutb, T dt, Dims d,
                                             int kb) {
    const int64_t sk = d.sk, sj = d.sj;
    for_box<RowUnroll<T>::value>(blk, d, 0, 0, d.nx, d.ny, kb, [&](int64_t o, int, int j) {
      tm.au[o] = fastwaves_adj_coef<T, true>(st, uoutb, o, j, sj, sk, dt, &tm.ax[o]);
      tm.av[o] = fastwaves_adj_coef<T, false>(st, voutb, o, j, sj, sk, dt, &tm.ay[o]);
    });
  }
};

template <class T>
struct FastwavesAdjSmem {
  T ax[kT][kR];  // au(i0-1+a, j0+b) gx, then au itself in the second half
  T au[kT][kR];
  T ay[kR][kT];  // av(i0+a, j0-1+b) gy
  T av[kR][kT];
};

// FUSED (1): the march forms au, au gx, av, av gy itself at each level it reads (the FP32 form:
// its divisions are cheap, and the 16 bytes a point the terms pass writes and the march reads
// back cost more), from `st`, with the terms pass's expressions; else it reads them from tm.
template <class T, int FUSED = 0>
struct fastwavesuv_adj_kernel {
  static constexpr int kStepOp = step_op<T>(FUSED ? kOpFwsAdjFused : kOpFwsAdj);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uinb, T* __restrict__ vinb,
                                             T* __restrict__ utensb, T* __restrict__ vtensb, T* __restrict__ ppuvb,
                                             const T* __restrict__ wgtfac, FastwavesAdjTerms<T> tm,
                                             FastwavesAdjState<T> st, const T* __restrict__ uoutb,
                                             const T* __restrict__ voutb, T dt, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FastwavesAdjSmem<T>& s = *reinterpret_cast<FastwavesAdjSmem<T>*>(smem_raw);
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int sj = (int)d.sj;
    const int64_t sk = d.sk;
    // output levels K in [Ks, Ke) of the extended range [-1, nz+1)
    const int Ks = -1 + (int)blk.z * kb, Ke = min(Ks + kb, d.nz + 1);
    constexpr int kPts = kT * kT / kThreads;
    T cm2[kPts], cm1[kPts], dir[kPts];  // cb(L-2), cb(L-1), direct terms of level L-1
    // outputs of this tile in the box [0, nx] x [0, ny]: a tile at its far edge holds one
    // column or row of them, and computes au / av only where those outputs read them (the
    // march below reads no other cell for an output it writes)
    const int vx = min(kT, d.nx + 1 - i0), vy = min(kT, d.ny + 1 - j0);
  #pragma unroll
    for (int t = 0; t < kPts; ++t) cm2[t] = cm1[t] = dir[t] = T(0);
    const int tid = threadIdx.y * kTX + threadIdx.x;
    // adjoint of ppgu (au) and of ppgv (av) at an interior point, and the same times g (pass 1)
    auto au_at = [&](int i, int j, int k, T* ag) -> T {
      if (i < 0 || i >= d.nx || j < 0 || j >= d.ny || k < 0 || k >= d.nz) {
        *ag = T(0);
        return T(0);
      }
      const int64_t o = (int64_t)k * sk + i + j * sj;
      if constexpr (FUSED) return fastwaves_adj_coef<T, true>(st, uoutb, o, j, sj, sk, dt, ag);
      *ag = ld(tm.ax + o);
      return ld(tm.au + o);
    };
    auto av_at = [&](int i, int j, int k, T* ag) -> T {
      if (i < 0 || i >= d.nx || j < 0 || j >= d.ny || k < 0 || k >= d.nz) {
        *ag = T(0);
        return T(0);
      }
      const int64_t o = (int64_t)k * sk + i + j * sj;
      if constexpr (FUSED) return fastwaves_adj_coef<T, false>(st, voutb, o, j, sj, sk, dt, ag);
      *ag = ld(tm.ay + o);
      return ld(tm.av + o);
    };
  #pragma unroll 1
    for (int L = Ks - 1; L <= Ke; ++L) {
      // au, av and their g-weighted versions at level L over the tile plus the low apron
      for_region_lim<kR, kT>(vx + 1, vy, [&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 + b;
        s.au[b][a] = au_at(i, j, L, &s.ax[b][a]);
      });
      for_region_lim<kT, kR>(vx, vy + 1, [&](int a, int b) {
        const int i = i0 + a, j = j0 - 1 + b;
        s.av[b][a] = av_at(i, j, L, &s.ay[b][a]);
      });
      __syncthreads();
  #pragma unroll
      for (int t = 0; t < kPts; ++t) {
        const int e = tid + t * kThreads;
        const int b = e / kT, a = e - b * kT;
        const int i = i0 + a, j = j0 + b;
        // cb(L) at (i, j): ppgc(i) feeds ppgu(i), ppgu(i-1), ppgv(j), ppgv(j-1)
        const T cl = (L >= 0 && L < d.nz) ? ((s.ax[b][a + 1] + s.ax[b][a]) + (s.ay[b + 1][a] + s.ay[b][a])) : T(0);
        const int K = L - 1;  // output level
        if (K >= Ks && K < Ke && i <= d.nx && j <= d.ny) {
          const int64_t o = (int64_t)K * sk + i + j * sj;
          const T kbK = cm2[t] - cm1[t];  // kb(K)   = cb(K-1) - cb(K)
          const T kbK1 = cm1[t] - cl;     // kb(K+1) = cb(K)   - cb(K+1)
          T acc = dir[t];
          if (K >= 0) acc = acc + ld(wgtfac + o) * kbK;
          if (K + 1 <= d.nz) acc = acc + (T(1.0) - ld(wgtfac + o + sk)) * kbK1;
          ppuvb[o] = acc;
          if (K >= 0 && K < d.nz && i < d.nx && j < d.ny) {
            const T ub = ld(uoutb + o), vb = ld(voutb + o);
            uinb[o] = ub;
            vinb[o] = vb;
            utensb[o] = dt * ub;
            vtensb[o] = dt * vb;
          }
        }
        // direct terms of level L: au(i-1) - au(i) + av(j-1) - av(j)
        dir[t] = (s.au[b][a] - s.au[b][a + 1]) + (s.av[b][a] - s.av[b + 1][a]);
        cm2[t] = cm1[t];
        cm1[t] = cl;
      }
      __syncthreads();
    }
  }
};

template <class T, class M3, class M1>
oeb_status fastwavesuv_adj_entry(const M3* uinb, const M3* vinb, const M3* utensb, const M3* vtensb,
                                 const M3* ppuvb, const M3* uin, const M3* vin, const M3* utens, const M3* vtens,
                                 const M3* wgtfac, const M3* ppuv, const M3* hhl, const M3* rho, const M1* fx,
                                 const M3* uoutb, const M3* voutb, T edadlat, T dt, const oeb_domain* dom,
                                 void* stream) {
  {
    // the state as the forward sees it, with the adjoint seeds in the outputs' places
    ValidateOnly guard;
    OEB_TRY(fastwavesuv_entry<T>(uoutb, voutb, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, edadlat, dt, dom,
                                 stream));
  }
  OEB_TRY(check_domain(dom));
  Grid<T> gub, gvb, gutb, gvtb, gpb, gw, gh, gr, guo, gvo;
  Line<T> lfx;
  OEB_TRY((check_field3<T>(uinb, *dom, kInterior, &gub)));
  OEB_TRY((check_field3<T>(vinb, *dom, kInterior, &gvb)));
  OEB_TRY((check_field3<T>(utensb, *dom, kInterior, &gutb)));
  OEB_TRY((check_field3<T>(vtensb, *dom, kInterior, &gvtb)));
  OEB_TRY((check_field3<T>(ppuvb, *dom, Reach{0, 1, 0, 1, 1, 1}, &gpb)));
  OEB_TRY((check_field3<T>(wgtfac, *dom, Reach{0, 1, 0, 1, 0, 1}, &gw)));
  OEB_TRY((check_field3<T>(hhl, *dom, Reach{0, 1, 0, 1, 0, 1}, &gh)));
  OEB_TRY((check_field3<T>(rho, *dom, Reach{0, 1, 0, 1, 0, 0}, &gr)));
  OEB_TRY((check_field3<T>(uoutb, *dom, kInterior, &guo)));
  OEB_TRY((check_field3<T>(voutb, *dom, kInterior, &gvo)));
  OEB_TRY((check_field1<T>(fx, *dom, 0, 0, &lfx)));
  OEB_TRY(check_same_strides<T>({&gub, &gvb, &gutb, &gvtb, &gpb, &gw, &gh, &gr, &guo, &gvo}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi, gutb.lo, gutb.hi, gvtb.lo, gvtb.hi, gpb.lo, gpb.hi},
                         {gw.lo, gw.hi, gh.lo, gh.hi, gr.lo, gr.hi, guo.lo, guo.hi, gvo.lo, gvo.hi, lfx.lo, lfx.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gw.sj, gw.sk};
  const T ed2 = T(2.0) * edadlat;
  cudaStream_t st = (cudaStream_t)stream;
  const FastwavesAdjState<T> state{gh.origin, gr.origin, lfx.origin, lfx.s, ed2};
  if constexpr (std::is_same<T, float>::value) if (adjoint_tiles()) {
    // one launch: the march forms the coefficients at the kb + 2 levels of its k-block
    const int kb = tuned_kb(kAdjFusedKB);
    return launch<fastwavesuv_adj_kernel<T, 1>>(tile_grid(d.nx + 1, d.ny + 1, d.nz + 2, kT, kT, kb),
                                                   sizeof(FastwavesAdjSmem<T>), st, gub.origin, gvb.origin,
                                                   gutb.origin, gvtb.origin, gpb.origin, gw.origin,
                                                   FastwavesAdjTerms<T>{}, state, guo.origin, gvo.origin, dt, d, kb);
  }
  // scratch for the four coefficient fields, in uoutb's layout
  const T* start = (uoutb->allocated && uoutb->allocated <= uoutb->aligned) ? uoutb->allocated : uoutb->aligned;
  const int64_t last = (uoutb->sizes[0] - 1) * uoutb->strides[0] + (uoutb->sizes[1] - 1) * uoutb->strides[1] +
                       (uoutb->sizes[2] - 1) * uoutb->strides[2];
  const int64_t n = (int64_t)(uoutb->aligned - start) + last + 1;
  const int64_t org = (int64_t)(uoutb->aligned - start) + uoutb->offset;
  void* buf = nullptr;
  OEB_TRY(scratch_alloc(&buf, (size_t)n * 4 * sizeof(T), st));
  T* base = static_cast<T*>(buf);
  const FastwavesAdjTerms<T> tm{base + org, base + n + org, base + 2 * n + org, base + 3 * n + org};
  oeb_status stt = launch<fastwavesuv_adj_terms_kernel<T>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, 1), 0, st, tm, state,
                                                           guo.origin, gvo.origin, dt, d, 1);
  // the march carries a three-level window of ppgc terms up the column; a k-block of kb
  // levels reads the coefficients at kb + 2
  const int kb = tuned_kb(adj_kb<T>());
  if (stt == OEB_OK)
    stt = launch<fastwavesuv_adj_kernel<T>>(tile_grid(d.nx + 1, d.ny + 1, d.nz + 2, kT, kT, kb),
                                            sizeof(FastwavesAdjSmem<T>), st, gub.origin, gvb.origin, gutb.origin,
                                            gvtb.origin, gpb.origin, gw.origin, tm, state, guo.origin, gvo.origin, dt,
                                            d, kb);
  scratch_free(buf, st);
  return stt;
}

}  // namespace
}  // namespace oeb

#ifndef OEB_BODIES_ONLY  // the entry points

using namespace oeb;

#define OEB_FW_ENTRY(S, T)                                                                                          \
  extern "C" oeb_status oeb_fastwavesuv_##S(                                                                       \
      const oeb_memref3d_##S* uout, const oeb_memref3d_##S* vout, const oeb_memref3d_##S* uin,                      \
      const oeb_memref3d_##S* vin, const oeb_memref3d_##S* utens, const oeb_memref3d_##S* vtens,                    \
      const oeb_memref3d_##S* wgtfac, const oeb_memref3d_##S* ppuv, const oeb_memref3d_##S* hhl,                    \
      const oeb_memref3d_##S* rho, const oeb_memref1d_##S* fx, T edadlat, T dt, const oeb_domain* dom,             \
      void* stream) {                                                                                              \
    return fastwavesuv_entry<T>(uout, vout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, edadlat, dt, dom,  \
                                stream);                                                                           \
  }                                                                                                                \
  extern "C" oeb_status oeb_fastwavesuv_tl_##S(                                                                    \
      const oeb_memref3d_##S* duout, const oeb_memref3d_##S* dvout, const oeb_memref3d_##S* uin,                    \
      const oeb_memref3d_##S* vin, const oeb_memref3d_##S* utens, const oeb_memref3d_##S* vtens,                    \
      const oeb_memref3d_##S* wgtfac, const oeb_memref3d_##S* ppuv, const oeb_memref3d_##S* hhl,                    \
      const oeb_memref3d_##S* rho, const oeb_memref1d_##S* fx, const oeb_memref3d_##S* duin,                        \
      const oeb_memref3d_##S* dvin, const oeb_memref3d_##S* dutens, const oeb_memref3d_##S* dvtens,                 \
      const oeb_memref3d_##S* dppuv, T edadlat, T dt, const oeb_domain* dom, void* stream) {                        \
    return fastwavesuv_tl_entry<T>(duout, dvout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx, duin, dvin,    \
                                   dutens, dvtens, dppuv, edadlat, dt, dom, stream);                               \
  }                                                                                                                \
  extern "C" oeb_status oeb_fastwavesuv_adj_##S(                                                                   \
      const oeb_memref3d_##S* uinb, const oeb_memref3d_##S* vinb, const oeb_memref3d_##S* utensb,                   \
      const oeb_memref3d_##S* vtensb, const oeb_memref3d_##S* ppuvb, const oeb_memref3d_##S* uin,                   \
      const oeb_memref3d_##S* vin, const oeb_memref3d_##S* utens, const oeb_memref3d_##S* vtens,                    \
      const oeb_memref3d_##S* wgtfac, const oeb_memref3d_##S* ppuv, const oeb_memref3d_##S* hhl,                    \
      const oeb_memref3d_##S* rho, const oeb_memref1d_##S* fx, const oeb_memref3d_##S* uoutb,                       \
      const oeb_memref3d_##S* voutb, T edadlat, T dt, const oeb_domain* dom, void* stream) {                        \
    return fastwavesuv_adj_entry<T>(uinb, vinb, utensb, vtensb, ppuvb, uin, vin, utens, vtens, wgtfac, ppuv, hhl,   \
                                    rho, fx, uoutb, voutb, edadlat, dt, dom, stream);                              \
  }

OEB_FW_ENTRY(f64, double)
OEB_FW_ENTRY(f32, float)

#endif  // OEB_BODIES_ONLY
