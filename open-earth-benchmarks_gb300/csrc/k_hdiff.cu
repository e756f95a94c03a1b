// k_hdiff.cu -- horizontal diffusion stencils whose intermediates are shared by neighbouring
// points: hdiffsa (kernels/hdiffsa.h:95-123) and hdiffsmag (kernels/hdiffsmag.h:205-263), in
// FP64 (bit-identical to the reference) and FP32 (hdiffsa with exact limiter sign tests;
// hdiffsmag the reference's float sequence, bit-identical to the reference compiled for
// float; precision.cuh).
//
// The reference's OpenMP variants recompute each intermediate for every point that uses it
// (three laplacians per point in hdiffsa, three T^2 and three S^2 per point in hdiffsmag).
// On GB300 the FP64 pipe, not HBM, bounds these kernels, so here every intermediate is
// computed once per (i, j, k) into a shared-memory tile (plus a one- or two-cell apron) and
// read by its neighbours.  Reusing a value is exact: it is the same expression on the same
// operands.  Differences are stored once and their negations used where the reference
// subtracts in the other order (x - y == -(y - x) exactly in IEEE round-to-nearest).
//
// Compiled with --fmad=false (see k_pointwise.cu).  One CTA of 32 x 8 threads per
// 32 x 32 tile and kb k-levels.
#include <mutex>
#include <type_traits>
#include <vector>

#include "precision.cuh"
#include "stage.cuh"
#include "stencil_util.cuh"
#include "tangent.cuh"

// Built on its own, this file's bodies and helpers are local to it; the step kernel
// (step.cu) includes it with OEB_BODIES_ONLY and a namespace of its own instead.
#ifndef OEB_BODIES_NS
#define OEB_BODIES_NS
#endif
namespace oeb {
namespace OEB_BODIES_NS {

constexpr int kT = 32;  // tile edge

// ============================== hdiffsa ===========================================
// Shared layout (per k-level), tile origin (i0, j0):
//   in  : 36 x 36, (i0-2+a, j0-2+b)
//   dy  : 34 x 35, (i0-1+a, j0-2+b)   dy(i,j)  = in(i,j+1) - in(i,j)
//   lap : 34 x 34, (i0-1+a, j0-1+b)
//   flx : 33 x 32, (i0-1+a, j0+b)
//   fly : 32 x 33, (i0+a,   j0-1+b)
template <class T>
struct HdiffsaSmem {
  T in[36][36];
  T dy[35][34];
  T lap[34][34];
  T flx[32][33];
  T fly[33][32];
  T crlato[34];  // j0-1+b
  T crlatu[34];
};

template <class T>
struct hdiffsa_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ out, const T* __restrict__ in,
                                             const T* __restrict__ mask, const T* __restrict__ crlato,
                                             const T* __restrict__ crlatu, int64_t s1d, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HdiffsaSmem<T>& s = *reinterpret_cast<HdiffsaSmem<T>*>(smem_raw);
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int sj = (int)d.sj;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    if (tid < 34) {
      const int j = j0 - 1 + tid;
      const bool ok = j >= -1 && j < d.ny + 1;
      s.crlato[tid] = ok ? ld(crlato + (int64_t)j * s1d) : T(0);
      s.crlatu[tid] = ok ? ld(crlatu + (int64_t)j * s1d) : T(0);
    }
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
    // outputs of this tile (fewer at the domain's far edge) and what each phase needs for them
    const int vx = max(0, min(kT, d.nx - i0)), vy = max(0, min(kT, d.ny - j0));
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      const T* pin = in + kofs;
      for_region_lim<36, 36>(vx + 4, vy + 4, [&](int a, int b) {
        const int i = i0 - 2 + a, j = j0 - 2 + b;
        const bool ok = i >= -2 && i < d.nx + 2 && j >= -2 && j < d.ny + 2;
        s.in[b][a] = ok ? ld(pin + i + j * sj) : T(0);
      });
      __syncthreads();
      for_region_lim<34, 35>(vx + 2, vy + 3, [&](int a, int b) { s.dy[b][a] = isub(s.in[b + 1][a + 1], s.in[b][a + 1]); });
      __syncthreads();
      // hdiffsa.h:101: in(i-1)+in(i+1) - 2 in + crlato (in(j+1)-in) + crlatu (in(j-1)-in)
      for_region_lim<34, 34>(vx + 2, vy + 2, [&](int a, int b) {
        const T c = s.in[b + 1][a + 1];
        s.lap[b][a] = ((iadd(s.in[b + 1][a], s.in[b + 1][a + 2]) - scale2<1>(c)) + s.crlato[b] * s.dy[b + 1][a]) +
                      s.crlatu[b] * (-s.dy[b][a]);
      });
      __syncthreads();
      // hdiffsa.h:106-113: limited fluxes
      for_region_lim<33, 32>(vx + 1, vy, [&](int a, int b) {
        T f = s.lap[b + 1][a + 1] - s.lap[b + 1][a];
        if (Prec<T>::prod_gt0(f, s.in[b + 2][a + 2] - s.in[b + 2][a + 1])) f = 0;
        s.flx[b][a] = f;
      });
      for_region_lim<32, 33>(vx, vy + 1, [&](int a, int b) {
        T f = s.crlato[b] * (s.lap[b + 1][a + 1] - s.lap[b][a + 1]);
        if (Prec<T>::prod_gt0(f, s.dy[b + 1][a + 1])) f = 0;
        s.fly[b][a] = f;
      });
      __syncthreads();
      // hdiffsa.h:118-119
      for_region<32, 32>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        if (i < d.nx && j < d.ny) {
          const int64_t o = kofs + i + j * sj;
          out[o] = s.in[b + 2][a + 2] + (((s.flx[b][a] - s.flx[b][a + 1]) + s.fly[b][a]) - s.fly[b + 1][a]) * ld(mask + o);
        }
      });
      __syncthreads();
    }
  }
};

// FP32 hdiffsa.  In FP32 the kernel above is bound by instruction issue, not by HBM (ncu at
// 256 x 256 x 80: 72 % issue active, "not selected" the top stall, 13 % of DRAM throughput):
// five shared-memory phases a level, each with its own index arithmetic.  Here a level takes
// two: the laplacian on its 34 x 34 box straight from the `in` tile (the differences
// in(j+1) - in and in(j-1) - in formed where they are used; the kernel above stores
// in(j+1) - in once and negates it, which gives the same bits), then each output forms the
// four limited fluxes it reads (each flux is formed by the two outputs beside it, with the
// same operations on the same operands).  The k-levels are marched: the `in` tile of level
// k+1 is copied by cp.async into a second buffer while level k is computed.  Results are
// hdiffsa_kernel<float>'s, bit for bit.  kb from staged_kb: about one wave of CTAs.
// Measured alone (back-to-back launches): 256 x 256 x 80 41.3 -> 38.6 us, 128 x 128 x 80
// 14.5 -> 12.7 us; 20 % fewer warp instructions (35.7 M -> 28.7 M a launch), still 67 % issue
// active.  The marching alone, with the five phases, measured 41.2 us: the kernel waits on
// its instructions, not on its loads.
struct hdiffsa_f32 {
  static constexpr int kCtasPerSm = 6;  // by registers (40)
  struct Smem {
    float in[2][36][36];  // (i0-2+a, j0-2+b)
    float lap[34][34];    // (i0-1+a, j0-1+b)
    float crlato[34], crlatu[34];  // j0-1+b
  };
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ out, const float* __restrict__ in,
                                             const float* __restrict__ mask, const float* __restrict__ crlato,
                                             const float* __restrict__ crlatu, int64_t s1d, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int sj = (int)d.sj;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    if (tid < 34) {
      const int j = j0 - 1 + tid;
      const bool ok = j >= -1 && j < d.ny + 1;
      s.crlato[tid] = ok ? ld(crlato + (int64_t)j * s1d) : 0.f;
      s.crlatu[tid] = ok ? ld(crlatu + (int64_t)j * s1d) : 0.f;
    }
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
    const int vx = max(0, min(kT, d.nx - i0)), vy = max(0, min(kT, d.ny - j0));
    auto issue = [&](int k, float (*t)[36]) {
      if (k < k1) {
        const float* pin = in + (int64_t)k * d.sk;
        for_region_lim<36, 36>(vx + 4, vy + 4, [&](int a, int b) {
          const int i = i0 - 2 + a, j = j0 - 2 + b;
          const bool ok = i >= -2 && i < d.nx + 2 && j >= -2 && j < d.ny + 2;
          cp_async4(&t[b][a], ok ? pin + i + j * sj : pin, ok);
        });
      }
      cp_async_commit();
    };
    issue(k0, s.in[0]);
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int cur = (k - k0) & 1;
      issue(k + 1, s.in[cur ^ 1]);  // the buffer level k-1 left
      const int64_t kofs = (int64_t)k * d.sk;
      cp_async_wait<1>();  // level k has landed
      __syncthreads();
      const float(*t)[36] = s.in[cur];
      // hdiffsa.h:101: in(i-1)+in(i+1) - 2 in + crlato (in(j+1)-in) + crlatu (in(j-1)-in)
      for_region_lim<34, 34>(vx + 2, vy + 2, [&](int a, int b) {
        const float c = t[b + 1][a + 1];
        s.lap[b][a] = (((t[b + 1][a] + t[b + 1][a + 2]) - 2.f * c) + s.crlato[b] * (t[b + 2][a + 1] - c)) +
                      s.crlatu[b] * (t[b][a + 1] - c);
      });
      __syncthreads();
      // hdiffsa.h:106-113 (limited fluxes) and :118-119 (the update)
      const int a = threadIdx.x;
#pragma unroll
      for (int r = 0; r < kT / kTY; ++r) {
        const int b = threadIdx.y + kTY * r;
        if (a < vx && b < vy) {
          const float lc = s.lap[b + 1][a + 1];
          const float ic = t[b + 2][a + 2];
          float fxw = lc - s.lap[b + 1][a];
          if (Prec<float>::prod_gt0(fxw, ic - t[b + 2][a + 1])) fxw = 0.f;
          float fxe = s.lap[b + 1][a + 2] - lc;
          if (Prec<float>::prod_gt0(fxe, t[b + 2][a + 3] - ic)) fxe = 0.f;
          float fys = s.crlato[b] * (lc - s.lap[b][a + 1]);
          if (Prec<float>::prod_gt0(fys, ic - t[b + 1][a + 2])) fys = 0.f;
          float fyn = s.crlato[b + 1] * (s.lap[b + 2][a + 1] - lc);
          if (Prec<float>::prod_gt0(fyn, t[b + 3][a + 2] - ic)) fyn = 0.f;
          const int64_t o = kofs + (i0 + a) + (int64_t)(j0 + b) * sj;
          out[o] = ic + (((fxw - fxe) + fys) - fyn) * ld(mask + o);
        }
      }
      __syncthreads();
    }
  }
};

// ============================== hdiffsmag =========================================
// Shared layout (per k-level), tile origin (i0, j0):
//   u, v : 34 x 34, (i0-1+a, j0-1+b)
//   dyv  : 33 x 33, (i0+a,   j0-1+b)   v(i,j+1) - v(i,j)
//   dyu  : 33 x 33, (i0-1+a, j0-1+b)   u(i,j+1) - u(i,j)
// (the x differences dxu = u(i+1,j) - u(i,j) at (i0-1+a, j0+b) and dxv = v(i+1,j) - v(i,j)
// at (i0-1+a, j0-1+b) are each read once, by the deformations of the same cell: they live in
// registers, which keeps the tile at 53 KB, four CTAs per SM)
//   tsq  : 33 x 33, (i0+a,   j0+b)     T_s^2
//   ssq  : 33 x 33, (i0-1+a, j0-1+b)   S_uv^2
template <class T>
struct HdiffsmagSmem {
  T u[34][34];
  T v[34][34];
  T dyv[33][33];
  T dyu[33][33];
  T tsq[33][33];
  T ssq[33][33];
  T acrlat0[34];  // j0-1+b
  T crlato[32], crlatu[32], crlavo[32], crlavu[32];
};

template <class T>
struct hdiffsmag_kernel {
  static constexpr int kStepOp = step_op<T>(kOpSmagFwd);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uout, T* __restrict__ vout,
                                             const T* __restrict__ uin, const T* __restrict__ vin,
                                             const T* __restrict__ mask, const T* __restrict__ crlavo,
                                             const T* __restrict__ crlavu, const T* __restrict__ crlato,
                                             const T* __restrict__ crlatu, const T* __restrict__ acrlat0, int64_t s1d,
                                             T eddlat, T eddlon, T tau_smag, T weight_smag, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HdiffsmagSmem<T>& s = *reinterpret_cast<HdiffsmagSmem<T>*>(smem_raw);
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int sj = (int)d.sj;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    constexpr T rr = earth_radius_recip<T>();
    if (tid < 34) {
      const int j = j0 - 1 + tid;
      s.acrlat0[tid] = (j >= -1 && j < d.ny + 1) ? ld(acrlat0 + (int64_t)j * s1d) : T(0);
    } else if (tid >= 64 && tid < 96) {
      const int b = tid - 64, j = j0 + b;
      const bool ok = j < d.ny;
      const int64_t jo = (int64_t)j * s1d;
      s.crlato[b] = ok ? ld(crlato + jo) : T(0);
      s.crlatu[b] = ok ? ld(crlatu + jo) : T(0);
      s.crlavo[b] = ok ? ld(crlavo + jo) : T(0);
      s.crlavu[b] = ok ? ld(crlavu + jo) : T(0);
    }
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
    // outputs of this tile (fewer at the domain's far edge) and what each phase needs for them
    const int vx = max(0, min(kT, d.nx - i0)), vy = max(0, min(kT, d.ny - j0));
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      for_region_lim<34, 34>(vx + 2, vy + 2, [&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 - 1 + b;
        const bool ok = i >= -1 && i < d.nx + 1 && j >= -1 && j < d.ny + 1;
        const int64_t o = kofs + i + j * sj;
        s.u[b][a] = ok ? ld(uin + o) : T(0);
        s.v[b][a] = ok ? ld(vin + o) : T(0);
      });
      __syncthreads();
      // hdiffsmag.h:213 T_s = (v(j-1)-v) eddlat R^-1 - (u(i-1)-u) acrlat0(j) eddlon
      //              :221 S_uv = (u(j+1)-u) eddlat R^-1 + (v(i+1)-v) acrlat0(j) eddlon
      for_region_lim<33, 33>(vx + 1, vy + 1, [&](int a, int b) {
        const T dxu = s.u[b + 1][a + 1] - s.u[b + 1][a];
        const T dyv = s.v[b + 1][a + 1] - s.v[b][a + 1];
        const T dyu = s.u[b + 1][a] - s.u[b][a];
        const T dxv = s.v[b][a + 1] - s.v[b][a];
        s.dyv[b][a] = dyv;
        s.dyu[b][a] = dyu;
        const T ts = ((-dyv) * eddlat) * rr - ((-dxu) * s.acrlat0[b + 1]) * eddlon;
        s.tsq[b][a] = ts * ts;
        const T su = (dyu * eddlat) * rr + (dxv * s.acrlat0[b]) * eddlon;
        s.ssq[b][a] = su * su;
      });
      __syncthreads();
      for_region<32, 32>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        if (i < d.nx && j < d.ny) {
          const int64_t o = kofs + i + j * sj;
          const T hdweight = weight_smag * ld(mask + o);
          // hdiffsmag.h:233-244 (the T^2 pair sums as integer-pipe additions: the FP64 pipe is the
          // busier one here; two per point measured best, four 6 % slower)
          T smag_u = tau_smag * Prec<T>::sqrt_(scale2<-1>(iadd(s.tsq[b][a + 1], s.tsq[b][a])) +
                                               scale2<-1>(s.ssq[b][a + 1] + s.ssq[b + 1][a + 1])) -
                     hdweight;
          smag_u = clamp_smag(smag_u);
          const T uc = s.u[b + 1][a + 1];
          // u(i+1) + u(i-1) - 2u + crlato (u(j+1) - u) + crlatu (u(j-1) - u), the reference's
          // sum in every precision: FP32 is then bit-identical to the reference compiled for
          // float.  A compensated FP32 sum (TwoSum / TwoProduct) measured the same largest error
          // against the FP64 oracle (5.5e-8) at about five times the sum's operations.
          Acc<T> lu(s.u[b + 1][a + 2]);
          lu.add(s.u[b + 1][a]);
          lu.add(-scale2<1>(uc));
          lu.add_prod(s.crlato[b], s.dyu[b + 1][a + 1]);
          lu.add_prod(s.crlatu[b], -s.dyu[b][a + 1]);
          uout[o] = uc + smag_u * lu.get();
          // hdiffsmag.h:248-259
          T smag_v = tau_smag * Prec<T>::sqrt_(scale2<-1>(iadd(s.tsq[b + 1][a], s.tsq[b][a])) +
                                               scale2<-1>(s.ssq[b + 1][a] + s.ssq[b + 1][a + 1])) -
                     hdweight;
          smag_v = clamp_smag(smag_v);
          const T vc = s.v[b + 1][a + 1];
          Acc<T> lv(s.v[b + 1][a + 2]);
          lv.add(s.v[b + 1][a]);
          lv.add(-scale2<1>(vc));
          lv.add_prod(s.crlavo[b], s.dyv[b + 1][a]);
          lv.add_prod(s.crlavu[b], -s.dyv[b][a]);
          vout[o] = vc + smag_v * lv.get();
        }
      });
      __syncthreads();
    }
  }
};

constexpr int kKB = 1;  // k-levels per CTA by default (the most CTAs hide latency best)

template <class T, class M3, class M1>
oeb_status hdiffsa_entry(const M3* out, const M3* in, const M3* mask, const M1* crlato, const M1* crlatu,
                         const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gout, gin, gmask;
  Line<T> lo, lu;
  OEB_TRY((check_field3<T>(out, *dom, kInterior, &gout)));
  OEB_TRY((check_field3<T>(in, *dom, Reach{2, 2, 2, 2, 0, 0}, &gin)));
  OEB_TRY((check_field3<T>(mask, *dom, kInterior, &gmask)));
  OEB_TRY((check_field1<T>(crlato, *dom, 1, 1, &lo)));
  OEB_TRY((check_field1<T>(crlatu, *dom, 1, 1, &lu)));
  if (lo.s != lu.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<T>({&gout, &gin, &gmask}));
  OEB_TRY(check_no_alias({gout.lo, gout.hi}, {gin.lo, gin.hi, gmask.lo, gmask.hi, lo.lo, lo.hi, lu.lo, lu.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gin.sj, gin.sk};
  if constexpr (std::is_same<T, float>::value) if (!fields_in_host_memory()) {
    const int tiles = ((d.nx + kT - 1) / kT) * ((d.ny + kT - 1) / kT);
    const int kb = tuned_kb(staged_kb(tiles, d.nz, hdiffsa_f32::kCtasPerSm));
    return launch<hdiffsa_f32>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(hdiffsa_f32::Smem), (cudaStream_t)stream,
                               gout.origin, gin.origin, gmask.origin, lo.origin, lu.origin, lo.s, d, kb);
  }
  const int kb = tuned_kb(kKB);
  return launch<hdiffsa_kernel<T>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(HdiffsaSmem<T>), (cudaStream_t)stream,
                                   gout.origin, gin.origin, gmask.origin, lo.origin, lu.origin, lo.s, d, kb);
}

template <class T, class M3, class M1>
oeb_status hdiffsmag_entry(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* mask,
                           const M1* crlavo, const M1* crlavu, const M1* crlato, const M1* crlatu, const M1* acrlat0,
                           T eddlat, T eddlon, T tau_smag, T weight_smag, const oeb_domain* dom, void* stream) {
  OEB_TRY(check_domain(dom));
  Grid<T> gu, gv, gui, gvi, gm;
  Line<T> lvo, lvu, lto, ltu, la0;
  OEB_TRY((check_field3<T>(uout, *dom, kInterior, &gu)));
  OEB_TRY((check_field3<T>(vout, *dom, kInterior, &gv)));
  OEB_TRY((check_field3<T>(uin, *dom, Reach{1, 1, 1, 1, 0, 0}, &gui)));
  OEB_TRY((check_field3<T>(vin, *dom, Reach{1, 1, 1, 1, 0, 0}, &gvi)));
  OEB_TRY((check_field3<T>(mask, *dom, kInterior, &gm)));
  OEB_TRY((check_field1<T>(crlavo, *dom, 0, 0, &lvo)));
  OEB_TRY((check_field1<T>(crlavu, *dom, 0, 0, &lvu)));
  OEB_TRY((check_field1<T>(crlato, *dom, 0, 0, &lto)));
  OEB_TRY((check_field1<T>(crlatu, *dom, 0, 0, &ltu)));
  OEB_TRY((check_field1<T>(acrlat0, *dom, 1, 1, &la0)));
  if (lvu.s != lvo.s || lto.s != lvo.s || ltu.s != lvo.s || la0.s != lvo.s) return OEB_ERR_LAYOUT;
  OEB_TRY(check_same_strides<T>({&gu, &gv, &gui, &gvi, &gm}));
  OEB_TRY(check_no_alias({gu.lo, gu.hi, gv.lo, gv.hi},
                         {gui.lo, gui.hi, gvi.lo, gvi.hi, gm.lo, gm.hi, lvo.lo, lvo.hi, lvu.lo, lvu.hi, lto.lo,
                          lto.hi, ltu.lo, ltu.hi, la0.lo, la0.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
  const int kb = tuned_kb(kKB);
  return launch<hdiffsmag_kernel<T>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(HdiffsmagSmem<T>),
                                     (cudaStream_t)stream, gu.origin, gv.origin, gui.origin, gvi.origin, gm.origin,
                                     lvo.origin, lvu.origin, lto.origin, ltu.origin, la0.origin, lvo.s, eddlat, eddlon,
                                     tau_smag, weight_smag, d, kb);
}

// Tangent-linear hdiffsmag: d(uout, vout) = J(uin, vin) d(uin, vin), the kernel on Dual<T>.
template <class T, class M3, class M1>
oeb_status hdiffsmag_tl_entry(const M3* duout, const M3* dvout, const M3* uin, const M3* vin, const M3* mask,
                              const M1* crlavo, const M1* crlavu, const M1* crlato, const M1* crlatu,
                              const M1* acrlat0, const M3* duin, const M3* dvin, T eddlat, T eddlon, T tau_smag,
                              T weight_smag, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(hdiffsmag_entry<T>(duout, dvout, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, eddlat, eddlon,
                               tau_smag, weight_smag, dom, stream));
    OEB_TRY(hdiffsmag_entry<T>(duout, dvout, duin, dvin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, eddlat,
                               eddlon, tau_smag, weight_smag, dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *u, *v, *m, *l0, *l1, *l2, *l3, *l4, *ou, *ov;
  OEB_TRY(arr.pack(uin, duin, &u));
  OEB_TRY(arr.pack(vin, dvin, &v));
  OEB_TRY(arr.pack(mask, (const M3*)nullptr, &m));
  OEB_TRY(arr.pack(crlavo, (const M1*)nullptr, &l0));
  OEB_TRY(arr.pack(crlavu, (const M1*)nullptr, &l1));
  OEB_TRY(arr.pack(crlato, (const M1*)nullptr, &l2));
  OEB_TRY(arr.pack(crlatu, (const M1*)nullptr, &l3));
  OEB_TRY(arr.pack(acrlat0, (const M1*)nullptr, &l4));
  OEB_TRY(arr.alloc(duout, &ou));
  OEB_TRY(arr.alloc(dvout, &ov));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, uin->strides[1], uin->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<hdiffsmag_kernel<D>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(HdiffsmagSmem<D>),
                                      (cudaStream_t)stream, ou, ov, u, v, m, l0, l1, l2, l3, l4, crlavo->strides[0],
                                      D(eddlat), D(eddlon), D(tau_smag), D(weight_smag), d, kb));
  OEB_TRY(arr.unpack(duout->aligned + duout->offset, ou, *dom, kInterior, d.sj, d.sk));
  return arr.unpack(dvout->aligned + dvout->offset, ov, *dom, kInterior, d.sj, d.sk);
}

// ============================== hdiffsa: tangent-linear and adjoint ===============
// Linearised at `in` with the flux limiters of hdiffsa.h:106-113 frozen:
//   out = in + mask (flx(i-1) - flx + fly(j-1) - fly),
//   flx = fx (lap(i+1) - lap),  fly = fy crlato(j) (lap(j+1) - lap),
//   fx = 0 where flx (in(i+1) - in) > 0 at the state, else 1 (fy likewise with j),
//   lap = in(i-1) + in(i+1) - 2 in + crlato(j) (in(j+1) - in) + crlatu(j) (in(j-1) - in).
// Active input: in (mask, crlato, crlatu are parameters).  The transpose for outb, with
// G = mask outb on the interior and 0 elsewhere:
//   Fx = fx (G(i+1) - G) on [-1,N) x [0,N),  Fy = fy crlato(j) (G(j+1) - G) on [0,N) x [-1,N),
//   lapb = Fx(i-1) - Fx + Fy(j-1) - Fy,
//   inb = outb (interior) + lapb(i-1) + lapb(i+1) - (2 + crlato(j) + crlatu(j)) lapb
//         + crlato(j-1) lapb(j-1) + crlatu(j+1) lapb(j+1)    on in's reach box [-2, N+2)^2.
// One kernel: a CTA stages its tile's in and G in shared memory, recomputes lap and the limiter
// flags exactly as the forward kernel does (the same operations on the same operands), then
// forms Fx, Fy, lapb and inb in shared memory.  Shared layout (per k-level), inb tile origin
// (i0, j0):
//   in   : 38 x 38, (i0-3+a, j0-3+b)
//   lap  : 36 x 36, (i0-2+a, j0-2+b)
//   gl   : 36 x 36, G at (i0-2+a, j0-2+b); then lapb, 34 x 34 at (i0-1+a, j0-1+b)
//   fx   : 35 x 34, (i0-2+a, j0-1+b);   fy : 34 x 35, (i0-1+a, j0-2+b)
template <class T>
struct HdiffsaAdjSmem {
  T in[38][38];
  T lap[36][36];
  T gl[36][36];
  T fx[34][35];
  T fy[35][34];
  T crlato[38], crlatu[38];  // j0-3+b
};

template <class T>
struct hdiffsa_adj_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ inb, const T* __restrict__ in,
                                             const T* __restrict__ mask, const T* __restrict__ crlato,
                                             const T* __restrict__ crlatu, int64_t s1d, const T* __restrict__ outb,
                                             Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HdiffsaAdjSmem<T>& s = *reinterpret_cast<HdiffsaAdjSmem<T>*>(smem_raw);
    T(*lapb)[34] = reinterpret_cast<T(*)[34]>(&s.gl[0][0]);
    const int i0 = -2 + (int)blk.x * kT, j0 = -2 + (int)blk.y * kT;
    const int64_t sj = d.sj;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    if (tid < 38) {
      const int j = j0 - 3 + tid;
      const bool ok = j >= -1 && j < d.ny + 1;
      s.crlato[tid] = ok ? ld(crlato + (int64_t)j * s1d) : T(0);
      s.crlatu[tid] = ok ? ld(crlatu + (int64_t)j * s1d) : T(0);
    }
    auto interior = [&](int i, int j) { return i >= 0 && i < d.nx && j >= 0 && j < d.ny; };
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      for_region<38, 38>([&](int a, int b) {
        const int i = i0 - 3 + a, j = j0 - 3 + b;
        const bool ok = i >= -2 && i < d.nx + 2 && j >= -2 && j < d.ny + 2;
        s.in[b][a] = ok ? ld(in + kofs + i + j * sj) : T(0);
      });
      for_region<36, 36>([&](int a, int b) {
        const int i = i0 - 2 + a, j = j0 - 2 + b;
        const int64_t o = kofs + i + j * sj;
        s.gl[b][a] = interior(i, j) ? ld(outb + o) * ld(mask + o) : T(0);
      });
      __syncthreads();
      // hdiffsa.h:101 where the forward forms lap (i, j in [-1, N+1)), its operations in its order
      for_region<36, 36>([&](int a, int b) {
        const int i = i0 - 2 + a, j = j0 - 2 + b;
        T v = T(0);
        if (i >= -1 && i < d.nx + 1 && j >= -1 && j < d.ny + 1) {
          const T c = s.in[b + 1][a + 1];
          v = (((s.in[b + 1][a] + s.in[b + 1][a + 2]) - scale2<1>(c)) + s.crlato[b + 1] * (s.in[b + 2][a + 1] - c)) +
              s.crlatu[b + 1] * (s.in[b][a + 1] - c);
        }
        s.lap[b][a] = v;
      });
      __syncthreads();
      // hdiffsa.h:106-109: Fx at (i, j), kept where the forward keeps flx
      for_region<35, 34>([&](int a, int b) {
        const int i = i0 - 2 + a, j = j0 - 1 + b;
        T v = T(0);
        if (i >= -1 && i < d.nx && j >= 0 && j < d.ny) {
          const T f = s.lap[b + 1][a + 1] - s.lap[b + 1][a];
          if (!Prec<T>::prod_gt0(f, s.in[b + 2][a + 2] - s.in[b + 2][a + 1])) v = s.gl[b + 1][a + 1] - s.gl[b + 1][a];
        }
        s.fx[b][a] = v;
      });
      // hdiffsa.h:110-113: Fy at (i, j), crlato(j) folded in
      for_region<34, 35>([&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 - 2 + b;
        T v = T(0);
        if (i >= 0 && i < d.nx && j >= -1 && j < d.ny) {
          const T co = s.crlato[b + 1];
          const T f = co * (s.lap[b + 1][a + 1] - s.lap[b][a + 1]);
          if (!Prec<T>::prod_gt0(f, s.in[b + 2][a + 2] - s.in[b + 1][a + 2])) v = co * (s.gl[b + 1][a + 1] - s.gl[b][a + 1]);
        }
        s.fy[b][a] = v;
      });
      __syncthreads();
      // lapb over the dead G
      for_region<34, 34>([&](int a, int b) { lapb[b][a] = (s.fx[b][a] - s.fx[b][a + 1]) + (s.fy[b][a] - s.fy[b + 1][a]); });
      __syncthreads();
      for_region<32, 32>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        if (i < d.nx + 2 && j < d.ny + 2) {
          const int64_t o = kofs + i + j * sj;
          const T c = lapb[b + 1][a + 1];
          T v = (lapb[b + 1][a] + lapb[b + 1][a + 2]) - ((T(2) + s.crlato[b + 3]) + s.crlatu[b + 3]) * c;
          v = fma(s.crlato[b + 2], lapb[b][a + 1], v);
          v = fma(s.crlatu[b + 4], lapb[b + 2][a + 1], v);
          if (interior(i, j)) v = v + ld(outb + o);
          inb[o] = v;
        }
      });
      __syncthreads();
    }
  }
};

template <class T, class M3, class M1>
oeb_status hdiffsa_tl_entry(const M3* dout, const M3* in, const M3* mask, const M1* crlato, const M1* crlatu,
                            const M3* din, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(hdiffsa_entry<T>(dout, in, mask, crlato, crlatu, dom, stream));
    OEB_TRY(hdiffsa_entry<T>(dout, din, mask, crlato, crlatu, dom, stream));
  }
  OEB_RETURN_IF_VALIDATING();
  using D = Dual<T>;
  DualArrays<T> arr((cudaStream_t)stream);
  D *x, *m, *lo, *lu, *y;
  OEB_TRY(arr.pack(in, din, &x));
  OEB_TRY(arr.pack(mask, (const M3*)nullptr, &m));
  OEB_TRY(arr.pack(crlato, (const M1*)nullptr, &lo));
  OEB_TRY(arr.pack(crlatu, (const M1*)nullptr, &lu));
  OEB_TRY(arr.alloc(dout, &y));
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, in->strides[1], in->strides[0]};
  const int kb = tuned_kb(kKB);
  OEB_TRY(launch<hdiffsa_kernel<D>>(tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(HdiffsaSmem<D>),
                                    (cudaStream_t)stream, y, x, m, lo, lu, crlato->strides[0], d, kb));
  return arr.unpack(dout->aligned + dout->offset, y, *dom, kInterior, d.sj, d.sk);
}

template <class T, class M3, class M1>
oeb_status hdiffsa_adj_entry(const M3* inb, const M3* in, const M3* mask, const M1* crlato, const M1* crlatu,
                             const M3* outb, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(hdiffsa_entry<T>(outb, in, mask, crlato, crlatu, dom, stream));
  }
  Grid<T> gib, gin, gm, gob;
  Line<T> lo, lu;
  OEB_TRY((check_field3<T>(inb, *dom, Reach{2, 2, 2, 2, 0, 0}, &gib)));
  OEB_TRY((check_field3<T>(in, *dom, Reach{2, 2, 2, 2, 0, 0}, &gin)));
  OEB_TRY((check_field3<T>(mask, *dom, kInterior, &gm)));
  OEB_TRY((check_field3<T>(outb, *dom, kInterior, &gob)));
  OEB_TRY((check_field1<T>(crlato, *dom, 1, 1, &lo)));
  OEB_TRY((check_field1<T>(crlatu, *dom, 1, 1, &lu)));
  OEB_TRY(check_same_strides<T>({&gib, &gin, &gm, &gob}));
  OEB_TRY(check_no_alias({gib.lo, gib.hi},
                         {gin.lo, gin.hi, gm.lo, gm.hi, gob.lo, gob.hi, lo.lo, lo.hi, lu.lo, lu.hi}));
  OEB_RETURN_IF_VALIDATING();
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gin.sj, gin.sk};
  const int kb = tuned_kb(kKB);
  return launch<hdiffsa_adj_kernel<T>>(tile_grid(d.nx + 4, d.ny + 4, d.nz, kT, kT, kb), sizeof(HdiffsaAdjSmem<T>),
                                       (cudaStream_t)stream, gib.origin, gin.origin, gm.origin, lo.origin, lu.origin,
                                       lo.s, gob.origin, d, kb);
}

// ============================== hdiffsmag adjoint ================================
// Linearised at (uin, vin) with the clamp of hdiffsmag.h:236/251 frozen:
//   uout = u + su Lu,  su = clamp(tau sqrt(Xu) - w mask),  Xu = (T(i+1)^2 + T^2)/2 + (S(j-1)^2 + S^2)/2
//   T = c1 (v(j-1) - v) - c2 (u(i-1) - u),  S = c1 (u(j+1) - u) + c2 (v(i+1) - v),
//   c1 = eddlat R^-1, c2(j) = acrlat0(j) eddlon, and likewise vout.
// The transpose for (uoutb, voutb), in three gather passes over scratch:
//   1. at interior points: LU = su uoutb, LV = sv voutb, and XU = Lu uoutb tau / (2 sqrt Xu)
//      where the clamp is open (0 < smag < 0.5), else 0; XV likewise;
//   2. TB = T (XU(i-1) + XU + XV(j-1) + XV) on [0,N]^2, SB = S (XU(j+1) + XU + XV(i+1) + XV)
//      on [-1,N)^2 (the T and S adjoints);
//   3. ubar, vbar on [-1,N+1)^2: identity, the transposed laplacians of LU/LV, and the T/S
//      differences of TB/SB.
template <class T>
struct SmagTerms {
  T *lu, *lv, *xu, *xv, *tb, *sb;
};

template <class T>
__device__ __forceinline__ T smag_T(const T* __restrict__ u, const T* __restrict__ v, int64_t o, int64_t sj, T c1,
                                    T c2) {
  return c1 * (ld(v + o - sj) - ld(v + o)) - c2 * (ld(u + o - 1) - ld(u + o));
}
template <class T>
__device__ __forceinline__ T smag_S(const T* __restrict__ u, const T* __restrict__ v, int64_t o, int64_t sj, T c1,
                                    T c2) {
  return c1 * (ld(u + o + sj) - ld(u + o)) + c2 * (ld(v + o + 1) - ld(v + o));
}

// T^2 and S^2 of a tile's cells, each computed once (every point reads three of each):
//   tsq : 33 x 33, (i0+a,   j0+b)     T_s^2
//   ssq : 33 x 33, (i0-1+a, j0-1+b)   S_uv^2
template <class T>
struct SmagAdjSmem {
  T tsq[33][33];
  T ssq[33][33];
};

template <class T>
struct hdiffsmag_adj_terms_kernel {
  static constexpr int kStepOp = step_op<T>(kOpSmagAdjTerms);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, SmagTerms<T> tm, const T* __restrict__ uin,
                                             const T* __restrict__ vin, const T* __restrict__ mask,
                                             const T* __restrict__ crlavo, const T* __restrict__ crlavu,
                                             const T* __restrict__ crlato, const T* __restrict__ crlatu,
                                             const T* __restrict__ acrlat0, int64_t s1d, const T* __restrict__ uoutb,
                                             const T* __restrict__ voutb, T eddlat, T eddlon, T tau_smag,
                                             T weight_smag, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmagAdjSmem<T>& s = *reinterpret_cast<SmagAdjSmem<T>*>(smem_raw);
    constexpr T rr = earth_radius_recip<T>();
    const T c1 = eddlat * rr;
    const int64_t sj = d.sj;
    const int i0 = blk.x * kT, j0 = blk.y * kT;
    const int vx = max(0, min(kT, d.nx - i0)), vy = max(0, min(kT, d.ny - j0));
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      // T at (i, j) for i in [i0, i0+vx], j in [j0, j0+vy]; S at (i, j) for i in [i0-1, i0+vx),
      // j in [j0-1, j0+vy): every cell the tile's points read
      for_region_lim<33, 33>(vx + 1, vy + 1, [&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        const T t = smag_T(uin, vin, kofs + i + j * sj, sj, c1, ld(acrlat0 + (int64_t)j * s1d) * eddlon);
        s.tsq[b][a] = t * t;
      });
      for_region_lim<33, 33>(vx + 1, vy + 1, [&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 - 1 + b;
        const T v = smag_S(uin, vin, kofs + i + j * sj, sj, c1, ld(acrlat0 + (int64_t)j * s1d) * eddlon);
        s.ssq[b][a] = v * v;
      });
      __syncthreads();
      for_region_lim<32, 32>(vx, vy, [&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        const int64_t o = kofs + i + j * sj;
        const T hdw = weight_smag * ld(mask + o);
        // T(i+1,j)^2 + T(i,j)^2, S(i,j-1)^2 + S(i,j)^2; T(i,j+1)^2 + T(i,j)^2, S(i-1,j)^2 + S(i,j)^2
        const T xu = T(0.5) * (s.tsq[b][a + 1] + s.tsq[b][a]) + T(0.5) * (s.ssq[b][a + 1] + s.ssq[b + 1][a + 1]);
        const T xv = T(0.5) * (s.tsq[b + 1][a] + s.tsq[b][a]) + T(0.5) * (s.ssq[b + 1][a] + s.ssq[b + 1][a + 1]);
        const T ru = Prec<T>::sqrt_(xu), rv = Prec<T>::sqrt_(xv);
        const T smu = tau_smag * ru - hdw, smv = tau_smag * rv - hdw;
        const T su = clamp_smag(smu), sv = clamp_smag(smv);
        const int64_t jo = (int64_t)j * s1d;
        const T u0 = ld(uin + o), v0 = ld(vin + o);
        const T lapu = (ld(uin + o + 1) + ld(uin + o - 1) - T(2) * u0) + ld(crlato + jo) * (ld(uin + o + sj) - u0) +
                       ld(crlatu + jo) * (ld(uin + o - sj) - u0);
        const T lapv = (ld(vin + o + 1) + ld(vin + o - 1) - T(2) * v0) + ld(crlavo + jo) * (ld(vin + o + sj) - v0) +
                       ld(crlavu + jo) * (ld(vin + o - sj) - v0);
        const T yu = ld(uoutb + o), yv = ld(voutb + o);
        tm.lu[o] = su * yu;
        tm.lv[o] = sv * yv;
        tm.xu[o] = (smu > T(0) && smu < T(0.5)) ? (lapu * yu) * (tau_smag / (T(2) * ru)) : T(0);
        tm.xv[o] = (smv > T(0) && smv < T(0.5)) ? (lapv * yv) * (tau_smag / (T(2) * rv)) : T(0);
      });
      __syncthreads();
    }
  }
};

template <class T>
struct hdiffsmag_adj_ts_kernel {
  static constexpr int kStepOp = step_op<T>(kOpSmagAdjTs);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, SmagTerms<T> tm, const T* __restrict__ uin,
                                             const T* __restrict__ vin, const T* __restrict__ acrlat0, int64_t s1d,
                                             T eddlat, T eddlon, Dims d, int kb) {
    constexpr T rr = earth_radius_recip<T>();
    const T c1 = eddlat * rr;
    const int64_t sj = d.sj;
    auto in = [&](int i, int j) { return i >= 0 && i < d.nx && j >= 0 && j < d.ny; };
    for_box<RowUnroll<T>::value>(blk, d, -1, -1, d.nx + 2, d.ny + 2, kb, [&](int64_t o, int i, int j) {
      const T c2 = ld(acrlat0 + (int64_t)j * s1d) * eddlon;
      if (i >= 0 && i <= d.nx && j >= 0 && j <= d.ny) {
        T w = T(0);
        if (in(i - 1, j)) w = w + tm.xu[o - 1];
        if (in(i, j)) w = w + tm.xu[o] + tm.xv[o];
        if (in(i, j - 1)) w = w + tm.xv[o - sj];
        tm.tb[o] = (w == T(0)) ? T(0) : smag_T(uin, vin, o, sj, c1, c2) * w;
      }
      if (i >= -1 && i < d.nx && j >= -1 && j < d.ny) {
        T w = T(0);
        if (in(i, j + 1)) w = w + tm.xu[o + sj];
        if (in(i, j)) w = w + tm.xu[o] + tm.xv[o];
        if (in(i + 1, j)) w = w + tm.xv[o + 1];
        tm.sb[o] = (w == T(0)) ? T(0) : smag_S(uin, vin, o, sj, c1, c2) * w;
      }
    });
  }
};

template <class T>
struct hdiffsmag_adj_gather_kernel {
  static constexpr int kStepOp = step_op<T>(kOpSmagAdjGather);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ uinb, T* __restrict__ vinb,
                                             SmagTerms<T> tm, const T* __restrict__ uoutb,
                                             const T* __restrict__ voutb, const T* __restrict__ crlavo,
                                             const T* __restrict__ crlavu, const T* __restrict__ crlato,
                                             const T* __restrict__ crlatu, const T* __restrict__ acrlat0, int64_t s1d,
                                             T eddlat, T eddlon, Dims d, int kb) {
    constexpr T rr = earth_radius_recip<T>();
    const T c1 = eddlat * rr;
    const int64_t sj = d.sj;
    auto in = [&](int i, int j) { return i >= 0 && i < d.nx && j >= 0 && j < d.ny; };
    auto inT = [&](int i, int j) { return i >= 0 && i <= d.nx && j >= 0 && j <= d.ny; };
    auto inS = [&](int i, int j) { return i >= -1 && i < d.nx && j >= -1 && j < d.ny; };
    for_box<RowUnroll<T>::value>(blk, d, -1, -1, d.nx + 2, d.ny + 2, kb, [&](int64_t o, int a, int b) {
      const T c2 = ld(acrlat0 + (int64_t)b * s1d) * eddlon;
      T ub = T(0), vb = T(0);
      if (in(a, b)) {
        const int64_t bo = (int64_t)b * s1d;
        ub = ld(uoutb + o) - (T(2) + ld(crlato + bo) + ld(crlatu + bo)) * tm.lu[o];
        vb = ld(voutb + o) - (T(2) + ld(crlavo + bo) + ld(crlavu + bo)) * tm.lv[o];
      }
      if (in(a - 1, b)) ub = ub + tm.lu[o - 1], vb = vb + tm.lv[o - 1];
      if (in(a + 1, b)) ub = ub + tm.lu[o + 1], vb = vb + tm.lv[o + 1];
      if (in(a, b - 1)) {
        const int64_t bo = (int64_t)(b - 1) * s1d;
        ub = fma(ld(crlato + bo), tm.lu[o - sj], ub);
        vb = fma(ld(crlavo + bo), tm.lv[o - sj], vb);
      }
      if (in(a, b + 1)) {
        const int64_t bo = (int64_t)(b + 1) * s1d;
        ub = fma(ld(crlatu + bo), tm.lu[o + sj], ub);
        vb = fma(ld(crlavu + bo), tm.lv[o + sj], vb);
      }
      const T tb0 = inT(a, b) ? tm.tb[o] : T(0);
      const T sb0 = inS(a, b) ? tm.sb[o] : T(0);
      if (inT(a + 1, b)) ub = fma(-c2, tm.tb[o + 1], ub);
      ub = fma(-c1, sb0, fma(c2, tb0, ub));
      if (inS(a, b - 1)) ub = fma(c1, tm.sb[o - sj], ub);
      if (inT(a, b + 1)) vb = fma(c1, tm.tb[o + sj], vb);
      vb = fma(-c2, sb0, fma(-c1, tb0, vb));
      if (inS(a - 1, b)) vb = fma(c2, tm.sb[o - 1], vb);
      uinb[o] = ub;
      vinb[o] = vb;
    });
  }
};

// FP32 adjoint in one launch.  The three passes above write six term fields to scratch and
// read them back (about 48 bytes a point of FP32 traffic beyond the adjoint's own fields, and
// three launches).  In FP32 the terms are cheap to recompute, so here a CTA forms, for a
// 32 x 32 tile of (ubar, vbar), everything its outputs gather in shared memory:
//   u, v   : 36 x 36 from (i0-2, j0-2)     (the fields, 0 outside their reach [-1, N+1)^2)
//   t      : 35 x 35 from (i0-1, j0-1)     T on [0, N]^2, else 0
//   s      : 35 x 35 from (i0-2, j0-2)     S on [-1, N)^2, else 0
//   lu, lv, xu, xv : 34 x 34 from (i0-1, j0-1), at interior points, else 0
//   tb     : 33 x 33 from (i0, j0)         TB on [0, N]^2, else 0   } over u, v
//   sb     : 33 x 33 from (i0-1, j0-1)     SB on [-1, N)^2, else 0  } (dead by then)
// with the output tile at (i0, j0) = (-1 + 32 bx, -1 + 32 by).  Every value is the same
// expression on the same operands as in the three passes (T and S from the same
// differences, the terms, TB and SB with the same guarded sums, the gather in the same
// order), so the results are theirs, bit for bit; the recomputed apron costs about 20 % more
// arithmetic than the passes.
struct SmagAdjF32Smem {
  union {
    struct {
      float u[36][36], v[36][36];
    } f;
    struct {
      float tb[33][33], sb[33][33];
    } g;
  } x;
  float t[35][35], s[35][35];
  float lu[34][34], lv[34][34], xu[34][34], xv[34][34];
  float acr[36], cto[36], ctu[36], cvo[36], cvu[36];  // rows j0-2+r
};

struct hdiffsmag_adj_f32 {
  static constexpr int kStepOp = step_op<float>(kOpSmagAdjFused);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, float* __restrict__ uinb, float* __restrict__ vinb,
                                             const float* __restrict__ uin, const float* __restrict__ vin,
                                             const float* __restrict__ mask, const float* __restrict__ crlavo,
                                             const float* __restrict__ crlavu, const float* __restrict__ crlato,
                                             const float* __restrict__ crlatu, const float* __restrict__ acrlat0,
                                             int64_t s1d, const float* __restrict__ uoutb,
                                             const float* __restrict__ voutb, float eddlat, float eddlon,
                                             float tau_smag, float weight_smag, Dims d, int kb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmagAdjF32Smem& s = *reinterpret_cast<SmagAdjF32Smem*>(smem_raw);
    constexpr float rr = earth_radius_recip<float>();
    const float c1 = eddlat * rr;
    const int nx = d.nx, ny = d.ny;
    const int64_t sj = d.sj;
    const int i0 = -1 + (int)blk.x * kT, j0 = -1 + (int)blk.y * kT;
    auto in = [&](int i, int j) { return i >= 0 && i < nx && j >= 0 && j < ny; };
    auto inT = [&](int i, int j) { return i >= 0 && i <= nx && j >= 0 && j <= ny; };
    auto inS = [&](int i, int j) { return i >= -1 && i < nx && j >= -1 && j < ny; };
    const int tid = threadIdx.y * kTX + threadIdx.x;
    if (tid < 36) {
      const int j = j0 - 2 + tid;
      const int64_t jo = (int64_t)j * s1d;
      const bool in1 = j >= -1 && j < ny + 1, in0 = j >= 0 && j < ny;
      s.acr[tid] = in1 ? ld(acrlat0 + jo) : 0.f;
      s.cto[tid] = in0 ? ld(crlato + jo) : 0.f;
      s.ctu[tid] = in0 ? ld(crlatu + jo) : 0.f;
      s.cvo[tid] = in0 ? ld(crlavo + jo) : 0.f;
      s.cvu[tid] = in0 ? ld(crlavu + jo) : 0.f;
    }
    const int k0 = blk.z * kb, k1 = min(k0 + kb, d.nz);
  #pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int64_t kofs = (int64_t)k * d.sk;
      for_region<36, 36>([&](int a, int b) {
        const int i = i0 - 2 + a, j = j0 - 2 + b;
        const bool ok = i >= -1 && i < nx + 1 && j >= -1 && j < ny + 1;
        const int64_t o = kofs + i + j * sj;
        s.x.f.u[b][a] = ok ? ld(uin + o) : 0.f;
        s.x.f.v[b][a] = ok ? ld(vin + o) : 0.f;
      });
      __syncthreads();
      // T = c1 (v(j-1) - v) - c2 (u(i-1) - u),  S = c1 (u(j+1) - u) + c2 (v(i+1) - v)  (smag_T, smag_S)
      for_region<35, 35>([&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 - 1 + b;
        float t = 0.f;
        if (inT(i, j)) {
          const float c2 = s.acr[b + 1] * eddlon;
          t = c1 * (s.x.f.v[b][a + 1] - s.x.f.v[b + 1][a + 1]) - c2 * (s.x.f.u[b + 1][a] - s.x.f.u[b + 1][a + 1]);
        }
        s.t[b][a] = t;
      });
      for_region<35, 35>([&](int a, int b) {
        const int i = i0 - 2 + a, j = j0 - 2 + b;
        float v = 0.f;
        if (inS(i, j)) {
          const float c2 = s.acr[b] * eddlon;
          v = c1 * (s.x.f.u[b + 1][a] - s.x.f.u[b][a]) + c2 * (s.x.f.v[b][a + 1] - s.x.f.v[b][a]);
        }
        s.s[b][a] = v;
      });
      __syncthreads();
      // the terms at interior points (hdiffsmag_adj_terms_kernel)
      for_region<34, 34>([&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 - 1 + b;
        float lu = 0.f, lv = 0.f, xu = 0.f, xv = 0.f;
        if (in(i, j)) {
          const int64_t o = kofs + i + j * sj;
          const float ti = s.t[b][a], tip = s.t[b][a + 1], tjp = s.t[b + 1][a];
          const float si = s.s[b + 1][a + 1], sjm = s.s[b][a + 1], sim = s.s[b + 1][a];
          const float xuu = 0.5f * (tip * tip + ti * ti) + 0.5f * (sjm * sjm + si * si);
          const float xvv = 0.5f * (tjp * tjp + ti * ti) + 0.5f * (sim * sim + si * si);
          const float hdw = weight_smag * ld(mask + o);
          const float ru = Prec<float>::sqrt_(xuu), rv = Prec<float>::sqrt_(xvv);
          const float smu = tau_smag * ru - hdw, smv = tau_smag * rv - hdw;
          const float su = clamp_smag(smu), sv = clamp_smag(smv);
          const float u0 = s.x.f.u[b + 1][a + 1], v0 = s.x.f.v[b + 1][a + 1];
          const float lapu = (s.x.f.u[b + 1][a + 2] + s.x.f.u[b + 1][a] - 2.f * u0) +
                             s.cto[b + 1] * (s.x.f.u[b + 2][a + 1] - u0) + s.ctu[b + 1] * (s.x.f.u[b][a + 1] - u0);
          const float lapv = (s.x.f.v[b + 1][a + 2] + s.x.f.v[b + 1][a] - 2.f * v0) +
                             s.cvo[b + 1] * (s.x.f.v[b + 2][a + 1] - v0) + s.cvu[b + 1] * (s.x.f.v[b][a + 1] - v0);
          const float yu = ld(uoutb + o), yv = ld(voutb + o);
          lu = su * yu;
          lv = sv * yv;
          xu = (smu > 0.f && smu < 0.5f) ? (lapu * yu) * (tau_smag / (2.f * ru)) : 0.f;
          xv = (smv > 0.f && smv < 0.5f) ? (lapv * yv) * (tau_smag / (2.f * rv)) : 0.f;
        }
        s.lu[b][a] = lu;
        s.lv[b][a] = lv;
        s.xu[b][a] = xu;
        s.xv[b][a] = xv;
      });
      __syncthreads();
      // the T and S adjoints (hdiffsmag_adj_ts_kernel), over the dead u, v
      for_region<33, 33>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        float tb = 0.f;
        if (inT(i, j)) {
          float w = 0.f;
          if (in(i - 1, j)) w = w + s.xu[b + 1][a];
          if (in(i, j)) w = w + s.xu[b + 1][a + 1] + s.xv[b + 1][a + 1];
          if (in(i, j - 1)) w = w + s.xv[b][a + 1];
          tb = (w == 0.f) ? 0.f : s.t[b + 1][a + 1] * w;
        }
        s.x.g.tb[b][a] = tb;
      });
      for_region<33, 33>([&](int a, int b) {
        const int i = i0 - 1 + a, j = j0 - 1 + b;
        float sb = 0.f;
        if (inS(i, j)) {
          float w = 0.f;
          if (in(i, j + 1)) w = w + s.xu[b + 1][a];
          if (in(i, j)) w = w + s.xu[b][a] + s.xv[b][a];
          if (in(i + 1, j)) w = w + s.xv[b][a + 1];
          sb = (w == 0.f) ? 0.f : s.s[b + 1][a + 1] * w;
        }
        s.x.g.sb[b][a] = sb;
      });
      __syncthreads();
      // the gather (hdiffsmag_adj_gather_kernel) on [-1, N+1)^2
      for_region<32, 32>([&](int a, int b) {
        const int i = i0 + a, j = j0 + b;
        if (i >= nx + 1 || j >= ny + 1) return;
        const int64_t o = kofs + i + j * sj;
        const float c2 = s.acr[b + 2] * eddlon;
        float ub = 0.f, vb = 0.f;
        if (in(i, j)) {
          ub = ld(uoutb + o) - (2.f + s.cto[b + 2] + s.ctu[b + 2]) * s.lu[b + 1][a + 1];
          vb = ld(voutb + o) - (2.f + s.cvo[b + 2] + s.cvu[b + 2]) * s.lv[b + 1][a + 1];
        }
        if (in(i - 1, j)) ub = ub + s.lu[b + 1][a], vb = vb + s.lv[b + 1][a];
        if (in(i + 1, j)) ub = ub + s.lu[b + 1][a + 2], vb = vb + s.lv[b + 1][a + 2];
        if (in(i, j - 1)) {
          ub = fmaf(s.cto[b + 1], s.lu[b][a + 1], ub);
          vb = fmaf(s.cvo[b + 1], s.lv[b][a + 1], vb);
        }
        if (in(i, j + 1)) {
          ub = fmaf(s.ctu[b + 3], s.lu[b + 2][a + 1], ub);
          vb = fmaf(s.cvu[b + 3], s.lv[b + 2][a + 1], vb);
        }
        const float tb0 = inT(i, j) ? s.x.g.tb[b][a] : 0.f;
        const float sb0 = inS(i, j) ? s.x.g.sb[b + 1][a + 1] : 0.f;
        if (inT(i + 1, j)) ub = fmaf(-c2, s.x.g.tb[b][a + 1], ub);
        ub = fmaf(-c1, sb0, fmaf(c2, tb0, ub));
        if (inS(i, j - 1)) ub = fmaf(c1, s.x.g.sb[b][a + 1], ub);
        if (inT(i, j + 1)) vb = fmaf(c1, s.x.g.tb[b + 1][a], vb);
        vb = fmaf(-c2, sb0, fmaf(-c1, tb0, vb));
        if (inS(i - 1, j)) vb = fmaf(c2, s.x.g.sb[b + 1][a], vb);
        uinb[o] = ub;
        vinb[o] = vb;
      });
      __syncthreads();
    }
  }
};

template <class T, class M3, class M1>
oeb_status hdiffsmag_adj_entry(const M3* uinb, const M3* vinb, const M3* uin, const M3* vin, const M3* mask,
                               const M1* crlavo, const M1* crlavu, const M1* crlato, const M1* crlatu,
                               const M1* acrlat0, const M3* uoutb, const M3* voutb, T eddlat, T eddlon, T tau_smag,
                               T weight_smag, const oeb_domain* dom, void* stream) {
  {
    ValidateOnly guard;
    OEB_TRY(hdiffsmag_entry<T>(uoutb, voutb, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, eddlat, eddlon,
                               tau_smag, weight_smag, dom, stream));
  }
  Grid<T> gub, gvb, gui, guo;
  OEB_TRY((check_field3<T>(uinb, *dom, Reach{1, 1, 1, 1, 0, 0}, &gub)));
  OEB_TRY((check_field3<T>(vinb, *dom, Reach{1, 1, 1, 1, 0, 0}, &gvb)));
  OEB_TRY((check_field3<T>(uin, *dom, Reach{1, 1, 1, 1, 0, 0}, &gui)));
  OEB_TRY((check_field3<T>(uoutb, *dom, kInterior, &guo)));
  OEB_TRY(check_same_strides<T>({&gub, &gvb, &gui, &guo}));
  OEB_TRY(check_no_alias({gub.lo, gub.hi, gvb.lo, gvb.hi}, {gui.lo, gui.hi, guo.lo, guo.hi}));
  OEB_RETURN_IF_VALIDATING();
  cudaStream_t st = (cudaStream_t)stream;
  if constexpr (std::is_same<T, float>::value) if (adjoint_tiles()) {
    const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
    const int kb = tuned_kb(kKB);
    auto org1 = [](const M1* m) { return (const float*)m->aligned + m->offset; };
    return launch<hdiffsmag_adj_f32>(tile_grid(d.nx + 2, d.ny + 2, d.nz, kT, kT, kb), sizeof(SmagAdjF32Smem), st,
                                     gub.origin, gvb.origin, gui.origin, (const float*)vin->aligned + vin->offset,
                                     (const float*)mask->aligned + mask->offset, org1(crlavo), org1(crlavu),
                                     org1(crlato), org1(crlatu), org1(acrlat0), acrlat0->strides[0], guo.origin,
                                     (const float*)voutb->aligned + voutb->offset, eddlat, eddlon, tau_smag,
                                     weight_smag, d, kb);
  }
  const T* start = (uin->allocated && uin->allocated <= uin->aligned) ? uin->allocated : uin->aligned;
  const int64_t last = (uin->sizes[0] - 1) * uin->strides[0] + (uin->sizes[1] - 1) * uin->strides[1] +
                       (uin->sizes[2] - 1) * uin->strides[2];
  const int64_t n = (int64_t)(uin->aligned - start) + last + 1;
  const int64_t org = (int64_t)(uin->aligned - start) + uin->offset;
  void* buf = nullptr;
  OEB_TRY(scratch_alloc(&buf, (size_t)n * 6 * sizeof(T), st));
  T* base = static_cast<T*>(buf);
  SmagTerms<T> tm{base + org, base + n + org, base + 2 * n + org, base + 3 * n + org, base + 4 * n + org,
                  base + 5 * n + org};
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
  auto org1 = [](const M1* m) { return (const T*)m->aligned + m->offset; };
  const int64_t s1d = acrlat0->strides[0];
  const int kb = tuned_kb(kKB);
  oeb_status stt = launch<hdiffsmag_adj_terms_kernel<T>>(
      tile_grid(d.nx, d.ny, d.nz, kT, kT, kb), sizeof(SmagAdjSmem<T>), st, tm, gui.origin, (const T*)vin->aligned + vin->offset,
      (const T*)mask->aligned + mask->offset, org1(crlavo), org1(crlavu), org1(crlato), org1(crlatu), org1(acrlat0), s1d,
      guo.origin, (const T*)voutb->aligned + voutb->offset, eddlat, eddlon, tau_smag, weight_smag, d, kb);
  if (stt == OEB_OK)
    stt = launch<hdiffsmag_adj_ts_kernel<T>>(tile_grid(d.nx + 2, d.ny + 2, d.nz, kT, kT, kb), 0, st, tm, gui.origin,
                                             (const T*)vin->aligned + vin->offset, org1(acrlat0), s1d, eddlat, eddlon,
                                             d, kb);
  if (stt == OEB_OK)
    stt = launch<hdiffsmag_adj_gather_kernel<T>>(
        tile_grid(d.nx + 2, d.ny + 2, d.nz, kT, kT, kb), 0, st, gub.origin, gvb.origin, tm, guo.origin,
        (const T*)voutb->aligned + voutb->offset, org1(crlavo), org1(crlavu), org1(crlato), org1(crlatu), org1(acrlat0),
        s1d, eddlat, eddlon, d, kb);
  scratch_free(buf, st);
  return stt;
}

#ifndef OEB_BODIES_ONLY
// ==================== hdiffsmag adjoint without any allocation (FP64) ====================
// oeb_hdiffsmag_adj_noalloc_f64 is for callers that cannot allocate device memory while they
// run: a host whose own allocator has already claimed the GPU's memory up front (an
// allocation from this library's pool could then fail in the middle of a run), or a
// time-stepping loop that must not take an allocation inside its step.  It runs the same three
// kernels as oeb_hdiffsmag_adj_f64, on the same validated arguments, but its six term fields
// live in one fixed array compiled into the library instead of coming from the pool.
//
//  * Limit: each term field holds kNoAllocCells = 2^21 cells, so the span of uin's
//    allocation (halo and padding included) may be at most 2^21 cells; a larger field is
//    rejected with OEB_ERR_TOO_LARGE before anything runs.  The array is 6 x 2^21 doubles =
//    96 MiB, and every GPU that loads the library holds it until the process exits.
//  * Every call uses the same array, which keeps the last call's contents.  Each cell the
//    kernels read is written earlier in the same call (the terms on the interior, the T/S
//    adjoints on their boxes), so nothing has to start at zero and nothing is cleared.  Calls
//    that overlap on the GPU -- on two streams, or from two host threads -- race on the array.
//  * Set-up: the array's name is only a host-side stand-in for the device variable.  The first
//    call on a device looks up its device address with cudaGetSymbolAddress, with that device
//    current, and keeps it for later calls; make that first call before any stream capture.
//    The kept address outlives a cudaDeviceReset of that device, after which it is stale: the
//    entry point is not for use on a device after such a reset.
constexpr int64_t kNoAllocCells = int64_t(1) << 21;
static __device__ __align__(256) double g_hdiffsmag_adj_scratch[6 * kNoAllocCells];

oeb_status hdiffsmag_adj_scratch_address(double** out) {
  static std::mutex mu;
  static std::vector<double*> addr;  // per device
  int dev = 0;
  OEB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)addr.size() <= dev) addr.resize(dev + 1, nullptr);
  if (!addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_hdiffsmag_adj_scratch);
    if (e != cudaSuccess) return cuda_fail(e);
    addr[dev] = static_cast<double*>(p);
  }
  *out = addr[dev];
  return OEB_OK;
}

oeb_status hdiffsmag_adj_noalloc_entry(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb,
                                       const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                       const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlavo,
                                       const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato,
                                       const oeb_memref1d_f64* crlatu, const oeb_memref1d_f64* acrlat0,
                                       const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double eddlat,
                                       double eddlon, double tau_smag, double weight_smag, const oeb_domain* dom,
                                       void* stream) {
  using T = double;
  {
    // every check of the pool-backed entry point, nothing launched
    ValidateOnly guard;
    OEB_TRY(hdiffsmag_adj_entry<T>(uinb, vinb, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, uoutb, voutb,
                                   eddlat, eddlon, tau_smag, weight_smag, dom, stream));
  }
  Grid<T> gub, gvb, gui, guo;
  OEB_TRY((check_field3<T>(uinb, *dom, Reach{1, 1, 1, 1, 0, 0}, &gub)));
  OEB_TRY((check_field3<T>(vinb, *dom, Reach{1, 1, 1, 1, 0, 0}, &gvb)));
  OEB_TRY((check_field3<T>(uin, *dom, Reach{1, 1, 1, 1, 0, 0}, &gui)));
  OEB_TRY((check_field3<T>(uoutb, *dom, kInterior, &guo)));
  const T* start = (uin->allocated && uin->allocated <= uin->aligned) ? uin->allocated : uin->aligned;
  const int64_t last = (uin->sizes[0] - 1) * uin->strides[0] + (uin->sizes[1] - 1) * uin->strides[1] +
                       (uin->sizes[2] - 1) * uin->strides[2];
  const int64_t n = (int64_t)(uin->aligned - start) + last + 1;
  const int64_t org = (int64_t)(uin->aligned - start) + uin->offset;
  if (n > kNoAllocCells) return OEB_ERR_TOO_LARGE;
  OEB_RETURN_IF_VALIDATING();
  T* base = nullptr;
  OEB_TRY(hdiffsmag_adj_scratch_address(&base));
  SmagTerms<T> tm{base + org, base + kNoAllocCells + org, base + 2 * kNoAllocCells + org,
                  base + 3 * kNoAllocCells + org, base + 4 * kNoAllocCells + org, base + 5 * kNoAllocCells + org};
  const Dims d{(int)dom->nx, (int)dom->ny, (int)dom->nz, gui.sj, gui.sk};
  auto org1 = [](const oeb_memref1d_f64* m) { return (const T*)m->aligned + m->offset; };
  const int64_t s1d = acrlat0->strides[0];
  cudaStream_t st = (cudaStream_t)stream;
  OEB_TRY(launch<hdiffsmag_adj_terms_kernel<T>>(
      tile_grid(d.nx, d.ny, d.nz, kT, kT, kKB), sizeof(SmagAdjSmem<T>), st, tm, gui.origin, (const T*)vin->aligned + vin->offset,
      (const T*)mask->aligned + mask->offset, org1(crlavo), org1(crlavu), org1(crlato), org1(crlatu), org1(acrlat0), s1d,
      guo.origin, (const T*)voutb->aligned + voutb->offset, eddlat, eddlon, tau_smag, weight_smag, d, kKB));
  OEB_TRY(launch<hdiffsmag_adj_ts_kernel<T>>(tile_grid(d.nx + 2, d.ny + 2, d.nz, kT, kT, kKB), 0, st, tm, gui.origin,
                                             (const T*)vin->aligned + vin->offset, org1(acrlat0), s1d, eddlat, eddlon,
                                             d, kKB));
  return launch<hdiffsmag_adj_gather_kernel<T>>(
      tile_grid(d.nx + 2, d.ny + 2, d.nz, kT, kT, kKB), 0, st, gub.origin, gvb.origin, tm, guo.origin,
      (const T*)voutb->aligned + voutb->offset, org1(crlavo), org1(crlavu), org1(crlato), org1(crlatu), org1(acrlat0),
      s1d, eddlat, eddlon, d, kKB);
}
#endif  // OEB_BODIES_ONLY

}  // namespace
}  // namespace oeb

#ifndef OEB_BODIES_ONLY  // the entry points

using namespace oeb;

#define OEB_HDIFF_ENTRIES(S, T)                                                                                     \
  extern "C" oeb_status oeb_hdiffsa_##S(const oeb_memref3d_##S* out, const oeb_memref3d_##S* in,                   \
                                        const oeb_memref3d_##S* mask, const oeb_memref1d_##S* crlato,             \
                                        const oeb_memref1d_##S* crlatu, const oeb_domain* dom, void* stream) {    \
    return hdiffsa_entry<T>(out, in, mask, crlato, crlatu, dom, stream);                                          \
  }                                                                                                                \
  extern "C" oeb_status oeb_hdiffsmag_##S(                                                                         \
      const oeb_memref3d_##S* uout, const oeb_memref3d_##S* vout, const oeb_memref3d_##S* uin,                      \
      const oeb_memref3d_##S* vin, const oeb_memref3d_##S* mask, const oeb_memref1d_##S* crlavo,                    \
      const oeb_memref1d_##S* crlavu, const oeb_memref1d_##S* crlato, const oeb_memref1d_##S* crlatu,               \
      const oeb_memref1d_##S* acrlat0, T eddlat, T eddlon, T tau_smag, T weight_smag, const oeb_domain* dom,       \
      void* stream) {                                                                                              \
    return hdiffsmag_entry<T>(uout, vout, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, eddlat, eddlon,\
                              tau_smag, weight_smag, dom, stream);                                                 \
  }                                                                                                                \
  extern "C" oeb_status oeb_hdiffsmag_tl_##S(                                                                      \
      const oeb_memref3d_##S* duout, const oeb_memref3d_##S* dvout, const oeb_memref3d_##S* uin,                    \
      const oeb_memref3d_##S* vin, const oeb_memref3d_##S* mask, const oeb_memref1d_##S* crlavo,                    \
      const oeb_memref1d_##S* crlavu, const oeb_memref1d_##S* crlato, const oeb_memref1d_##S* crlatu,               \
      const oeb_memref1d_##S* acrlat0, const oeb_memref3d_##S* duin, const oeb_memref3d_##S* dvin, T eddlat,        \
      T eddlon, T tau_smag, T weight_smag, const oeb_domain* dom, void* stream) {                                  \
    return hdiffsmag_tl_entry<T>(duout, dvout, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, duin, dvin, \
                                 eddlat, eddlon, tau_smag, weight_smag, dom, stream);                             \
  }                                                                                                                \
  extern "C" oeb_status oeb_hdiffsmag_adj_##S(                                                                     \
      const oeb_memref3d_##S* uinb, const oeb_memref3d_##S* vinb, const oeb_memref3d_##S* uin,                      \
      const oeb_memref3d_##S* vin, const oeb_memref3d_##S* mask, const oeb_memref1d_##S* crlavo,                    \
      const oeb_memref1d_##S* crlavu, const oeb_memref1d_##S* crlato, const oeb_memref1d_##S* crlatu,               \
      const oeb_memref1d_##S* acrlat0, const oeb_memref3d_##S* uoutb, const oeb_memref3d_##S* voutb, T eddlat,      \
      T eddlon, T tau_smag, T weight_smag, const oeb_domain* dom, void* stream) {                                  \
    return hdiffsmag_adj_entry<T>(uinb, vinb, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, uoutb,     \
                                  voutb, eddlat, eddlon, tau_smag, weight_smag, dom, stream);                     \
  }

#define OEB_HDIFFSA_DIFF_ENTRIES(S, T)                                                                              \
  extern "C" oeb_status oeb_hdiffsa_tl_##S(const oeb_memref3d_##S* dout, const oeb_memref3d_##S* in,               \
                                           const oeb_memref3d_##S* mask, const oeb_memref1d_##S* crlato,          \
                                           const oeb_memref1d_##S* crlatu, const oeb_memref3d_##S* din,           \
                                           const oeb_domain* dom, void* stream) {                                  \
    return hdiffsa_tl_entry<T>(dout, in, mask, crlato, crlatu, din, dom, stream);                                  \
  }                                                                                                                \
  extern "C" oeb_status oeb_hdiffsa_adj_##S(const oeb_memref3d_##S* inb, const oeb_memref3d_##S* in,              \
                                            const oeb_memref3d_##S* mask, const oeb_memref1d_##S* crlato,         \
                                            const oeb_memref1d_##S* crlatu, const oeb_memref3d_##S* outb,         \
                                            const oeb_domain* dom, void* stream) {                                 \
    return hdiffsa_adj_entry<T>(inb, in, mask, crlato, crlatu, outb, dom, stream);                                 \
  }

OEB_HDIFF_ENTRIES(f64, double)
OEB_HDIFF_ENTRIES(f32, float)
OEB_HDIFFSA_DIFF_ENTRIES(f64, double)
OEB_HDIFFSA_DIFF_ENTRIES(f32, float)

extern "C" oeb_status oeb_hdiffsmag_adj_noalloc_f64(
    const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* uin,
    const oeb_memref3d_f64* vin, const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlavo,
    const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu,
    const oeb_memref1d_f64* acrlat0, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double eddlat,
    double eddlon, double tau_smag, double weight_smag, const oeb_domain* dom, void* stream) {
  return hdiffsmag_adj_noalloc_entry(uinb, vinb, uin, vin, mask, crlavo, crlavu, crlato, crlatu, acrlat0, uoutb, voutb,
                                     eddlat, eddlon, tau_smag, weight_smag, dom, stream);
}

#endif  // OEB_BODIES_ONLY
