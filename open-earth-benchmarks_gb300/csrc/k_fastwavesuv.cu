// k_fastwavesuv.cu -- fastwavesuv (kernels/fastwavesuv.h:154-191) in FP64 and FP32.
//
// The OpenMP variant evaluates ppgk = wgtfac*ppuv + (1-wgtfac)*ppuv(k-1) six times per point
// ((i,j),(i+1,j),(i,j+1) at k and k+1).  Here each CTA marches upward through KB k-levels
// of a 32 x 32 tile: at level k every point of the tile plus a one-cell apron in i and j
// computes ppgk(k+1) once, keeps it in a register for level k+1, and publishes
// ppgc = ppgk(k+1) - ppgk(k) and the hhl sum and difference of its column through shared
// memory; the output pass then reads its i+1 and j+1 neighbours from there.
//
// Compiled with --fmad=false (see k_pointwise.cu).
#include "precision.cuh"
#include "stencil_util.cuh"

namespace oeb {
namespace {

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
__global__ void __launch_bounds__(kThreads) fastwavesuv_kernel(
    T* __restrict__ uout, T* __restrict__ vout, const T* __restrict__ uin, const T* __restrict__ vin,
    const T* __restrict__ utens, const T* __restrict__ vtens, const T* __restrict__ wgtfac,
    const T* __restrict__ ppuv, const T* __restrict__ hhl, const T* __restrict__ rho, const T* __restrict__ fx,
    int64_t s1d, T ed2, T dt, Dims d, int kb) {
  __shared__ FastwavesSmem<T> s;
  const int i0 = blockIdx.x * kT, j0 = blockIdx.y * kT;
  const int sj = (int)d.sj;
  const int64_t sk = d.sk;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  if (tid < kT) {
    const int j = j0 + tid;
    s.fx2[tid] = (j < d.ny) ? T(2.0) * ld(fx + (int64_t)j * s1d) : T(0);
  }
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, d.nz);

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
        const T ppgu = (ld(ppuv + o + 1) - p0) + (((s.ppgc[b][a + 1] + s.ppgc[b][a]) * T(0.5)) *
                                                      (s.hs[b][a] - s.hs[b][a + 1])) /
                                                         (s.hd[b][a] + s.hd[b][a + 1]);
        // fastwavesuv.h:177-180
        const T ppgv = (ld(ppuv + o + sj) - p0) + (((s.ppgc[b + 1][a] + s.ppgc[b][a]) * T(0.5)) *
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

constexpr int kKB = 4;

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
  fastwavesuv_kernel<T><<<tile_grid(d.nx, d.ny, d.nz, kT, kT, kKB), dim3(kTX, kTY), 0, (cudaStream_t)stream>>>(
      gu.origin, gv.origin, gui.origin, gvi.origin, gut.origin, gvt.origin, gw.origin, gp.origin, gh.origin,
      gr.origin, lfx.origin, lfx.s, ed2, dt, d, kKB);
  return after_launch();
}

}  // namespace
}  // namespace oeb

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
  }

OEB_FW_ENTRY(f64, double)
OEB_FW_ENTRY(f32, float)
