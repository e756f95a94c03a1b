// chain.cu -- the chained dycore step (fastwavesuv -> hadvuv5th -> update -> hdiffsmag ->
// fvtp2d), its tangent-linear and adjoint steps, and CUDA graphs of library calls.
//
// The reference has no chained step: each driver (src/<k>.cpp) runs one stencil.  The step
// here composes the stencils of this library through their own validated entry points, so
// the stage results are exactly those of single calls.  Halo handling is by recomputation:
// stage s runs over the interior widened by the cells that the later stages read, i.e. the
// entry point gets descriptors whose origin is shifted by -e in i and j and a domain of
// (nx + 2e, ny + 2e, nz).  With e = 7, 4, 4, 3, 0 the step reads only its inputs' halo and
// needs no exchange between stages.
//
// The adjoint step recomputes the forward intermediates from the step's inputs (no state
// is kept between calls) and runs the stage adjoints in reverse order; two small box
// kernels add the seeds of the step's own outputs and the identity part of stage 3.
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "fused.cuh"
#include "oeb_common.cuh"
#include "stencil_util.cuh"

struct oeb_chain_plan {
  int elem;  // sizeof(T)
  int modes;
  int device;
  oeb_domain dom;
  int64_t offset, sizes[3], strides[3];
  size_t field_bytes;
  std::vector<void*> bufs;  // one cudaMalloc per workspace field
  // workspace fields (nullptr when the plan's modes do not need them)
  void *u1, *v1, *tu, *tv, *u2, *v2, *qi, *qj, *fx2, *fy2;  // forward
  void *u3, *v3;                                            // the new u, v (TL and adjoint)
  void *du1, *dv1, *dtu, *dtv, *du2, *dv2, *dqi, *dqj, *dfx2, *dfy2, *zero;  // TL
  void *qb, *v3b, *u2b, *v2b, *wu, *wv, *utb, *vtb, *ppb;                     // adjoint
};

struct oeb_graph {
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  uint64_t kernels;
};

// Built on its own, this file's bodies and helpers are local to it; the step kernel
// (step.cu) includes it with OEB_BODIES_ONLY and a namespace of its own instead.
#ifndef OEB_BODIES_NS
#define OEB_BODIES_NS
#endif
namespace oeb {
namespace OEB_BODIES_NS {

// Halo widths of the stages (cells added on each side of the interior in i and j).
constexpr int kE1 = 7, kE2 = 4, kE3 = 3;

template <class T>
struct Abi;

template <>
struct Abi<double> {
  using M3 = oeb_memref3d_f64;
  using M1 = oeb_memref1d_f64;
  using Fields = oeb_chain_fields_f64;
  static constexpr auto fastwavesuv = &oeb_fastwavesuv_f64;
  static constexpr auto hadvuv5th = &oeb_hadvuv5th_f64;
  static constexpr auto hdiffsmag = &oeb_hdiffsmag_f64;
  static constexpr auto fvtp2d = &oeb_fvtp2d_f64;
  static constexpr auto fastwavesuv_tl = &oeb_fastwavesuv_tl_f64;
  static constexpr auto hadvuv5th_tl = &oeb_hadvuv5th_tl_f64;
  static constexpr auto hdiffsmag_tl = &oeb_hdiffsmag_tl_f64;
  static constexpr auto fvtp2d_tl = &oeb_fvtp2d_tl_f64;
  static constexpr auto fastwavesuv_adj = &oeb_fastwavesuv_adj_f64;
  static constexpr auto hadvuv5th_adj = &oeb_hadvuv5th_adj_f64;
  static constexpr auto hdiffsmag_adj = &oeb_hdiffsmag_adj_f64;
  static constexpr auto fvtp2d_adj = &oeb_fvtp2d_adj_f64;
};

template <>
struct Abi<float> {
  using M3 = oeb_memref3d_f32;
  using M1 = oeb_memref1d_f32;
  using Fields = oeb_chain_fields_f32;
  static constexpr auto fastwavesuv = &oeb_fastwavesuv_f32;
  static constexpr auto hadvuv5th = &oeb_hadvuv5th_f32;
  static constexpr auto hdiffsmag = &oeb_hdiffsmag_f32;
  static constexpr auto fvtp2d = &oeb_fvtp2d_f32;
  static constexpr auto fastwavesuv_tl = &oeb_fastwavesuv_tl_f32;
  static constexpr auto hadvuv5th_tl = &oeb_hadvuv5th_tl_f32;
  static constexpr auto hdiffsmag_tl = &oeb_hdiffsmag_tl_f32;
  static constexpr auto fvtp2d_tl = &oeb_fvtp2d_tl_f32;
  static constexpr auto fastwavesuv_adj = &oeb_fastwavesuv_adj_f32;
  static constexpr auto hadvuv5th_adj = &oeb_hadvuv5th_adj_f32;
  static constexpr auto hdiffsmag_adj = &oeb_hdiffsmag_adj_f32;
  static constexpr auto fvtp2d_adj = &oeb_fvtp2d_adj_f32;
};

// out = alpha x + (y on the box [-ey, n+ey) in i and j, else 0) over the box widened by e;
// x may be null (0) and may alias out.
template <class T>
struct combine_kernel {
  static constexpr int kStepOp = step_op<T>(kOpCombine);  // the step kernel's id
  static __device__ __forceinline__ void run(const uint3& blk, T* out, const T* x, T alpha, const T* __restrict__ y,
                                             int ey, Dims d, int e, int kb) {
    for_box(blk, d, -e, -e, d.nx + 2 * e, d.ny + 2 * e, kb, [&](int64_t o, int i, int j) {
      const bool in_y = y && i >= -ey && i < d.nx + ey && j >= -ey && j < d.ny + ey;
      const T a = x ? alpha * x[o] : T(0);
      out[o] = in_y ? a + y[o] : a;
    });
  }
};

constexpr int kBoxKB = 1;

// A 3-D descriptor whose origin is shifted by -e in i and j (the same memory).
template <class M>
M widen(const M* m, int e) {
  M r = *m;
  r.offset -= (int64_t)e * (m->strides[1] + m->strides[2]);
  return r;
}
template <class M>
M widen1(const M* m, int e) {
  M r = *m;
  r.offset -= (int64_t)e * m->strides[0];
  return r;
}
oeb_domain widen_dom(const oeb_domain& d, int e) { return oeb_domain{d.nx + 2 * e, d.ny + 2 * e, d.nz}; }

// The i/j halo below the origin of a 3-D field must hold e cells for its origin to be
// shifted by e (the stage's own checks cover the far side and k).
template <class M>
oeb_status check_ij_halo(const M* m, int e) {
  if (!m || !m->aligned) return OEB_ERR_NULL;
  const int64_t sk = m->strides[0], sj = m->strides[1];
  if (m->strides[2] != 1 || sj < 1 || sk < 1 || m->offset < 0) return OEB_ERR_LAYOUT;
  const int64_t rem = m->offset % sk;
  if (rem / sj < e || rem % sj < e) return OEB_ERR_HALO;
  return OEB_OK;
}
template <class M>
oeb_status check_j_halo1(const M* m, int e) {
  if (!m || !m->aligned) return OEB_ERR_NULL;
  if (m->strides[0] < 1 || m->offset < 0 || m->offset / m->strides[0] < e) return OEB_ERR_HALO;
  return OEB_OK;
}

template <class T>
oeb_status check_plan(const oeb_chain_plan* p, int mode) {
  if (!p) return OEB_ERR_NULL;
  if (p->elem != (int)sizeof(T)) return OEB_ERR_UNSUPPORTED;
  if (!(p->modes & mode)) return OEB_ERR_UNSUPPORTED;
  int dev = 0;
  OEB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != p->device) return OEB_ERR_ARGUMENT;
  return OEB_OK;
}

// The workspace field `buf` as a descriptor laid out like the plan's template.
template <class T>
typename Abi<T>::M3 ws(const oeb_chain_plan* p, void* buf) {
  typename Abi<T>::M3 m;
  m.allocated = static_cast<T*>(buf);
  m.aligned = static_cast<T*>(buf);
  m.offset = p->offset;
  for (int r = 0; r < 3; ++r) {
    m.sizes[r] = p->sizes[r];
    m.strides[r] = p->strides[r];
  }
  return m;
}

// The workspace field `buf`, with its origin shifted by -e in i and j.
template <class T>
typename Abi<T>::M3 wsw(const oeb_chain_plan* p, void* buf, int e) {
  typename Abi<T>::M3 m = ws<T>(p, buf);
  m.offset -= (int64_t)e * (m.strides[1] + m.strides[2]);
  return m;
}

template <class T>
oeb_status check_inputs(const typename Abi<T>::Fields* f) {
  using M3 = typename Abi<T>::M3;
  using M1 = typename Abi<T>::M1;
  if (!f) return OEB_ERR_NULL;
  const M3* s1[] = {f->u, f->v, f->utens, f->vtens, f->wgtfac, f->ppuv, f->hhl, f->rho};
  for (const M3* m : s1) OEB_TRY(check_ij_halo(m, kE1));
  OEB_TRY(check_j_halo1(f->fx, kE1));
  const M1* s2[] = {f->acrlat0, f->acrlat1, f->tgrlatda0, f->tgrlatda1};
  for (const M1* m : s2) OEB_TRY(check_j_halo1(m, kE2));
  OEB_TRY(check_ij_halo(f->mask, kE3));
  const M1* s4[] = {f->crlavo, f->crlavu, f->crlato, f->crlatu, f->smag_acrlat0};
  for (const M1* m : s4) OEB_TRY(check_j_halo1(m, kE3));
  const M3* s5[] = {f->crx, f->cry, f->ra_x, f->ra_y, f->xfx, f->yfx, f->area};
  for (const M3* m : s5)
    if (!m || !m->aligned) return OEB_ERR_NULL;
  return OEB_OK;
}

template <class T>
oeb_status launch_combine(const oeb_chain_plan* p, void* out, const void* x, T alpha, const void* y, int ey, int e,
                          cudaStream_t st) {
  const Dims d{(int)p->dom.nx, (int)p->dom.ny, (int)p->dom.nz, p->strides[1], p->strides[0]};
  auto org = [&](const void* b) { return b ? static_cast<const T*>(b) + p->offset : nullptr; };
  const int kb = tuned_kb(kBoxKB);
  return launch<combine_kernel<T>>(tile_grid(d.nx + 2 * e, d.ny + 2 * e, d.nz, 32, 32, kb), 0, st,
                                   static_cast<T*>(out) + p->offset, org(x), alpha, org(y), ey, d, e, kb);
}

// Stages 1-3: (u1, v1), (tu, tv), (u2, v2) into the workspace.
template <class T>
oeb_status run_stages_123(oeb_chain_plan* p, const typename Abi<T>::Fields* f, const oeb_chain_scalars* s,
                          void* stream) {
  using A = Abi<T>;
  using M3 = typename A::M3;
  using M1 = typename A::M1;
  const oeb_domain d1 = widen_dom(p->dom, kE1), d2 = widen_dom(p->dom, kE2);
  {
    const M3 o_u = wsw<T>(p, p->u1, kE1), o_v = wsw<T>(p, p->v1, kE1);
    const M3 u = widen(f->u, kE1), v = widen(f->v, kE1), ut = widen(f->utens, kE1), vt = widen(f->vtens, kE1),
             w = widen(f->wgtfac, kE1), pp = widen(f->ppuv, kE1), h = widen(f->hhl, kE1), r = widen(f->rho, kE1);
    const M1 fx = widen1(f->fx, kE1);
    OEB_TRY(A::fastwavesuv(&o_u, &o_v, &u, &v, &ut, &vt, &w, &pp, &h, &r, &fx, T(s->edadlat), T(s->dt), &d1, stream));
  }
  const M1 a0 = widen1(f->acrlat0, kE2), a1 = widen1(f->acrlat1, kE2), t0 = widen1(f->tgrlatda0, kE2),
           t1 = widen1(f->tgrlatda1, kE2);
  const M3 u = wsw<T>(p, p->u1, kE2), v = wsw<T>(p, p->v1, kE2);
  if (tuned_fusion() & OEB_FUSE_HADV_UPDATE) {  // stages 2 and 3 in one kernel: (u2, v2) directly
    const M3 o_u = wsw<T>(p, p->u2, kE2), o_v = wsw<T>(p, p->v2, kE2);
    return hadvuv5th_update(&o_u, &o_v, &u, &v, &a0, &a1, &t0, &t1, T(s->eddlat), T(s->eddlon), T(s->dt_adv), &d2,
                            stream);
  }
  {
    const M3 o_u = wsw<T>(p, p->tu, kE2), o_v = wsw<T>(p, p->tv, kE2);
    OEB_TRY(A::hadvuv5th(&o_u, &o_v, &u, &v, &a0, &a1, &t0, &t1, T(s->eddlat), T(s->eddlon), &d2, stream));
  }
  if (validating()) return OEB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  OEB_TRY(launch_combine<T>(p, p->u2, p->tu, T(s->dt_adv), p->u1, kE2, kE2, st));
  return launch_combine<T>(p, p->v2, p->tv, T(s->dt_adv), p->v1, kE2, kE2, st);
}

// Stage 4 on (u2, v2) into (uo, vo), widened by 3.
template <class T>
oeb_status run_stage_4(oeb_chain_plan* p, const typename Abi<T>::Fields* f, const oeb_chain_scalars* s,
                       const typename Abi<T>::M3* uo, const typename Abi<T>::M3* vo, void* stream) {
  using A = Abi<T>;
  using M3 = typename A::M3;
  using M1 = typename A::M1;
  const oeb_domain d3 = widen_dom(p->dom, kE3);
  const M3 o_u = widen(uo, kE3), o_v = widen(vo, kE3);
  const M3 u = wsw<T>(p, p->u2, kE3), v = wsw<T>(p, p->v2, kE3),
           m = widen(f->mask, kE3);
  const M1 c0 = widen1(f->crlavo, kE3), c1 = widen1(f->crlavu, kE3), c2 = widen1(f->crlato, kE3),
           c3 = widen1(f->crlatu, kE3), a0 = widen1(f->smag_acrlat0, kE3);
  return A::hdiffsmag(&o_u, &o_v, &u, &v, &m, &c0, &c1, &c2, &c3, &a0, T(s->eddlat), T(s->eddlon), T(s->tau_smag),
                      T(s->weight_smag), &d3, stream);
}

template <class T>
oeb_status chain_forward(oeb_chain_plan* p, const typename Abi<T>::Fields* f, const oeb_chain_scalars* s,
                         const typename Abi<T>::M3* uout, const typename Abi<T>::M3* vout,
                         const typename Abi<T>::M3* fx1, const typename Abi<T>::M3* fy1, void* stream) {
  using A = Abi<T>;
  using M3 = typename A::M3;
  OEB_TRY(check_plan<T>(p, OEB_CHAIN_FORWARD));
  if (!s) return OEB_ERR_NULL;
  OEB_TRY(check_inputs<T>(f));
  OEB_TRY(check_ij_halo(uout, kE3));
  OEB_TRY(check_ij_halo(vout, kE3));
  if (!fx1 || !fy1) return OEB_ERR_NULL;
  auto run = [&]() -> oeb_status {
    oeb_status st = run_stages_123<T>(p, f, s, stream);
    if (st == OEB_OK) st = run_stage_4<T>(p, f, s, uout, vout, stream);
    if (st == OEB_OK) {
      const M3 qi = ws<T>(p, p->qi), qj = ws<T>(p, p->qj), fx2 = ws<T>(p, p->fx2), fy2 = ws<T>(p, p->fy2);
      st = A::fvtp2d(&qi, &qj, fx1, &fx2, fy1, &fy2, uout, f->crx, f->cry, f->ra_x, f->ra_y, f->xfx, f->yfx, f->area,
                     T(s->ppm_p1), T(s->ppm_p2), &p->dom, stream);
    }
    return st;
  };
  {
    ValidateOnly guard;  // every stage is checked before any is launched
    OEB_TRY(run());
  }
  return run();
}

template <class T>
oeb_status chain_tl(oeb_chain_plan* p, const typename Abi<T>::Fields* f, const oeb_chain_scalars* s,
                    const typename Abi<T>::M3* du, const typename Abi<T>::M3* dv, const typename Abi<T>::M3* duout,
                    const typename Abi<T>::M3* dvout, const typename Abi<T>::M3* dfx1,
                    const typename Abi<T>::M3* dfy1, void* stream) {
  using A = Abi<T>;
  using M3 = typename A::M3;
  using M1 = typename A::M1;
  OEB_TRY(check_plan<T>(p, OEB_CHAIN_TL));
  if (!s) return OEB_ERR_NULL;
  OEB_TRY(check_inputs<T>(f));
  OEB_TRY(check_ij_halo(du, kE1));
  OEB_TRY(check_ij_halo(dv, kE1));
  OEB_TRY(check_ij_halo(duout, kE3));
  OEB_TRY(check_ij_halo(dvout, kE3));
  if (!dfx1 || !dfy1) return OEB_ERR_NULL;
  const oeb_domain d1 = widen_dom(p->dom, kE1), d2 = widen_dom(p->dom, kE2), d3 = widen_dom(p->dom, kE3);
  auto run = [&]() -> oeb_status {
    oeb_status st = run_stages_123<T>(p, f, s, stream);
    if (st == OEB_OK) {  // d(u1, v1)
      const M3 o_u = wsw<T>(p, p->du1, kE1), o_v = wsw<T>(p, p->dv1, kE1);
      const M3 u = widen(f->u, kE1), v = widen(f->v, kE1), ut = widen(f->utens, kE1), vt = widen(f->vtens, kE1),
               w = widen(f->wgtfac, kE1), pp = widen(f->ppuv, kE1), h = widen(f->hhl, kE1), r = widen(f->rho, kE1),
               du1 = widen(du, kE1), dv1 = widen(dv, kE1), z = wsw<T>(p, p->zero, kE1);
      const M1 fx = widen1(f->fx, kE1);
      st = A::fastwavesuv_tl(&o_u, &o_v, &u, &v, &ut, &vt, &w, &pp, &h, &r, &fx, &du1, &dv1, &z, &z, &z,
                             T(s->edadlat), T(s->dt), &d1, stream);
    }
    if (st == OEB_OK) {  // d(tu, tv)
      const M3 o_u = wsw<T>(p, p->dtu, kE2), o_v = wsw<T>(p, p->dtv, kE2);
      const M3 u = wsw<T>(p, p->u1, kE2), v = wsw<T>(p, p->v1, kE2),
               du1 = wsw<T>(p, p->du1, kE2), dv1 = wsw<T>(p, p->dv1, kE2);
      const M1 a0 = widen1(f->acrlat0, kE2), a1 = widen1(f->acrlat1, kE2), t0 = widen1(f->tgrlatda0, kE2),
               t1 = widen1(f->tgrlatda1, kE2);
      st = A::hadvuv5th_tl(&o_u, &o_v, &u, &v, &a0, &a1, &t0, &t1, &du1, &dv1, T(s->eddlat), T(s->eddlon), &d2,
                           stream);
    }
    if (st == OEB_OK && !validating()) {  // d(u2, v2)
      cudaStream_t cs = (cudaStream_t)stream;
      st = launch_combine<T>(p, p->du2, p->dtu, T(s->dt_adv), p->du1, kE2, kE2, cs);
      if (st == OEB_OK) st = launch_combine<T>(p, p->dv2, p->dtv, T(s->dt_adv), p->dv1, kE2, kE2, cs);
    }
    if (st == OEB_OK) {  // the new (u, v) and its perturbation
      const M3 u3 = ws<T>(p, p->u3), v3 = ws<T>(p, p->v3);
      st = run_stage_4<T>(p, f, s, &u3, &v3, stream);
    }
    if (st == OEB_OK) {
      const M3 o_u = widen(duout, kE3), o_v = widen(dvout, kE3);
      const M3 u = wsw<T>(p, p->u2, kE3), v = wsw<T>(p, p->v2, kE3),
               m = widen(f->mask, kE3), du2 = wsw<T>(p, p->du2, kE3),
               dv2 = wsw<T>(p, p->dv2, kE3);
      const M1 c0 = widen1(f->crlavo, kE3), c1 = widen1(f->crlavu, kE3), c2 = widen1(f->crlato, kE3),
               c3 = widen1(f->crlatu, kE3), a0 = widen1(f->smag_acrlat0, kE3);
      st = A::hdiffsmag_tl(&o_u, &o_v, &u, &v, &m, &c0, &c1, &c2, &c3, &a0, &du2, &dv2, T(s->eddlat), T(s->eddlon),
                           T(s->tau_smag), T(s->weight_smag), &d3, stream);
    }
    if (st == OEB_OK) {  // d(fx1, fy1), q = the new u
      const M3 u3 = ws<T>(p, p->u3), qi = ws<T>(p, p->dqi), qj = ws<T>(p, p->dqj), fx2 = ws<T>(p, p->dfx2),
               fy2 = ws<T>(p, p->dfy2);
      st = A::fvtp2d_tl(&qi, &qj, dfx1, &fx2, dfy1, &fy2, &u3, f->crx, f->cry, f->ra_x, f->ra_y, f->xfx, f->yfx,
                        f->area, duout, T(s->ppm_p1), T(s->ppm_p2), &p->dom, stream);
    }
    return st;
  };
  {
    ValidateOnly guard;
    OEB_TRY(run());
  }
  return run();
}

template <class T>
oeb_status chain_adj(oeb_chain_plan* p, const typename Abi<T>::Fields* f, const oeb_chain_scalars* s,
                     const typename Abi<T>::M3* uoutb, const typename Abi<T>::M3* voutb,
                     const typename Abi<T>::M3* fx1b, const typename Abi<T>::M3* fy1b, const typename Abi<T>::M3* ub,
                     const typename Abi<T>::M3* vb, void* stream) {
  using A = Abi<T>;
  using M3 = typename A::M3;
  using M1 = typename A::M1;
  OEB_TRY(check_plan<T>(p, OEB_CHAIN_ADJOINT));
  if (!s) return OEB_ERR_NULL;
  OEB_TRY(check_inputs<T>(f));
  OEB_TRY(check_ij_halo(ub, kE1));
  OEB_TRY(check_ij_halo(vb, kE1));
  if (!uoutb || !voutb || !fx1b || !fy1b) return OEB_ERR_NULL;
  // the seeds are read on the interior, in the plan's layout
  const M3* seeds[] = {uoutb, voutb};
  for (const M3* m : seeds) {
    if (m->offset != p->offset) return OEB_ERR_LAYOUT;
    for (int r = 0; r < 3; ++r)
      if (m->sizes[r] != p->sizes[r] || m->strides[r] != p->strides[r]) return OEB_ERR_LAYOUT;
  }
  const oeb_domain d1 = widen_dom(p->dom, kE1), d2 = widen_dom(p->dom, kE2), d3 = widen_dom(p->dom, kE3);
  cudaStream_t cs = (cudaStream_t)stream;
  const bool fused = (tuned_fusion() & OEB_FUSE_HADV_UPDATE) != 0;
  auto run = [&]() -> oeb_status {
    // recompute the forward intermediates
    oeb_status st = run_stages_123<T>(p, f, s, stream);
    if (st == OEB_OK) {
      const M3 u3 = ws<T>(p, p->u3), v3 = ws<T>(p, p->v3);
      st = run_stage_4<T>(p, f, s, &u3, &v3, stream);
    }
    if (st == OEB_OK) {  // fvtp2d: qb on the interior widened by 3
      const M3 qb = ws<T>(p, p->qb), u3 = ws<T>(p, p->u3);
      st = A::fvtp2d_adj(&qb, &u3, f->crx, f->cry, f->ra_x, f->ra_y, f->xfx, f->yfx, f->area, fx1b, fy1b,
                         T(s->ppm_p1), T(s->ppm_p2), &p->dom, stream);
    }
    if (st == OEB_OK && !validating()) {  // seeds of (uout, vout) on the interior
      st = launch_combine<T>(p, p->qb, p->qb, T(1), uoutb->aligned, 0, kE3, cs);
      if (st == OEB_OK) st = launch_combine<T>(p, p->v3b, nullptr, T(1), voutb->aligned, 0, kE3, cs);
    }
    if (st == OEB_OK) {  // hdiffsmag: (u2b, v2b) on the interior widened by 4
      const M3 o_u = wsw<T>(p, p->u2b, kE3), o_v = wsw<T>(p, p->v2b, kE3);
      const M3 u = wsw<T>(p, p->u2, kE3), v = wsw<T>(p, p->v2, kE3),
               m = widen(f->mask, kE3), yu = wsw<T>(p, p->qb, kE3),
               yv = wsw<T>(p, p->v3b, kE3);
      const M1 c0 = widen1(f->crlavo, kE3), c1 = widen1(f->crlavu, kE3), c2 = widen1(f->crlato, kE3),
               c3 = widen1(f->crlatu, kE3), a0 = widen1(f->smag_acrlat0, kE3);
      st = A::hdiffsmag_adj(&o_u, &o_v, &u, &v, &m, &c0, &c1, &c2, &c3, &a0, &yu, &yv, T(s->eddlat), T(s->eddlon),
                            T(s->tau_smag), T(s->weight_smag), &d3, stream);
    }
    if (st == OEB_OK) {  // hadvuv5th on (u2b, v2b): (wu, wv) on the interior widened by 7
      const M3 o_u = wsw<T>(p, p->wu, kE2), o_v = wsw<T>(p, p->wv, kE2);
      const M3 u = wsw<T>(p, p->u1, kE2), v = wsw<T>(p, p->v1, kE2),
               yu = wsw<T>(p, p->u2b, kE2), yv = wsw<T>(p, p->v2b, kE2);
      const M1 a0 = widen1(f->acrlat0, kE2), a1 = widen1(f->acrlat1, kE2), t0 = widen1(f->tgrlatda0, kE2),
               t1 = widen1(f->tgrlatda1, kE2);
      st = fused ? hadvuv5th_adj_update(&o_u, &o_v, &u, &v, &a0, &a1, &t0, &t1, &yu, &yv, T(s->eddlat),
                                        T(s->eddlon), T(s->dt_adv), &d2, stream)
                 : A::hadvuv5th_adj(&o_u, &o_v, &u, &v, &a0, &a1, &t0, &t1, &yu, &yv, T(s->eddlat), T(s->eddlon),
                                    &d2, stream);
    }
    // stage 3: (u1b, v1b) = dt_adv (wu, wv) + (u2b, v2b), unless the gather above added it
    if (st == OEB_OK && !validating() && !fused) {
      st = launch_combine<T>(p, p->wu, p->wu, T(s->dt_adv), p->u2b, kE2, kE1, cs);
      if (st == OEB_OK) st = launch_combine<T>(p, p->wv, p->wv, T(s->dt_adv), p->v2b, kE2, kE1, cs);
    }
    if (st == OEB_OK) {  // fastwavesuv: (ub, vb) on the interior widened by 7
      const M3 o_u = widen(ub, kE1), o_v = widen(vb, kE1), o_ut = wsw<T>(p, p->utb, kE1),
               o_vt = wsw<T>(p, p->vtb, kE1), o_pp = wsw<T>(p, p->ppb, kE1);
      const M3 u = widen(f->u, kE1), v = widen(f->v, kE1), ut = widen(f->utens, kE1), vt = widen(f->vtens, kE1),
               w = widen(f->wgtfac, kE1), pp = widen(f->ppuv, kE1), h = widen(f->hhl, kE1), r = widen(f->rho, kE1),
               yu = wsw<T>(p, p->wu, kE1), yv = wsw<T>(p, p->wv, kE1);
      const M1 fx = widen1(f->fx, kE1);
      st = A::fastwavesuv_adj(&o_u, &o_v, &o_ut, &o_vt, &o_pp, &u, &v, &ut, &vt, &w, &pp, &h, &r, &fx, &yu, &yv,
                              T(s->edadlat), T(s->dt), &d1, stream);
    }
    return st;
  };
  {
    ValidateOnly guard;
    OEB_TRY(run());
  }
  return run();
}

template <class T, class M3>
oeb_status plan_create(const M3* like, const oeb_domain* dom, int modes, oeb_chain_plan** out) {
  if (!like || !dom || !out) return OEB_ERR_NULL;
  *out = nullptr;
  if (modes <= 0 || modes > (OEB_CHAIN_FORWARD | OEB_CHAIN_TL | OEB_CHAIN_ADJOINT)) return OEB_ERR_ARGUMENT;
  OEB_TRY(check_domain(dom));
  OEB_TRY(check_ij_halo(like, kE1));
  {
    // the template must hold the widest stage box: interior + 8 in i and j, k halo 1
    Grid<T> g;
    OEB_TRY((check_field3<T>(like, *dom, Reach{kE1, kE1 + 1, kE1, kE1 + 1, 1, 1}, &g)));
  }
  oeb_chain_plan* p = new (std::nothrow) oeb_chain_plan();
  if (!p) return OEB_ERR_ALLOC;
  p->elem = (int)sizeof(T);
  p->modes = modes;
  p->dom = *dom;
  p->offset = like->offset;
  for (int r = 0; r < 3; ++r) {
    p->sizes[r] = like->sizes[r];
    p->strides[r] = like->strides[r];
  }
  p->field_bytes = (size_t)((like->sizes[0] - 1) * like->strides[0] + (like->sizes[1] - 1) * like->strides[1] +
                            like->sizes[2]) *
                   sizeof(T);
  cudaError_t e = cudaGetDevice(&p->device);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e);
  }
  std::vector<void**> want;
  const bool fwd = modes & OEB_CHAIN_FORWARD, tl = modes & OEB_CHAIN_TL, adj = modes & OEB_CHAIN_ADJOINT;
  for (void** w : {&p->u1, &p->v1, &p->tu, &p->tv, &p->u2, &p->v2}) want.push_back(w);
  if (fwd || adj) for (void** w : {&p->qi, &p->qj, &p->fx2, &p->fy2}) want.push_back(w);
  if (tl || adj) for (void** w : {&p->u3, &p->v3}) want.push_back(w);
  if (tl)
    for (void** w : {&p->du1, &p->dv1, &p->dtu, &p->dtv, &p->du2, &p->dv2, &p->dqi, &p->dqj, &p->dfx2, &p->dfy2,
                     &p->zero})
      want.push_back(w);
  for (void** w : want) {
    void* b = nullptr;
    e = cudaMalloc(&b, p->field_bytes);
    if (e != cudaSuccess) {
      for (void* q : p->bufs) cudaFree(q);
      delete p;
      cuda_fail(e);
      return OEB_ERR_ALLOC;
    }
    p->bufs.push_back(b);
    *w = b;
  }
  if (adj) {
    // The adjoint step's own fields share the buffers of fields that are dead while they are
    // live (a plan runs one call at a time, and every call writes a field before it reads it):
    //   qi, qj, fx2, fy2 are written only by the forward step's fvtp2d and read by nothing;
    //   tu, tv are dead once stage 3 has formed (u2, v2); v3 is never read by the adjoint
    //   step and u3 only by its fvtp2d adjoint.  In the adjoint step's order:
    //     qb (fvtp2d adjoint .. hdiffsmag adjoint)        in qi
    //     v3b (seed combine .. hdiffsmag adjoint)         in qj
    //     u2b, v2b (hdiffsmag adjoint .. stage-3 combine) in fx2, fy2
    //     wu, wv (hadvuv5th adjoint .. fastwavesuv adj.)  in tu, tv
    //     ppb (fastwavesuv adjoint; qb is dead by then)   in qi
    //     utb, vtb (fastwavesuv adjoint)                  in v3, u3
    // No call reads and writes one buffer under two names (every stage's outputs and inputs
    // stay distinct: the entry points check it).  12 fields instead of 21.
    p->qb = p->qi;
    p->v3b = p->qj;
    p->u2b = p->fx2;
    p->v2b = p->fy2;
    p->wu = p->tu;
    p->wv = p->tv;
    p->ppb = p->qi;
    p->utb = p->v3;
    p->vtb = p->u3;
  }
  if (p->zero) {
    e = cudaMemset(p->zero, 0, p->field_bytes);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      for (void* q : p->bufs) cudaFree(q);
      delete p;
      return cuda_fail(e);
    }
  }
  *out = p;
  return OEB_OK;
}

}  // namespace
}  // namespace oeb

#ifndef OEB_BODIES_ONLY  // the entry points

using namespace oeb;

extern "C" oeb_status oeb_chain_plan_create_f64(const oeb_memref3d_f64* like, const oeb_domain* dom, int modes,
                                                oeb_chain_plan** out) {
  return plan_create<double>(like, dom, modes, out);
}
extern "C" oeb_status oeb_chain_plan_create_f32(const oeb_memref3d_f32* like, const oeb_domain* dom, int modes,
                                                oeb_chain_plan** out) {
  return plan_create<float>(like, dom, modes, out);
}
extern "C" size_t oeb_chain_plan_bytes(const oeb_chain_plan* p) { return p ? p->bufs.size() * p->field_bytes : 0; }
extern "C" oeb_status oeb_chain_plan_destroy(oeb_chain_plan* p) {
  if (!p) return OEB_ERR_NULL;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(p->device);
  cudaError_t e = cudaDeviceSynchronize();
  for (void* b : p->bufs) cudaFree(b);
  cudaSetDevice(prev);
  delete p;
  return e == cudaSuccess ? OEB_OK : cuda_fail(e);
}

#define OEB_CHAIN_ENTRIES(S, T)                                                                                    \
  extern "C" oeb_status oeb_chain_forward_##S(oeb_chain_plan* plan, const oeb_chain_fields_##S* f,                 \
                                              const oeb_chain_scalars* s, const oeb_memref3d_##S* uout,           \
                                              const oeb_memref3d_##S* vout, const oeb_memref3d_##S* fx1,          \
                                              const oeb_memref3d_##S* fy1, void* stream) {                        \
    return chain_forward<T>(plan, f, s, uout, vout, fx1, fy1, stream);                                             \
  }                                                                                                                \
  extern "C" oeb_status oeb_chain_tl_##S(oeb_chain_plan* plan, const oeb_chain_fields_##S* f,                      \
                                         const oeb_chain_scalars* s, const oeb_memref3d_##S* du,                   \
                                         const oeb_memref3d_##S* dv, const oeb_memref3d_##S* duout,               \
                                         const oeb_memref3d_##S* dvout, const oeb_memref3d_##S* dfx1,             \
                                         const oeb_memref3d_##S* dfy1, void* stream) {                            \
    return chain_tl<T>(plan, f, s, du, dv, duout, dvout, dfx1, dfy1, stream);                                      \
  }                                                                                                                \
  extern "C" oeb_status oeb_chain_adj_##S(oeb_chain_plan* plan, const oeb_chain_fields_##S* f,                     \
                                          const oeb_chain_scalars* s, const oeb_memref3d_##S* uoutb,              \
                                          const oeb_memref3d_##S* voutb, const oeb_memref3d_##S* fx1b,            \
                                          const oeb_memref3d_##S* fy1b, const oeb_memref3d_##S* ub,               \
                                          const oeb_memref3d_##S* vb, void* stream) {                             \
    return chain_adj<T>(plan, f, s, uoutb, voutb, fx1b, fy1b, ub, vb, stream);                                     \
  }

OEB_CHAIN_ENTRIES(f64, double)
OEB_CHAIN_ENTRIES(f32, float)

extern "C" oeb_status oeb_graph_begin(void* stream) {
  if (!stream) return OEB_ERR_ARGUMENT;  // the legacy default stream cannot be captured
  if (capture_counting()) return OEB_ERR_ARGUMENT;  // one capture per thread at a time
  cudaMemPool_t pool;
  OEB_TRY(device_pool(&pool));
  OEB_CUDA_TRY(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
  capture_count_begin();
  return OEB_OK;
}

extern "C" oeb_status oeb_graph_end(void* stream, oeb_graph** out) {
  if (!out) return OEB_ERR_NULL;
  *out = nullptr;
  if (!capture_counting()) return OEB_ERR_ARGUMENT;
  const uint64_t kernels = capture_count_end();
  cudaGraph_t g = nullptr;
  OEB_CUDA_TRY(cudaStreamEndCapture((cudaStream_t)stream, &g));
  cudaGraphExec_t x = nullptr;
  cudaError_t e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(e);
  }
  oeb_graph* r = new (std::nothrow) oeb_graph{g, x, kernels};
  if (!r) {
    cudaGraphExecDestroy(x);
    cudaGraphDestroy(g);
    return OEB_ERR_ALLOC;
  }
  *out = r;
  return OEB_OK;
}

extern "C" oeb_status oeb_graph_launch(oeb_graph* g, void* stream) {
  if (!g) return OEB_ERR_NULL;
  OEB_CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  count_launches(g->kernels);
  return OEB_OK;
}

extern "C" uint64_t oeb_graph_kernel_count(const oeb_graph* g) { return g ? g->kernels : 0; }

extern "C" oeb_status oeb_graph_destroy(oeb_graph* g) {
  if (!g) return OEB_ERR_NULL;
  cudaGraphExecDestroy(g->exec);
  cudaGraphDestroy(g->graph);
  delete g;
  return OEB_OK;
}

#endif  // OEB_BODIES_ONLY
