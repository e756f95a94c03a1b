/*
 * oracle_impl.h -- body of the CPU oracle, included once per element type by oeb_oracle.c.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference kernels, used
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.  The
 * product (the CUDA library) never links, loads or calls it.
 *
 * Each function restates the reference's oracle variant -- `<k>_openmp` for nine kernels and
 * the serial `fvtp2d` -- with the same loop nests, the same OpenMP loop, the same
 * parenthesisation and the same literal types (a bare `-4.0` stays a double literal even
 * when T is float, `ElementType(2.0)` becomes `(T)2.0`), so that, compiled with
 * -ffp-contract=off, it reproduces the reference bit for bit.  Scratch fields are written
 * exactly where the reference writes them.
 *
 * The only generalisation: the reference's global `domain_size` bounds both the i and the j
 * loops (src/<k>.cpp:4); here i runs to nx and j to ny (nx == ny reproduces the reference).
 *
 * Required before inclusion: T, SUF (f64/f32), M3, M1 (memref types), SQRT.
 */

#define OEB_CAT2(a, b) a##b
#define OEB_CAT(a, b) OEB_CAT2(a, b)
#define OEB_FN(name) OEB_CAT(oeb_oracle_##name##_, SUF)

/* include/util.h:82-94: aligned[offset + strides[2]*i + strides[1]*j + strides[0]*k] */
#define A3(f, i, j, k) \
  ((f)->aligned[(f)->offset + (f)->strides[2] * (i) + (f)->strides[1] * (j) + (f)->strides[0] * (k)])
/* include/util.h:58-60 */
#define A1(f, j) ((f)->aligned[(f)->offset + (f)->strides[0] * (j)])

/* include/util.h:17-18 */
#define OEB_EARTH_RADIUS ((T)6371.229e3)
#define OEB_EARTH_RADIUS_RECIP ((T)1.0 / OEB_EARTH_RADIUS)

/* kernels/laplace.h:34-43 (laplace_openmp) */
void OEB_FN(laplace)(const M3* in, const M3* out, int64_t nx, int64_t ny, int64_t nz) {
#pragma omp parallel for
  for (int64_t i = 0; i < nx; ++i) {
    for (int64_t j = 0; j < ny; ++j) {
      for (int64_t k = 0; k < nz; ++k) {
        A3(out, i, j, k) = -4.0 * A3(in, i, j, k) +
                           ((A3(in, i - 1, j, k) + A3(in, i + 1, j, k)) + (A3(in, i, j + 1, k) + A3(in, i, j - 1, k)));
      }
    }
  }
}

/* kernels/hdiffsa.h:95-123 (hdiffsa_openmp) */
void OEB_FN(hdiffsa)(const M3* out, const M3* in, const M3* mask, const M1* crlato, const M1* crlatu, const M3* lap,
                     const M3* flx, const M3* fly, int64_t nx, int64_t ny, int64_t nz) {
  (void)lap; /* the openmp variant keeps the laplacian in registers (hdiffsa.h:101-103) */
#pragma omp parallel for
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -1; i < nx + 1; ++i) {
      for (int64_t j = -1; j < ny + 1; ++j) {
        T lap_ijk = A3(in, i - 1, j, k) + A3(in, i + 1, j, k) - (T)2.0 * A3(in, i, j, k) +
                    A1(crlato, j) * (A3(in, i, j + 1, k) - A3(in, i, j, k)) +
                    A1(crlatu, j) * (A3(in, i, j - 1, k) - A3(in, i, j, k));
        T lap_i1jk = A3(in, i, j, k) + A3(in, i + 2, j, k) - (T)2.0 * A3(in, i + 1, j, k) +
                     A1(crlato, j) * (A3(in, i + 1, j + 1, k) - A3(in, i + 1, j, k)) +
                     A1(crlatu, j) * (A3(in, i + 1, j - 1, k) - A3(in, i + 1, j, k));
        T lap_ij1k = A3(in, i - 1, j + 1, k) + A3(in, i + 1, j + 1, k) - (T)2.0 * A3(in, i, j + 1, k) +
                     A1(crlato, j + 1) * (A3(in, i, j + 2, k) - A3(in, i, j + 1, k)) +
                     A1(crlatu, j + 1) * (A3(in, i, j, k) - A3(in, i, j + 1, k));

        A3(flx, i, j, k) = lap_i1jk - lap_ijk;
        if (A3(flx, i, j, k) * (A3(in, i + 1, j, k) - A3(in, i, j, k)) > 0) {
          A3(flx, i, j, k) = 0;
        }
        A3(fly, i, j, k) = A1(crlato, j) * (lap_ij1k - lap_ijk);
        if (A3(fly, i, j, k) * (A3(in, i, j + 1, k) - A3(in, i, j, k)) > 0) {
          A3(fly, i, j, k) = 0;
        }
      }
    }
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(out, i, j, k) = A3(in, i, j, k) + (A3(flx, i - 1, j, k) - A3(flx, i, j, k) + A3(fly, i, j - 1, k) -
                                              A3(fly, i, j, k)) * A3(mask, i, j, k);
      }
    }
  }
}

/* std::max(a, b) is (a < b) ? b : a and std::min(a, b) is (b < a) ? b : a (libstdc++), which
 * fixes the result for NaN and signed zeros; hdiffsmag.h:236 and :251 use them as
 * min(0.5, max(0.0, x)). */
static inline T OEB_CAT(oeb_clamp_smag_, SUF)(T x) {
  T lo = ((T)0.0 < x) ? x : (T)0.0;
  return (lo < (T)0.5) ? lo : (T)0.5;
}

/* kernels/hdiffsmag.h:205-263 (hdiffsmag_openmp) */
void OEB_FN(hdiffsmag)(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* mask,
                       const M1* crlavo, const M1* crlavu, const M1* crlato, const M1* crlatu, const M1* acrlat0,
                       const M3* T_sqr_s, const M3* S_sqr_uv, T eddlat, T eddlon, T tau_smag, T weight_smag,
                       int64_t nx, int64_t ny, int64_t nz) {
  (void)T_sqr_s;
  (void)S_sqr_uv;
#pragma omp parallel for
  for (int64_t i = 0; i < nx; i++) {
    for (int64_t j = 0; j < ny; j++) {
      for (int64_t k = 0; k < nz; k++) {
        T T_s_ijk = (A3(vin, i, j - 1, k) - A3(vin, i, j, k)) * eddlat * OEB_EARTH_RADIUS_RECIP -
                    (A3(uin, i - 1, j, k) - A3(uin, i, j, k)) * A1(acrlat0, j) * eddlon;
        T T_sqr_s_ijk = T_s_ijk * T_s_ijk;
        T T_s_i1jk = (A3(vin, i + 1, j - 1, k) - A3(vin, i + 1, j, k)) * eddlat * OEB_EARTH_RADIUS_RECIP -
                     (A3(uin, i, j, k) - A3(uin, i + 1, j, k)) * A1(acrlat0, j) * eddlon;
        T T_sqr_s_i1jk = T_s_i1jk * T_s_i1jk;
        T T_s_ij1k = (A3(vin, i, j, k) - A3(vin, i, j + 1, k)) * eddlat * OEB_EARTH_RADIUS_RECIP -
                     (A3(uin, i - 1, j + 1, k) - A3(uin, i, j + 1, k)) * A1(acrlat0, j + 1) * eddlon;
        T T_sqr_s_ij1k = T_s_ij1k * T_s_ij1k;

        T S_uv_ijk = (A3(uin, i, j + 1, k) - A3(uin, i, j, k)) * eddlat * OEB_EARTH_RADIUS_RECIP +
                     (A3(vin, i + 1, j, k) - A3(vin, i, j, k)) * A1(acrlat0, j) * eddlon;
        T S_sqr_uv_ijk = S_uv_ijk * S_uv_ijk;
        T S_uv_im1jk = (A3(uin, i - 1, j + 1, k) - A3(uin, i - 1, j, k)) * eddlat * OEB_EARTH_RADIUS_RECIP +
                       (A3(vin, i, j, k) - A3(vin, i - 1, j, k)) * A1(acrlat0, j) * eddlon;
        T S_sqr_uv_im1jk = S_uv_im1jk * S_uv_im1jk;
        T S_uv_ijm1k = (A3(uin, i, j, k) - A3(uin, i, j - 1, k)) * eddlat * OEB_EARTH_RADIUS_RECIP +
                       (A3(vin, i + 1, j - 1, k) - A3(vin, i, j - 1, k)) * A1(acrlat0, j - 1) * eddlon;
        T S_sqr_uv_ijm1k = S_uv_ijm1k * S_uv_ijm1k;

        const T hdweight = weight_smag * A3(mask, i, j, k);

        T smag_u = tau_smag * SQRT((T)0.5 * (T_sqr_s_i1jk + T_sqr_s_ijk) + (T)0.5 * (S_sqr_uv_ijm1k + S_sqr_uv_ijk)) -
                   hdweight;
        smag_u = OEB_CAT(oeb_clamp_smag_, SUF)(smag_u);
        const T lapu = A3(uin, i + 1, j, k) + A3(uin, i - 1, j, k) - (T)2.0 * A3(uin, i, j, k) +
                       A1(crlato, j) * (A3(uin, i, j + 1, k) - A3(uin, i, j, k)) +
                       A1(crlatu, j) * (A3(uin, i, j - 1, k) - A3(uin, i, j, k));
        A3(uout, i, j, k) = A3(uin, i, j, k) + smag_u * lapu;

        T smag_v = tau_smag * SQRT((T)0.5 * (T_sqr_s_ij1k + T_sqr_s_ijk) + (T)0.5 * (S_sqr_uv_im1jk + S_sqr_uv_ijk)) -
                   hdweight;
        smag_v = OEB_CAT(oeb_clamp_smag_, SUF)(smag_v);
        const T lapv = A3(vin, i + 1, j, k) + A3(vin, i - 1, j, k) - (T)2.0 * A3(vin, i, j, k) +
                       A1(crlavo, j) * (A3(vin, i, j + 1, k) - A3(vin, i, j, k)) +
                       A1(crlavu, j) * (A3(vin, i, j - 1, k) - A3(vin, i, j, k));
        A3(vout, i, j, k) = A3(vin, i, j, k) + smag_v * lapv;
      }
    }
  }
}

/* kernels/hadvuv.h:4-27 (3rd-order advectionDriver; the field is passed by value there) */
static T OEB_CAT(oeb_adv3_, SUF)(const M3* f, int64_t i, int64_t j, int64_t k, T uavg, T vavg, T eddlat, T eddlon) {
  T result_x = 0.0;
  T result_y = 0.0;
  if (uavg > 0) {
    result_x = uavg * ((T)(-1.0) / (T)(6.0) * A3(f, i - 2, j, k) + A3(f, i - 1, j, k) + (T)(-0.5) * A3(f, i, j, k) +
                       (T)(-1.0) / (T)(3.0) * A3(f, i + 1, j, k));
  } else {
    result_x = -uavg * ((T)(-1.0) / (T)(3.0) * A3(f, i - 1, j, k) + (T)(-0.5) * A3(f, i, j, k) + A3(f, i + 1, j, k) +
                        (T)(-1.0) / (T)(6.0) * A3(f, i + 2, j, k));
  }
  if (vavg > 0) {
    result_y = vavg * ((T)(-1.0) / (T)(6.0) * A3(f, i, j - 2, k) + A3(f, i, j - 1, k) + (T)(-0.5) * A3(f, i, j, k) +
                       (T)(-1.0) / (T)(3.0) * A3(f, i, j + 1, k));
  } else {
    result_y = -vavg * ((T)(-1.0) / (T)(3.0) * A3(f, i, j - 1, k) + (T)(-0.5) * A3(f, i, j, k) + A3(f, i, j + 1, k) +
                        (T)(-1.0) / (T)(6.0) * A3(f, i, j + 2, k));
  }
  return eddlat * result_x + eddlon * result_y;
}

/* kernels/hadvuv5th.h:4-39 (5th-order advectionDriver) */
static T OEB_CAT(oeb_adv5_, SUF)(const M3* f, int64_t i, int64_t j, int64_t k, T uavg, T vavg, T eddlat, T eddlon) {
  T result_x = 0.0;
  T result_y = 0.0;
  if (uavg > 0) {
    result_x = uavg * ((T)(1.0) / (T)(30.0) * A3(f, i - 3, j, k) + (T)(-1.0) / (T)(4.0) * A3(f, i - 2, j, k) +
                       A3(f, i - 1, j, k) + (T)(-1.0) / (T)(3.0) * A3(f, i, j, k) +
                       (T)(-1.0) / (T)(2.0) * A3(f, i + 1, j, k) + (T)(1.0) / (T)(20.0) * A3(f, i + 2, j, k));
  } else {
    result_x = -uavg * ((T)(1.0) / (T)(20.0) * A3(f, i - 2, j, k) + (T)(-1.0) / (T)(2.0) * A3(f, i - 1, j, k) +
                        (T)(-1.0) / (T)(3.0) * A3(f, i, j, k) + A3(f, i + 1, j, k) +
                        (T)(-1.0) / (T)(4.0) * A3(f, i + 2, j, k) + (T)(1.0) / (T)(30.0) * A3(f, i + 3, j, k));
  }
  if (vavg > 0) {
    result_y = vavg * ((T)(1.0) / (T)(30.0) * A3(f, i, j - 3, k) + (T)(-1.0) / (T)(4.0) * A3(f, i, j - 2, k) +
                       A3(f, i, j - 1, k) + (T)(-1.0) / (T)(3.0) * A3(f, i, j, k) +
                       (T)(-1.0) / (T)(2.0) * A3(f, i, j + 1, k) + (T)(1.0) / (T)(20.0) * A3(f, i, j + 2, k));
  } else {
    result_y = -vavg * ((T)(1.0) / (T)(20.0) * A3(f, i, j - 2, k) + (T)(-1.0) / (T)(2.0) * A3(f, i, j - 1, k) +
                        (T)(-1.0) / (T)(3.0) * A3(f, i, j, k) + A3(f, i, j + 1, k) +
                        (T)(-1.0) / (T)(4.0) * A3(f, i, j + 2, k) + (T)(1.0) / (T)(30.0) * A3(f, i, j + 3, k));
  }
  return eddlat * result_x + eddlon * result_y;
}

/* kernels/hadvuv.h:178-210 (hadvuv_openmp) and kernels/hadvuv5th.h:177-201 (hadvuv5th_openmp):
 * identical bodies apart from the advection driver. */
#define OEB_HADV_BODY(ADV)                                                                                          \
  for (int64_t k = 0; k < nz; ++k) {                                                                                \
    for (int64_t i = 0; i < nx; ++i) {                                                                              \
      for (int64_t j = 0; j < ny; ++j) {                                                                            \
        T u_atupos = ((T)1.0 / (T)3.0) * (A3(uin, i - 1, j, k) + A3(uin, i, j, k) + A3(uin, i + 1, j, k));          \
        T v_atupos = (T)0.25 * (A3(vin, i + 1, j, k) + A3(vin, i + 1, j - 1, k) + A3(vin, i, j, k) +                \
                                A3(vin, i, j - 1, k));                                                              \
        T u_avg = A1(acrlat0, j) * u_atupos;                                                                        \
        T v_avg = OEB_EARTH_RADIUS_RECIP * v_atupos;                                                                \
        T u_res = ADV(uin, i, j, k, u_avg, v_avg, eddlat, eddlon);                                                  \
        A3(uout, i, j, k) = u_res + A1(tgrlatda0, j) * A3(uin, i, j, k) * v_atupos;                                 \
        T u_atvpos = (T)0.25 * (A3(uin, i - 1, j, k) + A3(uin, i, j, k) + A3(uin, i, j + 1, k) +                    \
                                A3(uin, i - 1, j + 1, k));                                                          \
        T v_atvpos = (T)1.0 / (T)3.0 * (A3(vin, i, j - 1, k) + A3(vin, i, j, k) + A3(vin, i, j + 1, k));            \
        u_avg = A1(acrlat1, j) * u_atvpos;                                                                          \
        v_avg = OEB_EARTH_RADIUS_RECIP * v_atvpos;                                                                  \
        T v_res = ADV(vin, i, j, k, u_avg, v_avg, eddlat, eddlon);                                                  \
        A3(vout, i, j, k) = v_res - A1(tgrlatda1, j) * u_atvpos * u_atvpos;                                         \
      }                                                                                                             \
    }                                                                                                               \
  }

void OEB_FN(hadvuv)(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M1* acrlat0,
                    const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, const M3* uatupos,
                    const M3* vatupos, const M3* uatvpos, const M3* vatvpos, const M3* uavg, const M3* vavg,
                    const M3* ures, const M3* vres, T eddlat, T eddlon, int64_t nx, int64_t ny, int64_t nz) {
  /* the openmp variant keeps every intermediate in registers and never touches the scratch fields */
  (void)uatupos; (void)vatupos; (void)uatvpos; (void)vatvpos; (void)uavg; (void)vavg; (void)ures; (void)vres;
#pragma omp parallel for
  OEB_HADV_BODY(OEB_CAT(oeb_adv3_, SUF))
}

void OEB_FN(hadvuv5th)(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M1* acrlat0,
                       const M1* acrlat1, const M1* tgrlatda0, const M1* tgrlatda1, const M3* uatupos,
                       const M3* vatupos, const M3* uatvpos, const M3* vatvpos, const M3* uavg, const M3* vavg,
                       const M3* ures, const M3* vres, T eddlat, T eddlon, int64_t nx, int64_t ny, int64_t nz) {
  /* the openmp variant keeps every intermediate in registers and never touches the scratch fields */
  (void)uatupos; (void)vatupos; (void)uatvpos; (void)vatvpos; (void)uavg; (void)vavg; (void)ures; (void)vres;
#pragma omp parallel for
  OEB_HADV_BODY(OEB_CAT(oeb_adv5_, SUF))
}

/* kernels/fastwavesuv.h:154-191 (fastwavesuv_openmp) */
void OEB_FN(fastwavesuv)(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* utens,
                         const M3* vtens, const M3* wgtfac, const M3* ppuv, const M3* hhl, const M3* rho,
                         const M1* fx, const M3* ppgk, const M3* ppgc, const M3* ppgu, const M3* ppgv, T edadlat,
                         T dt, int64_t nx, int64_t ny, int64_t nz) {
  (void)ppgk; (void)ppgc; (void)ppgu; (void)ppgv; /* unused by the openmp variant */
#pragma omp parallel for
  for (int64_t i = 0; i < nx; ++i) {
    for (int64_t j = 0; j < ny; ++j) {
      for (int64_t k = 0; k < nz; ++k) {
        T ppgk_ijk = A3(wgtfac, i, j, k) * A3(ppuv, i, j, k) + ((T)1.0 - A3(wgtfac, i, j, k)) * A3(ppuv, i, j, k - 1);
        T ppgk_i1jk = A3(wgtfac, i + 1, j, k) * A3(ppuv, i + 1, j, k) +
                      ((T)1.0 - A3(wgtfac, i + 1, j, k)) * A3(ppuv, i + 1, j, k - 1);
        T ppgk_ij1k = A3(wgtfac, i, j + 1, k) * A3(ppuv, i, j + 1, k) +
                      ((T)1.0 - A3(wgtfac, i, j + 1, k)) * A3(ppuv, i, j + 1, k - 1);
        T ppgk_ijk1 = A3(wgtfac, i, j, k + 1) * A3(ppuv, i, j, k + 1) +
                      ((T)1.0 - A3(wgtfac, i, j, k + 1)) * A3(ppuv, i, j, k);
        T ppgk_i1jk1 = A3(wgtfac, i + 1, j, k + 1) * A3(ppuv, i + 1, j, k + 1) +
                       ((T)1.0 - A3(wgtfac, i + 1, j, k + 1)) * A3(ppuv, i + 1, j, k);
        T ppgk_ij1k1 = A3(wgtfac, i, j + 1, k + 1) * A3(ppuv, i, j + 1, k + 1) +
                       ((T)1.0 - A3(wgtfac, i, j + 1, k + 1)) * A3(ppuv, i, j + 1, k);

        T ppgc_ijk = ppgk_ijk1 - ppgk_ijk;
        T ppgc_i1jk = ppgk_i1jk1 - ppgk_i1jk;
        T ppgc_ij1k = ppgk_ij1k1 - ppgk_ij1k;

        T ppgu = (A3(ppuv, i + 1, j, k) - A3(ppuv, i, j, k)) +
                 (ppgc_i1jk + ppgc_ijk) * (T)0.5 *
                     ((A3(hhl, i, j, k + 1) + A3(hhl, i, j, k)) - (A3(hhl, i + 1, j, k + 1) + A3(hhl, i + 1, j, k))) /
                     ((A3(hhl, i, j, k + 1) - A3(hhl, i, j, k)) + (A3(hhl, i + 1, j, k + 1) - A3(hhl, i + 1, j, k)));
        T ppgv = (A3(ppuv, i, j + 1, k) - A3(ppuv, i, j, k)) +
                 (ppgc_ij1k + ppgc_ijk) * (T)0.5 *
                     ((A3(hhl, i, j, k + 1) + A3(hhl, i, j, k)) - (A3(hhl, i, j + 1, k + 1) + A3(hhl, i, j + 1, k))) /
                     ((A3(hhl, i, j, k + 1) - A3(hhl, i, j, k)) + (A3(hhl, i, j + 1, k + 1) - A3(hhl, i, j + 1, k)));

        A3(uout, i, j, k) =
            A3(uin, i, j, k) +
            dt * (A3(utens, i, j, k) - ppgu * ((T)2.0 * A1(fx, j) / (A3(rho, i + 1, j, k) + A3(rho, i, j, k))));
        A3(vout, i, j, k) =
            A3(vin, i, j, k) +
            dt * (A3(vtens, i, j, k) - ppgv * ((T)2.0 * edadlat / (A3(rho, i, j + 1, k) + A3(rho, i, j, k))));
      }
    }
  }
}

/* kernels/uvbke.h:61-75 (uvbke_openmp); dt5 is a double in the driver even when T is float
 * (src/uvbke.cpp:11-12). */
void OEB_FN(uvbke)(const M3* ub, const M3* vb, const M3* uc, const M3* vc, const M3* cosa, const M3* rsina,
                   double dt5, int64_t nx, int64_t ny, int64_t nz) {
#pragma omp parallel for
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(ub, i, j, k) = ((dt5 * ((A3(uc, i, j - 1, k) + A3(uc, i, j, k)) -
                                   ((A3(vc, i - 1, j, k) + A3(vc, i, j, k)) * A3(cosa, i, j, k)))) *
                           A3(rsina, i, j, k));
        A3(vb, i, j, k) = ((dt5 * ((A3(vc, i - 1, j, k) + A3(vc, i, j, k)) -
                                   ((A3(uc, i, j - 1, k) + A3(uc, i, j, k)) * A3(cosa, i, j, k)))) *
                           A3(rsina, i, j, k));
      }
    }
  }
}

/* kernels/nh_p_grad.h:116-146 (nh_p_grad_openmp) */
void OEB_FN(nh_p_grad)(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdx, const M3* rdy,
                       const M3* gz, const M3* pp, const M3* pk3, const M3* wk1, const M3* wk, const M3* du,
                       const M3* dv, T dt, int64_t nx, int64_t ny, int64_t nz) {
  (void)wk; (void)du; (void)dv; /* unused by the openmp variant */
#pragma omp parallel for
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        T wk_ijk = (A3(pk3, i, j, k + 1) - A3(pk3, i, j, k));
        T wk_i1jk = (A3(pk3, i + 1, j, k + 1) - A3(pk3, i + 1, j, k));
        T wk_ij1k = (A3(pk3, i, j + 1, k + 1) - A3(pk3, i, j + 1, k));
        T du = ((dt / (wk_ijk + wk_i1jk)) *
                (((A3(gz, i, j, k + 1) - A3(gz, i + 1, j, k)) * (A3(pk3, i + 1, j, k + 1) - A3(pk3, i, j, k))) +
                 ((A3(gz, i, j, k) - A3(gz, i + 1, j, k + 1)) * (A3(pk3, i, j, k + 1) - A3(pk3, i + 1, j, k)))));
        A3(uout, i, j, k) =
            (((A3(uin, i, j, k) + du) +
              ((dt / (A3(wk1, i, j, k) + A3(wk1, i + 1, j, k))) *
               (((A3(gz, i, j, k + 1) - A3(gz, i + 1, j, k)) * (A3(pp, i + 1, j, k + 1) - A3(pp, i, j, k))) +
                ((A3(gz, i, j, k) - A3(gz, i + 1, j, k + 1)) * (A3(pp, i, j, k + 1) - A3(pp, i + 1, j, k)))))) *
             A3(rdx, i, j, k));
        T dv = ((dt / (wk_ijk + wk_ij1k)) *
                (((A3(gz, i, j, k + 1) - A3(gz, i, j + 1, k)) * (A3(pk3, i, j + 1, k + 1) - A3(pk3, i, j, k))) +
                 ((A3(gz, i, j, k) - A3(gz, i, j + 1, k + 1)) * (A3(pk3, i, j, k + 1) - A3(pk3, i, j + 1, k)))));
        A3(vout, i, j, k) =
            (((A3(vin, i, j, k) + dv) +
              ((dt / (A3(wk1, i, j, k) + A3(wk1, i, j + 1, k))) *
               (((A3(gz, i, j, k + 1) - A3(gz, i, j + 1, k)) * (A3(pp, i, j + 1, k + 1) - A3(pp, i, j, k))) +
                ((A3(gz, i, j, k) - A3(gz, i, j + 1, k + 1)) * (A3(pp, i, j, k + 1) - A3(pp, i, j + 1, k)))))) *
             A3(rdy, i, j, k));
      }
    }
  }
}

/* kernels/p_grad_c.h:80-101 (p_grad_c_openmp) */
void OEB_FN(p_grad_c)(const M3* uout, const M3* vout, const M3* uin, const M3* vin, const M3* rdxc, const M3* rdyc,
                      const M3* delpc, const M3* gz, const M3* pkc, const M3* wk, T dt2, int64_t nx, int64_t ny,
                      int64_t nz) {
  (void)wk; /* unused by the openmp variant */
#pragma omp parallel for
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        T wk_ijk = A3(delpc, i, j, k);
        T wk_im1jk = A3(delpc, i - 1, j, k);
        T wk_ijm1k = A3(delpc, i, j - 1, k);
        A3(uout, i, j, k) =
            (A3(uin, i, j, k) +
             (((dt2 * A3(rdxc, i, j, k)) / (wk_im1jk + wk_ijk)) *
              (((A3(gz, i - 1, j, k + 1) - A3(gz, i, j, k)) * (A3(pkc, i, j, k + 1) - A3(pkc, i - 1, j, k))) +
               ((A3(gz, i - 1, j, k) - A3(gz, i, j, k + 1)) * (A3(pkc, i - 1, j, k + 1) - A3(pkc, i, j, k))))));
        A3(vout, i, j, k) =
            (A3(vin, i, j, k) +
             (((dt2 * A3(rdyc, i, j, k)) / (wk_ijm1k + wk_ijk)) *
              (((A3(gz, i, j - 1, k + 1) - A3(gz, i, j, k)) * (A3(pkc, i, j, k + 1) - A3(pkc, i, j - 1, k))) +
               ((A3(gz, i, j - 1, k) - A3(gz, i, j, k + 1)) * (A3(pkc, i, j - 1, k + 1) - A3(pkc, i, j, k))))));
      }
    }
  }
}

/* kernels/fvtp2d.h:4-177 (serial fvtp2d; the reference has no OpenMP variant of it).  The
 * PPM flags are stored as T, as in the reference ((almq*br) < int64_t(0) converted to T). */
void OEB_FN(fvtp2d)(const M3* q_i, const M3* q_j, const M3* fx1, const M3* fx2, const M3* fy1, const M3* fy2,
                    const M3* q, const M3* crx, const M3* cry, const M3* ra_x, const M3* ra_y, const M3* xfx,
                    const M3* yfx, const M3* area, const M3* fxx, const M3* fyy, const M3* al, const M3* almq,
                    const M3* br, const M3* b0, const M3* smt5, T p1, T p2, int64_t nx, int64_t ny, int64_t nz) {
  /* fy2: fvtp2d.h:8-37 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -3; i < nx + 2; ++i) {
      for (int64_t j = -1; j < ny + 2; ++j) {
        A3(al, i, j, k) = ((p1 * (A3(q, i, j - 1, k) + A3(q, i, j, k))) + (p2 * (A3(q, i, j - 2, k) + A3(q, i, j + 1, k))));
      }
    }
  }
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -3; i < nx + 2; ++i) {
      for (int64_t j = -1; j < ny + 1; ++j) {
        A3(almq, i, j, k) = (A3(al, i, j, k) - A3(q, i, j, k));
        A3(br, i, j, k) = (A3(al, i, j + 1, k) - A3(q, i, j, k));
        A3(b0, i, j, k) = (A3(almq, i, j, k) + A3(br, i, j, k));
        A3(smt5, i, j, k) = ((A3(almq, i, j, k) * A3(br, i, j, k)) < (int64_t)0);
      }
    }
    for (int64_t i = -3; i < nx + 2; ++i) {
      for (int64_t j = 0; j < ny + 1; ++j) {
        T smt5tmp = (A3(smt5, i, j - 1, k) + (A3(smt5, i, j, k) * (A3(smt5, i, j - 1, k) == (int64_t)0)));
        T crytmp = ((A3(cry, i, j, k) > (T)(0.))
                        ? (((T)(1.) - A3(cry, i, j, k)) * (A3(br, i, j - 1, k) - (A3(cry, i, j, k) * A3(b0, i, j - 1, k))))
                        : (((T)(1.) + A3(cry, i, j, k)) * (A3(almq, i, j, k) + (A3(cry, i, j, k) * A3(b0, i, j, k)))));
        A3(fy2, i, j, k) = ((A3(cry, i, j, k) > (T)(0.)) ? (A3(q, i, j - 1, k) + (crytmp * smt5tmp))
                                                        : (A3(q, i, j, k) + (crytmp * smt5tmp)));
      }
    }
  }

  /* q_i: fvtp2d.h:39-51 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -3; i < nx + 2; ++i) {
      for (int64_t j = 0; j < ny + 1; ++j) {
        A3(fyy, i, j, k) = (A3(yfx, i, j, k) * A3(fy2, i, j, k));
      }
    }
    for (int64_t i = -3; i < nx + 2; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(q_i, i, j, k) =
            ((((A3(q, i, j, k) * A3(area, i, j, k)) + A3(fyy, i, j, k)) - A3(fyy, i, j + 1, k)) / A3(ra_y, i, j, k));
      }
    }
  }

  /* fx1: fvtp2d.h:53-82 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -1; i < nx + 1; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(al, i, j, k) = ((p1 * (A3(q_i, i - 1, j, k) + A3(q_i, i, j, k))) +
                           (p2 * (A3(q_i, i - 2, j, k) + A3(q_i, i + 1, j, k))));
      }
    }
  }
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -1; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(almq, i, j, k) = (A3(al, i, j, k) - A3(q_i, i, j, k));
        A3(br, i, j, k) = (A3(al, i + 1, j, k) - A3(q_i, i, j, k));
        A3(b0, i, j, k) = (A3(almq, i, j, k) + A3(br, i, j, k));
        A3(smt5, i, j, k) = ((A3(almq, i, j, k) * A3(br, i, j, k)) < (int64_t)0);
      }
    }
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        T smt5tmp = (A3(smt5, i - 1, j, k) + (A3(smt5, i, j, k) * (A3(smt5, i - 1, j, k) == (int64_t)0)));
        T crxtmp = ((A3(crx, i, j, k) > (T)(0.))
                        ? (((T)(1.) - A3(crx, i, j, k)) * (A3(br, i - 1, j, k) - (A3(crx, i, j, k) * A3(b0, i - 1, j, k))))
                        : (((T)(1.) + A3(crx, i, j, k)) * (A3(almq, i, j, k) + (A3(crx, i, j, k) * A3(b0, i, j, k)))));
        A3(fx1, i, j, k) = ((A3(crx, i, j, k) > (T)(0.)) ? (A3(q_i, i - 1, j, k) + (crxtmp * smt5tmp))
                                                        : (A3(q_i, i, j, k) + (crxtmp * smt5tmp)));
      }
    }
  }

  /* fx2: fvtp2d.h:84-113 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -1; i < nx + 2; ++i) {
      for (int64_t j = -3; j < ny + 2; ++j) {
        A3(al, i, j, k) = ((p1 * (A3(q, i - 1, j, k) + A3(q, i, j, k))) + (p2 * (A3(q, i - 2, j, k) + A3(q, i + 1, j, k))));
      }
    }
  }
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = -1; i < nx + 1; ++i) {
      for (int64_t j = -3; j < ny + 2; ++j) {
        A3(almq, i, j, k) = (A3(al, i, j, k) - A3(q, i, j, k));
        A3(br, i, j, k) = (A3(al, i + 1, j, k) - A3(q, i, j, k));
        A3(b0, i, j, k) = (A3(almq, i, j, k) + A3(br, i, j, k));
        A3(smt5, i, j, k) = ((A3(almq, i, j, k) * A3(br, i, j, k)) < (int64_t)0);
      }
    }
    for (int64_t i = 0; i < nx + 1; ++i) {
      for (int64_t j = -3; j < ny + 2; ++j) {
        T smt5tmp = (A3(smt5, i - 1, j, k) + (A3(smt5, i, j, k) * (A3(smt5, i - 1, j, k) == (int64_t)0)));
        T crxtmp = ((A3(crx, i, j, k) > (T)(0.))
                        ? (((T)(1.) - A3(crx, i, j, k)) * (A3(br, i - 1, j, k) - (A3(crx, i, j, k) * A3(b0, i - 1, j, k))))
                        : (((T)(1.) + A3(crx, i, j, k)) * (A3(almq, i, j, k) + (A3(crx, i, j, k) * A3(b0, i, j, k)))));
        A3(fx2, i, j, k) = ((A3(crx, i, j, k) > (T)(0.)) ? (A3(q, i - 1, j, k) + (crxtmp * smt5tmp))
                                                        : (A3(q, i, j, k) + (crxtmp * smt5tmp)));
      }
    }
  }

  /* q_j: fvtp2d.h:115-127 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx + 1; ++i) {
      for (int64_t j = -3; j < ny + 2; ++j) {
        A3(fxx, i, j, k) = (A3(xfx, i, j, k) * A3(fx2, i, j, k));
      }
    }
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = -3; j < ny + 2; ++j) {
        A3(q_j, i, j, k) =
            ((((A3(q, i, j, k) * A3(area, i, j, k)) + A3(fxx, i, j, k)) - A3(fxx, i + 1, j, k)) / A3(ra_x, i, j, k));
      }
    }
  }

  /* fy1: fvtp2d.h:129-158 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = -1; j < ny + 1; ++j) {
        A3(al, i, j, k) = ((p1 * (A3(q_j, i, j - 1, k) + A3(q_j, i, j, k))) +
                           (p2 * (A3(q_j, i, j - 2, k) + A3(q_j, i, j + 1, k))));
      }
    }
  }
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = -1; j < ny; ++j) {
        A3(almq, i, j, k) = (A3(al, i, j, k) - A3(q_j, i, j, k));
        A3(br, i, j, k) = (A3(al, i, j + 1, k) - A3(q_j, i, j, k));
        A3(b0, i, j, k) = (A3(almq, i, j, k) + A3(br, i, j, k));
        A3(smt5, i, j, k) = ((A3(almq, i, j, k) * A3(br, i, j, k)) < (int64_t)0);
      }
    }
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        T smt5tmp = (A3(smt5, i, j - 1, k) + (A3(smt5, i, j, k) * (A3(smt5, i, j - 1, k) == (int64_t)0)));
        T crytmp = ((A3(cry, i, j, k) > (T)(0.))
                        ? (((T)(1.) - A3(cry, i, j, k)) * (A3(br, i, j - 1, k) - (A3(cry, i, j, k) * A3(b0, i, j - 1, k))))
                        : (((T)(1.) + A3(cry, i, j, k)) * (A3(almq, i, j, k) + (A3(cry, i, j, k) * A3(b0, i, j, k)))));
        A3(fy1, i, j, k) = ((A3(cry, i, j, k) > (T)(0.)) ? (A3(q_j, i, j - 1, k) + (crytmp * smt5tmp))
                                                        : (A3(q_j, i, j, k) + (crytmp * smt5tmp)));
      }
    }
  }

  /* transport_flux: fvtp2d.h:160-176 */
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(fx1, i, j, k) = (((T)(0.5) * (A3(fx1, i, j, k) + A3(fx2, i, j, k))) * A3(xfx, i, j, k));
      }
    }
  }
  for (int64_t k = 0; k < nz; ++k) {
    for (int64_t i = 0; i < nx; ++i) {
      for (int64_t j = 0; j < ny; ++j) {
        A3(fy1, i, j, k) = (((T)(0.5) * (A3(fy1, i, j, k) + A3(fy2, i, j, k))) * A3(yfx, i, j, k));
      }
    }
  }
}

#undef OEB_HADV_BODY
#undef OEB_EARTH_RADIUS
#undef OEB_EARTH_RADIUS_RECIP
#undef A3
#undef A1
#undef OEB_FN
