// oeb_dropin_calls.hpp -- overloads of the C ABI entry points on the descriptor type, so
// that one drop-in function body serves ElementType = double and = float.
#ifndef OEB_DROPIN_CALLS_HPP
#define OEB_DROPIN_CALLS_HPP

#include "../oeb_gb300.h"

namespace oeb_dropin {

inline int call_laplace(const oeb_memref3d_f64* a_in, const oeb_memref3d_f64* a_out, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_laplace_f64(a_in, a_out, a_dom, a_stream)
                : (int)oeb_laplace_f64_host(a_in, a_out, a_dom, a_stream);
}
inline int call_hdiffsa(const oeb_memref3d_f64* a_out, const oeb_memref3d_f64* a_in, const oeb_memref3d_f64* a_mask, const oeb_memref1d_f64* a_crlato, const oeb_memref1d_f64* a_crlatu, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hdiffsa_f64(a_out, a_in, a_mask, a_crlato, a_crlatu, a_dom, a_stream)
                : (int)oeb_hdiffsa_f64_host(a_out, a_in, a_mask, a_crlato, a_crlatu, a_dom, a_stream);
}
inline int call_hdiffsmag(const oeb_memref3d_f64* a_uout, const oeb_memref3d_f64* a_vout, const oeb_memref3d_f64* a_uin, const oeb_memref3d_f64* a_vin, const oeb_memref3d_f64* a_mask, const oeb_memref1d_f64* a_crlavo, const oeb_memref1d_f64* a_crlavu, const oeb_memref1d_f64* a_crlato, const oeb_memref1d_f64* a_crlatu, const oeb_memref1d_f64* a_acrlat0, double a_eddlat, double a_eddlon, double a_tau_smag, double a_weight_smag, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hdiffsmag_f64(a_uout, a_vout, a_uin, a_vin, a_mask, a_crlavo, a_crlavu, a_crlato, a_crlatu, a_acrlat0, a_eddlat, a_eddlon, a_tau_smag, a_weight_smag, a_dom, a_stream)
                : (int)oeb_hdiffsmag_f64_host(a_uout, a_vout, a_uin, a_vin, a_mask, a_crlavo, a_crlavu, a_crlato, a_crlatu, a_acrlat0, a_eddlat, a_eddlon, a_tau_smag, a_weight_smag, a_dom, a_stream);
}
inline int call_hadvuv(const oeb_memref3d_f64* a_uout, const oeb_memref3d_f64* a_vout, const oeb_memref3d_f64* a_uin, const oeb_memref3d_f64* a_vin, const oeb_memref1d_f64* a_acrlat0, const oeb_memref1d_f64* a_acrlat1, const oeb_memref1d_f64* a_tgrlatda0, const oeb_memref1d_f64* a_tgrlatda1, double a_eddlat, double a_eddlon, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hadvuv_f64(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream)
                : (int)oeb_hadvuv_f64_host(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream);
}
inline int call_hadvuv5th(const oeb_memref3d_f64* a_uout, const oeb_memref3d_f64* a_vout, const oeb_memref3d_f64* a_uin, const oeb_memref3d_f64* a_vin, const oeb_memref1d_f64* a_acrlat0, const oeb_memref1d_f64* a_acrlat1, const oeb_memref1d_f64* a_tgrlatda0, const oeb_memref1d_f64* a_tgrlatda1, double a_eddlat, double a_eddlon, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hadvuv5th_f64(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream)
                : (int)oeb_hadvuv5th_f64_host(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream);
}
inline int call_fastwavesuv(const oeb_memref3d_f64* a_uout, const oeb_memref3d_f64* a_vout, const oeb_memref3d_f64* a_uin, const oeb_memref3d_f64* a_vin, const oeb_memref3d_f64* a_utens, const oeb_memref3d_f64* a_vtens, const oeb_memref3d_f64* a_wgtfac, const oeb_memref3d_f64* a_ppuv, const oeb_memref3d_f64* a_hhl, const oeb_memref3d_f64* a_rho, const oeb_memref1d_f64* a_fx, double a_edadlat, double a_dt, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_fastwavesuv_f64(a_uout, a_vout, a_uin, a_vin, a_utens, a_vtens, a_wgtfac, a_ppuv, a_hhl, a_rho, a_fx, a_edadlat, a_dt, a_dom, a_stream)
                : (int)oeb_fastwavesuv_f64_host(a_uout, a_vout, a_uin, a_vin, a_utens, a_vtens, a_wgtfac, a_ppuv, a_hhl, a_rho, a_fx, a_edadlat, a_dt, a_dom, a_stream);
}
inline int call_uvbke(const oeb_memref3d_f64* a_ub, const oeb_memref3d_f64* a_vb, const oeb_memref3d_f64* a_uc, const oeb_memref3d_f64* a_vc, const oeb_memref3d_f64* a_cosa, const oeb_memref3d_f64* a_rsina, double a_dt5, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_uvbke_f64(a_ub, a_vb, a_uc, a_vc, a_cosa, a_rsina, a_dt5, a_dom, a_stream)
                : (int)oeb_uvbke_f64_host(a_ub, a_vb, a_uc, a_vc, a_cosa, a_rsina, a_dt5, a_dom, a_stream);
}
inline int call_nh_p_grad(const oeb_memref3d_f64* a_uout, const oeb_memref3d_f64* a_vout, const oeb_memref3d_f64* a_uin, const oeb_memref3d_f64* a_vin, const oeb_memref3d_f64* a_rdx, const oeb_memref3d_f64* a_rdy, const oeb_memref3d_f64* a_gz, const oeb_memref3d_f64* a_pp, const oeb_memref3d_f64* a_pk3, const oeb_memref3d_f64* a_wk1, double a_dt, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_nh_p_grad_f64(a_uout, a_vout, a_uin, a_vin, a_rdx, a_rdy, a_gz, a_pp, a_pk3, a_wk1, a_dt, a_dom, a_stream)
                : (int)oeb_nh_p_grad_f64_host(a_uout, a_vout, a_uin, a_vin, a_rdx, a_rdy, a_gz, a_pp, a_pk3, a_wk1, a_dt, a_dom, a_stream);
}
inline int call_p_grad_c(const oeb_memref3d_f64* a_uout, const oeb_memref3d_f64* a_vout, const oeb_memref3d_f64* a_uin, const oeb_memref3d_f64* a_vin, const oeb_memref3d_f64* a_rdxc, const oeb_memref3d_f64* a_rdyc, const oeb_memref3d_f64* a_delpc, const oeb_memref3d_f64* a_gz, const oeb_memref3d_f64* a_pkc, double a_dt2, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_p_grad_c_f64(a_uout, a_vout, a_uin, a_vin, a_rdxc, a_rdyc, a_delpc, a_gz, a_pkc, a_dt2, a_dom, a_stream)
                : (int)oeb_p_grad_c_f64_host(a_uout, a_vout, a_uin, a_vin, a_rdxc, a_rdyc, a_delpc, a_gz, a_pkc, a_dt2, a_dom, a_stream);
}
inline int call_fvtp2d(const oeb_memref3d_f64* a_q_i, const oeb_memref3d_f64* a_q_j, const oeb_memref3d_f64* a_fx1, const oeb_memref3d_f64* a_fx2, const oeb_memref3d_f64* a_fy1, const oeb_memref3d_f64* a_fy2, const oeb_memref3d_f64* a_q, const oeb_memref3d_f64* a_crx, const oeb_memref3d_f64* a_cry, const oeb_memref3d_f64* a_ra_x, const oeb_memref3d_f64* a_ra_y, const oeb_memref3d_f64* a_xfx, const oeb_memref3d_f64* a_yfx, const oeb_memref3d_f64* a_area, double a_p1, double a_p2, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_fvtp2d_f64(a_q_i, a_q_j, a_fx1, a_fx2, a_fy1, a_fy2, a_q, a_crx, a_cry, a_ra_x, a_ra_y, a_xfx, a_yfx, a_area, a_p1, a_p2, a_dom, a_stream)
                : (int)oeb_fvtp2d_f64_host(a_q_i, a_q_j, a_fx1, a_fx2, a_fy1, a_fy2, a_q, a_crx, a_cry, a_ra_x, a_ra_y, a_xfx, a_yfx, a_area, a_p1, a_p2, a_dom, a_stream);
}

inline int call_laplace(const oeb_memref3d_f32* a_in, const oeb_memref3d_f32* a_out, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_laplace_f32(a_in, a_out, a_dom, a_stream)
                : (int)oeb_laplace_f32_host(a_in, a_out, a_dom, a_stream);
}
inline int call_hdiffsa(const oeb_memref3d_f32* a_out, const oeb_memref3d_f32* a_in, const oeb_memref3d_f32* a_mask, const oeb_memref1d_f32* a_crlato, const oeb_memref1d_f32* a_crlatu, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hdiffsa_f32(a_out, a_in, a_mask, a_crlato, a_crlatu, a_dom, a_stream)
                : (int)oeb_hdiffsa_f32_host(a_out, a_in, a_mask, a_crlato, a_crlatu, a_dom, a_stream);
}
inline int call_hdiffsmag(const oeb_memref3d_f32* a_uout, const oeb_memref3d_f32* a_vout, const oeb_memref3d_f32* a_uin, const oeb_memref3d_f32* a_vin, const oeb_memref3d_f32* a_mask, const oeb_memref1d_f32* a_crlavo, const oeb_memref1d_f32* a_crlavu, const oeb_memref1d_f32* a_crlato, const oeb_memref1d_f32* a_crlatu, const oeb_memref1d_f32* a_acrlat0, float a_eddlat, float a_eddlon, float a_tau_smag, float a_weight_smag, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hdiffsmag_f32(a_uout, a_vout, a_uin, a_vin, a_mask, a_crlavo, a_crlavu, a_crlato, a_crlatu, a_acrlat0, a_eddlat, a_eddlon, a_tau_smag, a_weight_smag, a_dom, a_stream)
                : (int)oeb_hdiffsmag_f32_host(a_uout, a_vout, a_uin, a_vin, a_mask, a_crlavo, a_crlavu, a_crlato, a_crlatu, a_acrlat0, a_eddlat, a_eddlon, a_tau_smag, a_weight_smag, a_dom, a_stream);
}
inline int call_hadvuv(const oeb_memref3d_f32* a_uout, const oeb_memref3d_f32* a_vout, const oeb_memref3d_f32* a_uin, const oeb_memref3d_f32* a_vin, const oeb_memref1d_f32* a_acrlat0, const oeb_memref1d_f32* a_acrlat1, const oeb_memref1d_f32* a_tgrlatda0, const oeb_memref1d_f32* a_tgrlatda1, float a_eddlat, float a_eddlon, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hadvuv_f32(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream)
                : (int)oeb_hadvuv_f32_host(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream);
}
inline int call_hadvuv5th(const oeb_memref3d_f32* a_uout, const oeb_memref3d_f32* a_vout, const oeb_memref3d_f32* a_uin, const oeb_memref3d_f32* a_vin, const oeb_memref1d_f32* a_acrlat0, const oeb_memref1d_f32* a_acrlat1, const oeb_memref1d_f32* a_tgrlatda0, const oeb_memref1d_f32* a_tgrlatda1, float a_eddlat, float a_eddlon, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_hadvuv5th_f32(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream)
                : (int)oeb_hadvuv5th_f32_host(a_uout, a_vout, a_uin, a_vin, a_acrlat0, a_acrlat1, a_tgrlatda0, a_tgrlatda1, a_eddlat, a_eddlon, a_dom, a_stream);
}
inline int call_fastwavesuv(const oeb_memref3d_f32* a_uout, const oeb_memref3d_f32* a_vout, const oeb_memref3d_f32* a_uin, const oeb_memref3d_f32* a_vin, const oeb_memref3d_f32* a_utens, const oeb_memref3d_f32* a_vtens, const oeb_memref3d_f32* a_wgtfac, const oeb_memref3d_f32* a_ppuv, const oeb_memref3d_f32* a_hhl, const oeb_memref3d_f32* a_rho, const oeb_memref1d_f32* a_fx, float a_edadlat, float a_dt, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_fastwavesuv_f32(a_uout, a_vout, a_uin, a_vin, a_utens, a_vtens, a_wgtfac, a_ppuv, a_hhl, a_rho, a_fx, a_edadlat, a_dt, a_dom, a_stream)
                : (int)oeb_fastwavesuv_f32_host(a_uout, a_vout, a_uin, a_vin, a_utens, a_vtens, a_wgtfac, a_ppuv, a_hhl, a_rho, a_fx, a_edadlat, a_dt, a_dom, a_stream);
}
inline int call_uvbke(const oeb_memref3d_f32* a_ub, const oeb_memref3d_f32* a_vb, const oeb_memref3d_f32* a_uc, const oeb_memref3d_f32* a_vc, const oeb_memref3d_f32* a_cosa, const oeb_memref3d_f32* a_rsina, double a_dt5, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_uvbke_f32(a_ub, a_vb, a_uc, a_vc, a_cosa, a_rsina, a_dt5, a_dom, a_stream)
                : (int)oeb_uvbke_f32_host(a_ub, a_vb, a_uc, a_vc, a_cosa, a_rsina, a_dt5, a_dom, a_stream);
}
inline int call_nh_p_grad(const oeb_memref3d_f32* a_uout, const oeb_memref3d_f32* a_vout, const oeb_memref3d_f32* a_uin, const oeb_memref3d_f32* a_vin, const oeb_memref3d_f32* a_rdx, const oeb_memref3d_f32* a_rdy, const oeb_memref3d_f32* a_gz, const oeb_memref3d_f32* a_pp, const oeb_memref3d_f32* a_pk3, const oeb_memref3d_f32* a_wk1, float a_dt, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_nh_p_grad_f32(a_uout, a_vout, a_uin, a_vin, a_rdx, a_rdy, a_gz, a_pp, a_pk3, a_wk1, a_dt, a_dom, a_stream)
                : (int)oeb_nh_p_grad_f32_host(a_uout, a_vout, a_uin, a_vin, a_rdx, a_rdy, a_gz, a_pp, a_pk3, a_wk1, a_dt, a_dom, a_stream);
}
inline int call_p_grad_c(const oeb_memref3d_f32* a_uout, const oeb_memref3d_f32* a_vout, const oeb_memref3d_f32* a_uin, const oeb_memref3d_f32* a_vin, const oeb_memref3d_f32* a_rdxc, const oeb_memref3d_f32* a_rdyc, const oeb_memref3d_f32* a_delpc, const oeb_memref3d_f32* a_gz, const oeb_memref3d_f32* a_pkc, float a_dt2, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_p_grad_c_f32(a_uout, a_vout, a_uin, a_vin, a_rdxc, a_rdyc, a_delpc, a_gz, a_pkc, a_dt2, a_dom, a_stream)
                : (int)oeb_p_grad_c_f32_host(a_uout, a_vout, a_uin, a_vin, a_rdxc, a_rdyc, a_delpc, a_gz, a_pkc, a_dt2, a_dom, a_stream);
}
inline int call_fvtp2d(const oeb_memref3d_f32* a_q_i, const oeb_memref3d_f32* a_q_j, const oeb_memref3d_f32* a_fx1, const oeb_memref3d_f32* a_fx2, const oeb_memref3d_f32* a_fy1, const oeb_memref3d_f32* a_fy2, const oeb_memref3d_f32* a_q, const oeb_memref3d_f32* a_crx, const oeb_memref3d_f32* a_cry, const oeb_memref3d_f32* a_ra_x, const oeb_memref3d_f32* a_ra_y, const oeb_memref3d_f32* a_xfx, const oeb_memref3d_f32* a_yfx, const oeb_memref3d_f32* a_area, float a_p1, float a_p2, const oeb_domain* a_dom, void* a_stream, bool a_device) {
  return a_device ? (int)oeb_fvtp2d_f32(a_q_i, a_q_j, a_fx1, a_fx2, a_fy1, a_fy2, a_q, a_crx, a_cry, a_ra_x, a_ra_y, a_xfx, a_yfx, a_area, a_p1, a_p2, a_dom, a_stream)
                : (int)oeb_fvtp2d_f32_host(a_q_i, a_q_j, a_fx1, a_fx2, a_fy1, a_fy2, a_q, a_crx, a_cry, a_ra_x, a_ra_y, a_xfx, a_yfx, a_area, a_p1, a_p2, a_dom, a_stream);
}

}  // namespace oeb_dropin

#endif  // OEB_DROPIN_CALLS_HPP
