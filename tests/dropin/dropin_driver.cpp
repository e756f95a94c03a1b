// dropin_driver.cpp -- a driver in the style of the reference's src/<k>.cpp that calls the
// ten kernel functions through the drop-in headers (include/oeb/<k>.h) on host-memory
// fields, and on device-memory fields for laplace and hdiffsa, and checks every output bit
// for bit against the oracle (liboeb_oracle.so).  Exit status 0 = all identical.
//
// Build (tests/test_dropin.py):  g++ -std=c++17 -O1 -I include/oeb -I tests/dropin
//   tests/dropin/dropin_driver.cpp -L <lib dirs> -loeb_gb300 -loeb_oracle -lcudart
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

// globals every reference driver defines before util.h (src/<k>.cpp:4-9)
int64_t domain_size = 20;
int64_t domain_height = 4;
int64_t halo_width = 4;
typedef double ElementType;
const double dt5 = 0.5 * 225.0;  // src/uvbke.cpp:11-12
#define p1 ElementType(0.583333)  // src/fvtp2d.cpp:11-12
#define p2 ElementType(0.083333)

#include "storage_compat.h"

#include "laplace.h"
#include "hdiffsa.h"
#include "hdiffsmag.h"
#include "hadvuv.h"
#include "hadvuv5th.h"
#include "fastwavesuv.h"
#include "uvbke.h"
#include "nh_p_grad.h"
#include "p_grad_c.h"
#include "fvtp2d.h"

extern "C" {
typedef oeb_memref3d_f64 M3;
typedef oeb_memref1d_f64 M1;
void oeb_oracle_laplace_f64(const M3*, const M3*, int64_t, int64_t, int64_t);
void oeb_oracle_hdiffsa_f64(const M3*, const M3*, const M3*, const M1*, const M1*, const M3*, const M3*, const M3*,
                            int64_t, int64_t, int64_t);
void oeb_oracle_hdiffsmag_f64(const M3*, const M3*, const M3*, const M3*, const M3*, const M1*, const M1*, const M1*,
                              const M1*, const M1*, const M3*, const M3*, double, double, double, double, int64_t,
                              int64_t, int64_t);
void oeb_oracle_hadvuv_f64(const M3*, const M3*, const M3*, const M3*, const M1*, const M1*, const M1*, const M1*,
                           const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                           double, double, int64_t, int64_t, int64_t);
void oeb_oracle_hadvuv5th_f64(const M3*, const M3*, const M3*, const M3*, const M1*, const M1*, const M1*, const M1*,
                              const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                              double, double, int64_t, int64_t, int64_t);
void oeb_oracle_fastwavesuv_f64(const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                                const M3*, const M3*, const M3*, const M1*, const M3*, const M3*, const M3*,
                                const M3*, double, double, int64_t, int64_t, int64_t);
void oeb_oracle_uvbke_f64(const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, double, int64_t, int64_t,
                          int64_t);
void oeb_oracle_nh_p_grad_f64(const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                              const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, double, int64_t,
                              int64_t, int64_t);
void oeb_oracle_p_grad_c_f64(const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                             const M3*, const M3*, double, int64_t, int64_t, int64_t);
void oeb_oracle_fvtp2d_f64(const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                           const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*, const M3*,
                           const M3*, const M3*, const M3*, const M3*, const M3*, double, double, int64_t, int64_t,
                           int64_t);
}

static int failures = 0;

// A field and its twin for the oracle run; both start from the same deterministic values.
struct F3 {
  std::vector<double> a, b;
  Storage3D s, t;
  M3 ma() { return oeb_dropin::m3(s); }
  M3 mb() { return oeb_dropin::m3(t); }
};
struct F1 {
  std::vector<double> a, b;
  Storage1D s, t;
  M1 mb() { return oeb_dropin::m1(t); }
};

static double value(int seed, size_t idx) {  // smooth-ish deterministic values, with sign changes
  return 10.0 * std::sin(0.37 * (double)idx + 1.3 * seed) + 0.01 * std::cos(1.7 * (double)idx * (seed + 1));
}

static F3 field(int seed, double lo = 0.0, double fill = -1.0) {
  F3 f;
  f.s = make3(domain_size, domain_height, halo_width, f.a);
  f.t = make3(domain_size, domain_height, halo_width, f.b);
  for (size_t i = 0; i < f.a.size(); ++i) f.a[i] = (seed < 0) ? fill : lo + value(seed, i);
  f.b = f.a;
  return f;
}
static F1 line(int seed) {
  F1 f;
  f.s = make1(domain_size, halo_width, f.a);
  f.t = make1(domain_size, halo_width, f.b);
  for (size_t i = 0; i < f.a.size(); ++i) f.a[i] = 1.0 + 0.01 * value(seed, i);
  f.b = f.a;
  return f;
}

static void same(const char* what, const F3& f) {
  if (f.a.size() != f.b.size() || std::memcmp(f.a.data(), f.b.data(), f.a.size() * sizeof(double)) != 0) {
    size_t bad = 0;
    for (size_t i = 0; i < f.a.size(); ++i) bad += std::memcmp(&f.a[i], &f.b[i], sizeof(double)) != 0;
    std::printf("FAIL %s: %zu cells differ\n", what, bad);
    ++failures;
  } else {
    std::printf("ok   %s\n", what);
  }
}

int main() {
  const int64_t n = domain_size, nz = domain_height;
  {  // laplace
    F3 in = field(1), out = field(-1);
    laplace(in.s, out.s);
    M3 i = in.mb(), o = out.mb();
    oeb_oracle_laplace_f64(&i, &o, n, n, nz);
    same("laplace", out);
  }
  {  // hdiffsa
    F3 out = field(-1), in = field(2), mask = field(3, 0.0), lap = field(-1), flx = field(-1), fly = field(-1);
    F1 a = line(4), b = line(5);
    hdiffsa(out.s, in.s, mask.s, a.s, b.s, lap.s, flx.s, fly.s);
    M3 o = out.mb(), i = in.mb(), m = mask.mb(), l = lap.mb(), fx = flx.mb(), fy = fly.mb();
    M1 la = a.mb(), lb = b.mb();
    oeb_oracle_hdiffsa_f64(&o, &i, &m, &la, &lb, &l, &fx, &fy, n, n, nz);
    same("hdiffsa", out);
  }
  {  // hdiffsmag
    F3 uo = field(-1), vo = field(-1), ui = field(6), vi = field(7), mask = field(8, 20.0), t = field(-1), s = field(-1);
    F1 c0 = line(9), c1 = line(10), c2 = line(11), c3 = line(12), c4 = line(13);
    hdiffsmag(uo.s, vo.s, ui.s, vi.s, mask.s, c0.s, c1.s, c2.s, c3.s, c4.s, t.s, s.s, 0.05, 0.06, 0.07, 0.001);
    M3 a = uo.mb(), b = vo.mb(), c = ui.mb(), d = vi.mb(), e = mask.mb(), x = t.mb(), y = s.mb();
    M1 l0 = c0.mb(), l1 = c1.mb(), l2 = c2.mb(), l3 = c3.mb(), l4 = c4.mb();
    oeb_oracle_hdiffsmag_f64(&a, &b, &c, &d, &e, &l0, &l1, &l2, &l3, &l4, &x, &y, 0.05, 0.06, 0.07, 0.001, n, n, nz);
    same("hdiffsmag.uout", uo);
    same("hdiffsmag.vout", vo);
  }
  for (int order = 3; order <= 5; order += 2) {  // hadvuv, hadvuv5th
    F3 uo = field(-1), vo = field(-1), ui = field(14), vi = field(15);
    F1 a0 = line(16), a1 = line(17), t0 = line(18), t1 = line(19);
    F3 sc[8] = {field(-1), field(-1), field(-1), field(-1), field(-1), field(-1), field(-1), field(-1)};
    if (order == 3)
      hadvuv(uo.s, vo.s, ui.s, vi.s, a0.s, a1.s, t0.s, t1.s, sc[0].s, sc[1].s, sc[2].s, sc[3].s, sc[4].s, sc[5].s,
             sc[6].s, sc[7].s, 0.03, 0.04);
    else
      hadvuv5th(uo.s, vo.s, ui.s, vi.s, a0.s, a1.s, t0.s, t1.s, sc[0].s, sc[1].s, sc[2].s, sc[3].s, sc[4].s, sc[5].s,
                sc[6].s, sc[7].s, 0.03, 0.04);
    M3 a = uo.mb(), b = vo.mb(), c = ui.mb(), d = vi.mb();
    M1 l0 = a0.mb(), l1 = a1.mb(), l2 = t0.mb(), l3 = t1.mb();
    M3 s[8];
    for (int q = 0; q < 8; ++q) s[q] = sc[q].mb();
    if (order == 3)
      oeb_oracle_hadvuv_f64(&a, &b, &c, &d, &l0, &l1, &l2, &l3, &s[0], &s[1], &s[2], &s[3], &s[4], &s[5], &s[6],
                            &s[7], 0.03, 0.04, n, n, nz);
    else
      oeb_oracle_hadvuv5th_f64(&a, &b, &c, &d, &l0, &l1, &l2, &l3, &s[0], &s[1], &s[2], &s[3], &s[4], &s[5], &s[6],
                               &s[7], 0.03, 0.04, n, n, nz);
    same(order == 3 ? "hadvuv.uout" : "hadvuv5th.uout", uo);
    same(order == 3 ? "hadvuv.vout" : "hadvuv5th.vout", vo);
  }
  {  // fastwavesuv (positive, separated rho and a monotone-ish hhl keep the divisors away from 0)
    F3 uo = field(-1), vo = field(-1), ui = field(20), vi = field(21), ut = field(22), vt = field(23),
       w = field(24, 40.0), pp = field(25), hhl = field(26), rho = field(27, 100.0);
    for (int64_t k = -halo_width; k < nz + halo_width; ++k)
      for (int64_t j = -halo_width; j < n + halo_width; ++j)
        for (int64_t i = -halo_width; i < n + halo_width; ++i) {
          hhl.s.at(i, j, k) = 1000.0 - 50.0 * k + 0.1 * std::sin(0.3 * i + 0.2 * j);
          hhl.t.at(i, j, k) = hhl.s.at(i, j, k);
        }
    F1 fx = line(28);
    F3 sc[4] = {field(-1), field(-1), field(-1), field(-1)};
    fastwavesuv(uo.s, vo.s, ui.s, vi.s, ut.s, vt.s, w.s, pp.s, hhl.s, rho.s, fx.s, sc[0].s, sc[1].s, sc[2].s, sc[3].s,
                0.02, 0.5);
    M3 a = uo.mb(), b = vo.mb(), c = ui.mb(), d = vi.mb(), e = ut.mb(), f = vt.mb(), g = w.mb(), h = pp.mb(),
       x = hhl.mb(), y = rho.mb();
    M1 l = fx.mb();
    M3 s[4];
    for (int q = 0; q < 4; ++q) s[q] = sc[q].mb();
    oeb_oracle_fastwavesuv_f64(&a, &b, &c, &d, &e, &f, &g, &h, &x, &y, &l, &s[0], &s[1], &s[2], &s[3], 0.02, 0.5, n,
                               n, nz);
    same("fastwavesuv.uout", uo);
    same("fastwavesuv.vout", vo);
  }
  {  // uvbke
    F3 ub = field(-1), vb = field(-1), uc = field(29), vc = field(30), ca = field(31), rs = field(32);
    uvbke(ub.s, vb.s, uc.s, vc.s, ca.s, rs.s);
    M3 a = ub.mb(), b = vb.mb(), c = uc.mb(), d = vc.mb(), e = ca.mb(), f = rs.mb();
    oeb_oracle_uvbke_f64(&a, &b, &c, &d, &e, &f, dt5, n, n, nz);
    same("uvbke.ub", ub);
    same("uvbke.vb", vb);
  }
  {  // nh_p_grad (pk3 and wk1 shifted so the divisors stay away from 0)
    F3 uo = field(-1), vo = field(-1), ui = field(33), vi = field(34), rdx = field(35), rdy = field(36),
       gz = field(37), pp = field(38), pk3 = field(39), wk1 = field(40, 50.0), wk = field(-1), du = field(-1),
       dv = field(-1);
    for (int64_t k = -halo_width; k < nz + halo_width; ++k)
      for (int64_t j = -halo_width; j < n + halo_width; ++j)
        for (int64_t i = -halo_width; i < n + halo_width; ++i) {
          pk3.s.at(i, j, k) = 800.0 - 30.0 * k + 0.2 * std::cos(0.1 * i * j);
          pk3.t.at(i, j, k) = pk3.s.at(i, j, k);
        }
    nh_p_grad(uo.s, vo.s, ui.s, vi.s, rdx.s, rdy.s, gz.s, pp.s, pk3.s, wk1.s, wk.s, du.s, dv.s, 0.1);
    M3 a = uo.mb(), b = vo.mb(), c = ui.mb(), d = vi.mb(), e = rdx.mb(), f = rdy.mb(), g = gz.mb(), h = pp.mb(),
       x = pk3.mb(), y = wk1.mb(), z = wk.mb(), u = du.mb(), v = dv.mb();
    oeb_oracle_nh_p_grad_f64(&a, &b, &c, &d, &e, &f, &g, &h, &x, &y, &z, &u, &v, 0.1, n, n, nz);
    same("nh_p_grad.uout", uo);
    same("nh_p_grad.vout", vo);
  }
  {  // p_grad_c
    F3 uo = field(-1), vo = field(-1), ui = field(41), vi = field(42), rx = field(43), ry = field(44),
       dp = field(45, 50.0), gz = field(46), pk = field(47), wk = field(-1);
    p_grad_c(uo.s, vo.s, ui.s, vi.s, rx.s, ry.s, dp.s, gz.s, pk.s, wk.s, 0.1);
    M3 a = uo.mb(), b = vo.mb(), c = ui.mb(), d = vi.mb(), e = rx.mb(), f = ry.mb(), g = dp.mb(), h = gz.mb(),
       x = pk.mb(), y = wk.mb();
    oeb_oracle_p_grad_c_f64(&a, &b, &c, &d, &e, &f, &g, &h, &x, &y, 0.1, n, n, nz);
    same("p_grad_c.uout", uo);
    same("p_grad_c.vout", vo);
  }
  {  // fvtp2d
    F3 o[6] = {field(-1), field(-1), field(-1), field(-1), field(-1), field(-1)};
    F3 q = field(48), crx = field(49), cry = field(50), rax = field(51, 40.0), ray = field(52, 40.0),
       xfx = field(53), yfx = field(54), area = field(55);
    for (F3* c : {&crx, &cry, &xfx, &yfx})  // Courant numbers and fluxes in [-0.8, 0.8]
      for (size_t i = 0; i < c->a.size(); ++i) c->a[i] = c->b[i] = 0.07 * c->a[i];
    F3 sc[7] = {field(-1), field(-1), field(-1), field(-1), field(-1), field(-1), field(-1)};
    fvtp2d(o[0].s, o[1].s, o[2].s, o[3].s, o[4].s, o[5].s, q.s, crx.s, cry.s, rax.s, ray.s, xfx.s, yfx.s, area.s,
           sc[0].s, sc[1].s, sc[2].s, sc[3].s, sc[4].s, sc[5].s, sc[6].s);
    M3 m[6], s[7];
    for (int i = 0; i < 6; ++i) m[i] = o[i].mb();
    for (int i = 0; i < 7; ++i) s[i] = sc[i].mb();
    M3 a = q.mb(), b = crx.mb(), c = cry.mb(), d = rax.mb(), e = ray.mb(), f = xfx.mb(), g = yfx.mb(), h = area.mb();
    oeb_oracle_fvtp2d_f64(&m[0], &m[1], &m[2], &m[3], &m[4], &m[5], &a, &b, &c, &d, &e, &f, &g, &h, &s[0], &s[1],
                          &s[2], &s[3], &s[4], &s[5], &s[6], p1, p2, n, n, nz);
    const char* names[6] = {"fvtp2d.q_i", "fvtp2d.q_j", "fvtp2d.fx1", "fvtp2d.fx2", "fvtp2d.fy1", "fvtp2d.fy2"};
    for (int i = 0; i < 6; ++i) same(names[i], o[i]);
  }
  {  // device-memory fields: laplace through the same drop-in function
    F3 in = field(56), out = field(-1);
    const size_t bytes = in.a.size() * sizeof(double);
    double *din = nullptr, *dout = nullptr;
    if (cudaMalloc(&din, bytes) != cudaSuccess || cudaMalloc(&dout, bytes) != cudaSuccess) {
      std::printf("FAIL cudaMalloc\n");
      return 1;
    }
    cudaMemcpy(din, in.a.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dout, out.a.data(), bytes, cudaMemcpyHostToDevice);
    Storage3D ds = in.s, dso = out.s;
    ds.allocatedPtr = din;
    ds.alignedPtr = din + (in.s.alignedPtr - in.s.allocatedPtr);
    dso.allocatedPtr = dout;
    dso.alignedPtr = dout + (out.s.alignedPtr - out.s.allocatedPtr);
    laplace_openmp(ds, dso);
    cudaMemcpy(out.a.data(), dout, bytes, cudaMemcpyDeviceToHost);
    M3 i = in.mb(), o = out.mb();
    oeb_oracle_laplace_f64(&i, &o, n, n, nz);
    same("laplace (device fields)", out);
    cudaFree(din);
    cudaFree(dout);
  }
  std::printf("%s: %d failure(s)\n", failures ? "FAILED" : "PASSED", failures);
  return failures ? 1 : 0;
}
