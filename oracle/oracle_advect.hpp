// ORACLE — test infrastructure only (see wrf_oracle.hpp).
// Restatement of dyn_em/module_advect_em.F advect_u/v/w/scalar/scalar_pd for
// h_*_adv_order=5, v_*_adv_order=3 with periodic, symmetric or open lateral
// boundaries: next to an open boundary the reference degrades the horizontal
// flux order (degrade_xs/xe/ys/ye, module_advect_em.F:500-516) and adds the
// radiation terms of the open-boundary rows.
#pragma once
#include "wrf_oracle.hpp"

namespace wrforacle {

inline void check_lateral(const WrfDynConfig& cf) {
  if (cf.specified || cf.nested || cf.polar) throw std::runtime_error("specified/nested/polar boundaries not supported");
}

// module_advect_em.F:126-1526 (5th-order horizontal :486-745, radiation
// boundary terms :1241-1335, 3rd-order vertical :1338-1356, :1470-1497).
template <typename R>
void advect_u(R* u_p, R* u_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p, R* mut_p,
              const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
              R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzw_p, const Dims& d) {
  (void)msfuy_p; (void)msfvx_p; (void)msfvy_p; (void)msftx_p; (void)msfty_p;
  check_lateral(cf);
  A3<R> u(u_p, d), u_old(u_old_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msfux(msfux_p, d), mut(mut_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d), fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const R cb = R(25.);  // share/module_model_constants.F:47
  const int ktf = std::min(d.kte, d.kde - 1);
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  // module_advect_em.F:500-516
  const bool degrade_xs = !(cf.periodic_x || cf.symmetric_xs || d.its > ids + 3);
  const bool degrade_xe = !(cf.periodic_x || cf.symmetric_xe || d.ite < ide - 2);
  const bool degrade_ys = !(cf.periodic_y || cf.symmetric_ys || d.jts > jds + 3);
  const bool degrade_ye = !(cf.periodic_y || cf.symmetric_ye || d.jte < jde - 4);
  // y flux divergence
  int i_start = d.its, i_end = d.ite;
  if (cf.open_xs) i_start = std::max(ids + 1, d.its);
  if (cf.open_xe) i_end = std::min(ide - 1, d.ite);
  if (cf.periodic_x) { i_start = d.its; i_end = d.ite; }
  int j_start = d.jts, j_end = std::min(d.jte, jde - 1);
  int j_start_f = j_start, j_end_f = j_end + 1;
  if (degrade_ys) { j_start = std::max(d.jts, jds + 1); j_start_f = jds + 3; }
  if (degrade_ye) { j_end = std::min(d.jte, jde - 2); j_end_f = jde - 3; }
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        if (j >= j_start_f && j <= j_end_f) {
          R vel = R(0.5) * (rv(i, k, j) + rv(i - 1, k, j));
          fqy(i, k, jp1) = vel * flux5(u(i, k, j - 3), u(i, k, j - 2), u(i, k, j - 1), u(i, k, j), u(i, k, j + 1), u(i, k, j + 2), vel);
        } else if (j == jds + 1 || j == jde - 1) {
          fqy(i, k, jp1) = R(0.25) * (rv(i, k, j) + rv(i - 1, k, j)) * (u(i, k, j) + u(i, k, j - 1));
        } else if (j == jds + 2 || j == jde - 2) {
          R vel = R(0.5) * (rv(i, k, j) + rv(i - 1, k, j));
          fqy(i, k, jp1) = vel * flux3(u(i, k, j - 2), u(i, k, j - 1), u(i, k, j), u(i, k, j + 1), vel);
        }
      }
    if (j > j_start)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msfux(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  // x flux divergence
  i_start = d.its; i_end = d.ite;
  j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  int i_start_f = i_start, i_end_f = i_end + 1;
  if (degrade_xs) { i_start = std::max(ids + 1, d.its); i_start_f = ids + 3; }
  if (degrade_xe) { i_end = std::min(ide - 1, d.ite); i_end_f = ide - 2; }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = R(0.5) * (ru(i, k, j) + ru(i - 1, k, j));
        fqx(i, k) = vel * flux5(u(i - 3, k, j), u(i - 2, k, j), u(i - 1, k, j), u(i, k, j), u(i + 1, k, j), u(i + 2, k, j), vel);
      }
    if (degrade_xs) {
      if (i_start == ids + 1) {
        int i = ids + 1;
        for (int k = d.kts; k <= ktf; ++k) {
          R ub = u(i - 1, k, j);
          fqx(i, k) = R(0.25) * (ru(i, k, j) + ru(i - 1, k, j)) * (u(i, k, j) + ub);
        }
      }
      int i = ids + 2;
      for (int k = d.kts; k <= ktf; ++k) {
        R vel = R(0.5) * (ru(i, k, j) + ru(i - 1, k, j));
        fqx(i, k) = vel * flux3(u(i - 2, k, j), u(i - 1, k, j), u(i, k, j), u(i + 1, k, j), vel);
      }
    }
    if (degrade_xe) {
      if (i_end == ide - 1) {
        int i = ide;
        for (int k = d.kts; k <= ktf; ++k) {
          R ub = u(i, k, j);
          fqx(i, k) = R(0.25) * (ru(i, k, j) + ru(i - 1, k, j)) * (u(i - 1, k, j) + ub);
        }
      }
      int i = ide - 1;
      for (int k = d.kts; k <= ktf; ++k) {
        R vel = R(0.5) * (ru(i, k, j) + ru(i - 1, k, j));
        fqx(i, k) = vel * flux3(u(i - 2, k, j), u(i - 1, k, j), u(i, k, j), u(i + 1, k, j), vel);
      }
    }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msfux(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  // radiative lateral boundary condition in x for the normal velocity
  if (cf.open_xs && d.its == ids)
    for (int j = d.jts; j <= std::min(d.jte, jde - 1); ++j)
      for (int k = d.kts; k <= ktf; ++k) {
        R ub = fminr(ru(d.its, k, j) - cb * (c1(k) * mut(d.its, j) + c2(k)), R(0.));
        tendency(d.its, k, j) = tendency(d.its, k, j) - rdx * ub * (u_old(d.its + 1, k, j) - u_old(d.its, k, j));
      }
  if (cf.open_xe && d.ite == ide)
    for (int j = d.jts; j <= std::min(d.jte, jde - 1); ++j)
      for (int k = d.kts; k <= ktf; ++k) {
        R ub = fmaxr(ru(d.ite, k, j) + cb * (c1(k) * mut(d.ite - 1, j) + c2(k)), R(0.));
        tendency(d.ite, k, j) = tendency(d.ite, k, j) - rdx * ub * (u_old(d.ite, k, j) - u_old(d.ite - 1, k, j));
      }
  // the rest of the radiation conditions (module_advect_em.F:1277-1335)
  i_start = d.its; i_end = std::min(d.ite, ide);
  int imin = ids, imax = ide - 1;
  if (cf.open_xs) i_start = std::max(ids + 1, d.its);
  if (cf.open_xe) i_end = std::min(d.ite, ide - 1);
  if (cf.open_ys && d.jts == jds)
    for (int i = i_start; i <= i_end; ++i) {
      R mrdy = msfux(i, d.jts) * rdy;
      int ip = std::min(imax, i), im = std::max(imin, i - 1);
      for (int k = d.kts; k <= ktf; ++k) {
        R vw = R(0.5) * (rv(ip, k, d.jts) + rv(im, k, d.jts));
        R vb = fminr(vw, R(0.));
        R dvm = rv(ip, k, d.jts + 1) - rv(ip, k, d.jts);
        R dvp = rv(im, k, d.jts + 1) - rv(im, k, d.jts);
        tendency(i, k, d.jts) = tendency(i, k, d.jts) -
            mrdy * (vb * (u_old(i, k, d.jts + 1) - u_old(i, k, d.jts)) + R(0.5) * u(i, k, d.jts) * (dvm + dvp));
      }
    }
  if (cf.open_ye && d.jte == jde)
    for (int i = i_start; i <= i_end; ++i) {
      R mrdy = msfux(i, d.jte - 1) * rdy;
      int ip = std::min(imax, i), im = std::max(imin, i - 1);
      for (int k = d.kts; k <= ktf; ++k) {
        R vw = R(0.5) * (rv(ip, k, d.jte) + rv(im, k, d.jte));
        R vb = fmaxr(vw, R(0.));
        R dvm = rv(ip, k, d.jte) - rv(ip, k, d.jte - 1);
        R dvp = rv(im, k, d.jte) - rv(im, k, d.jte - 1);
        tendency(i, k, d.jte - 1) = tendency(i, k, d.jte - 1) -
            mrdy * (vb * (u_old(i, k, d.jte - 1) - u_old(i, k, d.jte - 2)) + R(0.5) * u(i, k, d.jte - 1) * (dvm + dvp));
      }
    }
  // vertical (the reference narrows the i range here on open_ys / open_ye)
  i_start = d.its; i_end = d.ite; j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  if (cf.open_ys) i_start = std::max(ids + 1, d.its);
  if (cf.open_ye) i_end = std::min(ide - 1, d.ite);
  if (cf.periodic_x) { i_start = d.its; i_end = d.ite; }
  for (int i = i_start; i <= i_end; ++i) { vflux(i, d.kts) = R(0.); vflux(i, d.kte) = R(0.); }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts + 2; k <= ktf - 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = R(0.5) * (rom(i - 1, k, j) + rom(i, k, j));
        vflux(i, k) = vel * flux3(u(i, k - 2, j), u(i, k - 1, j), u(i, k, j), u(i, k + 1, j), -vel);
      }
    for (int i = i_start; i <= i_end; ++i) {
      int k = d.kts + 1;
      vflux(i, k) = R(0.5) * (rom(i, k, j) + rom(i - 1, k, j)) * (fzm(k) * u(i, k, j) + fzp(k) * u(i, k - 1, j));
      k = ktf;
      vflux(i, k) = R(0.5) * (rom(i, k, j) + rom(i - 1, k, j)) * (fzm(k) * u(i, k, j) + fzp(k) * u(i, k - 1, j));
    }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) - rdzw(k) * (vflux(i, k + 1) - vflux(i, k));
  }
}

// module_advect_em.F:1530-3024 (5th-order horizontal :1904-2171, radiation
// boundary terms :2711-2808, 3rd-order vertical :2961-2995).
template <typename R>
void advect_v(R* v_p, R* v_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p, R* mut_p,
              const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
              R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzw_p, const Dims& d) {
  (void)msfux_p; (void)msfuy_p; (void)msftx_p; (void)msfty_p;
  check_lateral(cf);
  A3<R> v(v_p, d), v_old(v_old_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msfvx(msfvx_p, d), msfvy(msfvy_p, d), mut(mut_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d), fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const R cb = R(25.);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  // module_advect_em.F:1918-1934
  const bool degrade_xs = !(cf.periodic_x || cf.symmetric_xs || d.its > ids + 3);
  const bool degrade_xe = !(cf.periodic_x || cf.symmetric_xe || d.ite < ide - 3);
  const bool degrade_ys = !(cf.periodic_y || cf.symmetric_ys || d.jts > jds + 3);
  const bool degrade_ye = !(cf.periodic_y || cf.symmetric_ye || d.jte < jde - 3);
  int i_start = d.its, i_end = std::min(d.ite, ide - 1);
  int j_start = d.jts, j_end = d.jte;
  int j_start_f = j_start, j_end_f = j_end + 1;
  if (degrade_ys) { j_start = std::max(d.jts, jds + 1); j_start_f = jds + 3; }
  if (degrade_ye) { j_end = std::min(d.jte, jde - 1); j_end_f = jde - 2; }
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        if (j >= j_start_f && j <= j_end_f) {
          R vel = R(0.5) * (rv(i, k, j) + rv(i, k, j - 1));
          fqy(i, k, jp1) = vel * flux5(v(i, k, j - 3), v(i, k, j - 2), v(i, k, j - 1), v(i, k, j), v(i, k, j + 1), v(i, k, j + 2), vel);
        } else if (j == jds + 1) {
          R vb = v(i, k, j - 1);
          fqy(i, k, jp1) = R(0.25) * (rv(i, k, j) + rv(i, k, j - 1)) * (v(i, k, j) + vb);
        } else if (j == jds + 2 || j == jde - 1) {
          R vel = R(0.5) * (rv(i, k, j) + rv(i, k, j - 1));
          fqy(i, k, jp1) = vel * flux3(v(i, k, j - 2), v(i, k, j - 1), v(i, k, j), v(i, k, j + 1), vel);
        } else if (j == jde) {
          R vb = v(i, k, j);
          fqy(i, k, jp1) = R(0.25) * (rv(i, k, j) + rv(i, k, j - 1)) * (vb + v(i, k, j - 1));
        }
      }
    if (j > j_start)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msfvy(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  j_start = d.jts; j_end = d.jte;
  if (cf.open_ys) j_start = std::max(jds + 1, d.jts);
  if (cf.open_ye) j_end = std::min(jde - 1, d.jte);
  int i_start_f = i_start, i_end_f = i_end + 1;
  if (degrade_xs) { i_start = std::max(ids + 1, d.its); i_start_f = std::min(i_start + 2, ids + 3); }
  if (degrade_xe) { i_end = std::min(ide - 2, d.ite); i_end_f = ide - 3; }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = R(0.5) * (ru(i, k, j) + ru(i, k, j - 1));
        fqx(i, k) = vel * flux5(v(i - 3, k, j), v(i - 2, k, j), v(i - 1, k, j), v(i, k, j), v(i + 1, k, j), v(i + 2, k, j), vel);
      }
    if (degrade_xs)
      for (int i = i_start; i <= i_start_f - 1; ++i) {
        if (i == ids + 1)
          for (int k = d.kts; k <= ktf; ++k)
            fqx(i, k) = R(0.25) * (ru(i, k, j) + ru(i, k, j - 1)) * (v(i, k, j) + v(i - 1, k, j));
        if (i == ids + 2)
          for (int k = d.kts; k <= ktf; ++k) {
            R vel = R(0.5) * (ru(i, k, j) + ru(i, k, j - 1));
            fqx(i, k) = vel * flux3(v(i - 2, k, j), v(i - 1, k, j), v(i, k, j), v(i + 1, k, j), vel);
          }
      }
    if (degrade_xe)
      for (int i = i_end_f + 1; i <= i_end + 1; ++i) {
        if (i == ide - 1)
          for (int k = d.kts; k <= ktf; ++k)
            fqx(i, k) = R(0.25) * (ru(i_end + 1, k, j) + ru(i_end + 1, k, j - 1)) * (v(i_end + 1, k, j) + v(i_end, k, j));
        if (i == ide - 2)
          for (int k = d.kts; k <= ktf; ++k) {
            R vel = R(0.5) * (ru(i, k, j) + ru(i, k, j - 1));
            fqx(i, k) = vel * flux3(v(i - 2, k, j), v(i - 1, k, j), v(i, k, j), v(i + 1, k, j), vel);
          }
      }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msfvy(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  // radiative lateral boundary condition in y for the normal velocity
  if (cf.open_ys && d.jts == jds)
    for (int i = d.its; i <= std::min(d.ite, ide - 1); ++i)
      for (int k = d.kts; k <= ktf; ++k) {
        R vb = fminr(rv(i, k, d.jts) - cb * (c1(k) * mut(i, d.jts) + c2(k)), R(0.));
        tendency(i, k, d.jts) = tendency(i, k, d.jts) - rdy * vb * (v_old(i, k, d.jts + 1) - v_old(i, k, d.jts));
      }
  if (cf.open_ye && d.jte == jde)
    for (int i = d.its; i <= std::min(d.ite, ide - 1); ++i)
      for (int k = d.kts; k <= ktf; ++k) {
        R vb = fmaxr(rv(i, k, d.jte) + cb * (c1(k) * mut(i, d.jte - 1) + c2(k)), R(0.));
        tendency(i, k, d.jte) = tendency(i, k, d.jte) - rdy * vb * (v_old(i, k, d.jte) - v_old(i, k, d.jte - 1));
      }
  // the rest of the radiation conditions (module_advect_em.F:2741-2808)
  j_start = d.jts; j_end = std::min(d.jte, jde);
  int jmin = jds, jmax = jde - 1;
  if (cf.open_ys) j_start = std::max(jds + 1, d.jts);
  if (cf.open_ye) j_end = std::min(d.jte, jde - 1);
  if (cf.open_xs && d.its == ids)
    for (int j = j_start; j <= j_end; ++j) {
      R mrdx = msfvy(d.its, j) * rdx;
      int jp = std::min(jmax, j), jm = std::max(jmin, j - 1);
      for (int k = d.kts; k <= ktf; ++k) {
        R uw = R(0.5) * (ru(d.its, k, jp) + ru(d.its, k, jm));
        R ub = fminr(uw, R(0.));
        R dup = ru(d.its + 1, k, jp) - ru(d.its, k, jp);
        R dum = ru(d.its + 1, k, jm) - ru(d.its, k, jm);
        tendency(d.its, k, j) = tendency(d.its, k, j) -
            mrdx * (ub * (v_old(d.its + 1, k, j) - v_old(d.its, k, j)) + R(0.5) * v(d.its, k, j) * (dup + dum));
      }
    }
  if (cf.open_xe && d.ite == ide)
    for (int j = j_start; j <= j_end; ++j) {
      R mrdx = msfvy(d.ite - 1, j) * rdx;
      int jp = std::min(jmax, j), jm = std::max(jmin, j - 1);
      for (int k = d.kts; k <= ktf; ++k) {
        R uw = R(0.5) * (ru(d.ite, k, jp) + ru(d.ite, k, jm));
        R ub = fmaxr(uw, R(0.));
        R dup = ru(d.ite, k, jp) - ru(d.ite - 1, k, jp);
        R dum = ru(d.ite, k, jm) - ru(d.ite - 1, k, jm);
        tendency(d.ite - 1, k, j) = tendency(d.ite - 1, k, j) -
            mrdx * (ub * (v_old(d.ite - 1, k, j) - v_old(d.ite - 2, k, j)) + R(0.5) * v(d.ite - 1, k, j) * (dup + dum));
      }
    }
  i_start = d.its; i_end = std::min(d.ite, ide - 1); j_start = d.jts; j_end = d.jte;
  for (int i = i_start; i <= i_end; ++i) { vflux(i, d.kts) = R(0.); vflux(i, d.kte) = R(0.); }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts + 2; k <= ktf - 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = R(0.5) * (rom(i, k, j) + rom(i, k, j - 1));
        vflux(i, k) = vel * flux3(v(i, k - 2, j), v(i, k - 1, j), v(i, k, j), v(i, k + 1, j), -vel);
      }
    for (int i = i_start; i <= i_end; ++i) {
      int k = d.kts + 1;
      vflux(i, k) = R(0.5) * (rom(i, k, j) + rom(i, k, j - 1)) * (fzm(k) * v(i, k, j) + fzp(k) * v(i, k - 1, j));
      k = ktf;
      vflux(i, k) = R(0.5) * (rom(i, k, j) + rom(i, k, j - 1)) * (fzm(k) * v(i, k, j) + fzp(k) * v(i, k - 1, j));
    }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) - (msfvy(i, j) / msfvx(i, j)) * rdzw(k) * (vflux(i, k + 1) - vflux(i, k));
  }
}

// module_advect_em.F:3029-4359 (5th-order horizontal :3394-3650, radiation
// boundary terms :4104-4175, 3rd-order vertical :4306-4333).
template <typename R>
void advect_scalar(R* field_p, R* field_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p,
                   R* mut_p, const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p,
                   R* msfty_p, R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzw_p, const Dims& d) {
  (void)c1_p; (void)c2_p; (void)mut_p; (void)msfux_p; (void)msfuy_p; (void)msfvx_p; (void)msfvy_p; (void)msfty_p;
  check_lateral(cf);
  A3<R> field(field_p, d), field_old(field_old_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msftx(msftx_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  // module_advect_em.F:3403-3419
  const bool degrade_xs = !(cf.periodic_x || cf.symmetric_xs || d.its > ids + 3);
  const bool degrade_xe = !(cf.periodic_x || cf.symmetric_xe || d.ite < ide - 3);
  const bool degrade_ys = !(cf.periodic_y || cf.symmetric_ys || d.jts > jds + 3);
  const bool degrade_ye = !(cf.periodic_y || cf.symmetric_ye || d.jte < jde - 4);
  int i_start = d.its, i_end = std::min(d.ite, ide - 1);
  int j_start = d.jts, j_end = std::min(d.jte, jde - 1);
  int j_start_f = j_start, j_end_f = j_end + 1;
  if (degrade_ys) { j_start = std::max(d.jts, jds + 1); j_start_f = jds + 3; }
  if (degrade_ye) { j_end = std::min(d.jte, jde - 2); j_end_f = jde - 3; }
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        if (j >= j_start_f && j <= j_end_f) {
          R vel = rv(i, k, j);
          fqy(i, k, jp1) = vel * flux5(field(i, k, j - 3), field(i, k, j - 2), field(i, k, j - 1), field(i, k, j),
                                       field(i, k, j + 1), field(i, k, j + 2), vel);
        } else if (j == jds + 1 || j == jde - 1) {
          fqy(i, k, jp1) = R(0.5) * rv(i, k, j) * (field(i, k, j) + field(i, k, j - 1));
        } else if (j == jds + 2 || j == jde - 2) {
          R vel = rv(i, k, j);
          fqy(i, k, jp1) = vel * flux3(field(i, k, j - 2), field(i, k, j - 1), field(i, k, j), field(i, k, j + 1), vel);
        }
      }
    if (j > j_start)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msftx(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  int i_start_f = i_start, i_end_f = i_end + 1;
  if (degrade_xs) { i_start = std::max(ids + 1, d.its); i_start_f = std::min(i_start + 2, ids + 3); }
  if (degrade_xe) { i_end = std::min(ide - 2, d.ite); i_end_f = ide - 3; }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = ru(i, k, j);
        fqx(i, k) = vel * flux5(field(i - 3, k, j), field(i - 2, k, j), field(i - 1, k, j), field(i, k, j),
                                field(i + 1, k, j), field(i + 2, k, j), vel);
      }
    if (degrade_xs)
      for (int i = i_start; i <= i_start_f - 1; ++i) {
        if (i == ids + 1)
          for (int k = d.kts; k <= ktf; ++k) fqx(i, k) = R(0.5) * (ru(i, k, j)) * (field(i, k, j) + field(i - 1, k, j));
        if (i == ids + 2)
          for (int k = d.kts; k <= ktf; ++k) {
            R vel = ru(i, k, j);
            fqx(i, k) = vel * flux3(field(i - 2, k, j), field(i - 1, k, j), field(i, k, j), field(i + 1, k, j), vel);
          }
      }
    if (degrade_xe)
      for (int i = i_end_f + 1; i <= i_end + 1; ++i) {
        if (i == ide - 1)
          for (int k = d.kts; k <= ktf; ++k) fqx(i, k) = R(0.5) * (ru(i, k, j)) * (field(i, k, j) + field(i - 1, k, j));
        if (i == ide - 2)
          for (int k = d.kts; k <= ktf; ++k) {
            R vel = ru(i, k, j);
            fqx(i, k) = vel * flux3(field(i - 2, k, j), field(i - 1, k, j), field(i, k, j), field(i + 1, k, j), vel);
          }
      }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msftx(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  // radiation conditions of the open boundaries (no map factors)
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  if (cf.open_xs && d.its == ids)
    for (int j = j_start; j <= j_end; ++j)
      for (int k = d.kts; k <= ktf; ++k) {
        R ub = fminr(R(0.5) * (ru(d.its, k, j) + ru(d.its + 1, k, j)), R(0.));
        tendency(d.its, k, j) = tendency(d.its, k, j) -
            rdx * (ub * (field_old(d.its + 1, k, j) - field_old(d.its, k, j)) +
                   field(d.its, k, j) * (ru(d.its + 1, k, j) - ru(d.its, k, j)));
      }
  if (cf.open_xe && d.ite == ide)
    for (int j = j_start; j <= j_end; ++j)
      for (int k = d.kts; k <= ktf; ++k) {
        R ub = fmaxr(R(0.5) * (ru(d.ite - 1, k, j) + ru(d.ite, k, j)), R(0.));
        tendency(i_end, k, j) = tendency(i_end, k, j) -
            rdx * (ub * (field_old(i_end, k, j) - field_old(i_end - 1, k, j)) +
                   field(i_end, k, j) * (ru(d.ite, k, j) - ru(d.ite - 1, k, j)));
      }
  if (cf.open_ys && d.jts == jds)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vb = fminr(R(0.5) * (rv(i, k, d.jts) + rv(i, k, d.jts + 1)), R(0.));
        tendency(i, k, d.jts) = tendency(i, k, d.jts) -
            rdy * (vb * (field_old(i, k, d.jts + 1) - field_old(i, k, d.jts)) +
                   field(i, k, d.jts) * (rv(i, k, d.jts + 1) - rv(i, k, d.jts)));
      }
  if (cf.open_ye && d.jte == jde)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vb = fmaxr(R(0.5) * (rv(i, k, d.jte - 1) + rv(i, k, d.jte)), R(0.));
        tendency(i, k, j_end) = tendency(i, k, j_end) -
            rdy * (vb * (field_old(i, k, j_end) - field_old(i, k, j_end - 1)) +
                   field(i, k, j_end) * (rv(i, k, d.jte) - rv(i, k, d.jte - 1)));
      }
  i_start = d.its; i_end = std::min(d.ite, ide - 1); j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  for (int i = i_start; i <= i_end; ++i) { vflux(i, d.kts) = R(0.); vflux(i, d.kte) = R(0.); }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts + 2; k <= ktf - 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = rom(i, k, j);
        vflux(i, k) = vel * flux3(field(i, k - 2, j), field(i, k - 1, j), field(i, k, j), field(i, k + 1, j), -vel);
      }
    for (int i = i_start; i <= i_end; ++i) {
      int k = d.kts + 1;
      vflux(i, k) = rom(i, k, j) * (fzm(k) * field(i, k, j) + fzp(k) * field(i, k - 1, j));
      k = ktf;
      vflux(i, k) = rom(i, k, j) * (fzm(k) * field(i, k, j) + fzp(k) * field(i, k - 1, j));
    }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) - rdzw(k) * (vflux(i, k + 1) - vflux(i, k));
  }
}

// module_advect_em.F:4364-6064 (5th-order horizontal :4784-5096, radiation
// boundary terms :5689-5841, 3rd-order vertical :5996-6031).
template <typename R>
void advect_w(R* w_p, R* w_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p, R* mut_p,
              const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
              R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzu_p, const Dims& d) {
  (void)c1_p; (void)c2_p; (void)mut_p; (void)msfux_p; (void)msfuy_p; (void)msfvx_p;
  (void)msfvy_p; (void)msfty_p;
  check_lateral(cf);
  A3<R> w(w_p, d), w_old(w_old_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msftx(msftx_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d), rdzu(rdzu_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  // face velocity at level k of a horizontal mass-flux array (k = ktf+1: the
  // top extrapolation)
  auto velz = [&](const A3<R>& rr, int i, int k, int j) -> R {
    if (k <= ktf) return fzm(k) * rr(i, k, j) + fzp(k) * rr(i, k - 1, j);
    return (R(2.) - fzm(k - 1)) * rr(i, k - 1, j) - fzp(k - 1) * rr(i, k - 2, j);
  };
  // module_advect_em.F:4794-4809
  const bool degrade_xs = !(cf.periodic_x || cf.symmetric_xs || d.its > ids + 3);
  const bool degrade_xe = !(cf.periodic_x || cf.symmetric_xe || d.ite < ide - 3);
  const bool degrade_ys = !(cf.periodic_y || cf.symmetric_ys || d.jts > jds + 3);
  const bool degrade_ye = !(cf.periodic_y || cf.symmetric_ye || d.jte < jde - 4);
  int i_start = d.its, i_end = std::min(d.ite, ide - 1);
  int j_start = d.jts, j_end = std::min(d.jte, jde - 1);
  int j_start_f = j_start, j_end_f = j_end + 1;
  if (degrade_ys) { j_start = std::max(d.jts, jds + 1); j_start_f = jds + 3; }
  if (degrade_ye) { j_end = std::min(d.jte, jde - 2); j_end_f = jde - 3; }
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts + 1; k <= ktf + 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = velz(rv, i, k, j);
        if (j >= j_start_f && j <= j_end_f)
          fqy(i, k, jp1) = vel * flux5(w(i, k, j - 3), w(i, k, j - 2), w(i, k, j - 1), w(i, k, j), w(i, k, j + 1), w(i, k, j + 2), vel);
        else if (j == jds + 1 || j == jde - 1)
          fqy(i, k, jp1) = R(0.5) * vel * (w(i, k, j) + w(i, k, j - 1));
        else if (j == jds + 2 || j == jde - 2)
          fqy(i, k, jp1) = vel * flux3(w(i, k, j - 2), w(i, k, j - 1), w(i, k, j), w(i, k, j + 1), vel);
      }
    if (j > j_start)
      for (int k = d.kts + 1; k <= ktf + 1; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msftx(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  int i_start_f = i_start, i_end_f = i_end + 1;
  if (degrade_xs) { i_start = std::max(ids + 1, d.its); i_start_f = std::min(i_start + 2, ids + 3); }
  if (degrade_xe) { i_end = std::min(ide - 2, d.ite); i_end_f = ide - 3; }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts + 1; k <= ktf + 1; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = velz(ru, i, k, j);
        fqx(i, k) = vel * flux5(w(i - 3, k, j), w(i - 2, k, j), w(i - 1, k, j), w(i, k, j), w(i + 1, k, j), w(i + 2, k, j), vel);
      }
    if (degrade_xs)
      for (int i = i_start; i <= i_start_f - 1; ++i)
        for (int k = d.kts + 1; k <= ktf + 1; ++k) {
          R vel = velz(ru, i, k, j);
          if (i == ids + 1) fqx(i, k) = R(0.5) * vel * (w(i, k, j) + w(i - 1, k, j));
          if (i == ids + 2) fqx(i, k) = vel * flux3(w(i - 2, k, j), w(i - 1, k, j), w(i, k, j), w(i + 1, k, j), vel);
        }
    if (degrade_xe)
      for (int i = i_end_f + 1; i <= i_end + 1; ++i)
        for (int k = d.kts + 1; k <= ktf + 1; ++k) {
          R vel = velz(ru, i, k, j);
          if (i == ide - 1) fqx(i, k) = R(0.5) * vel * (w(i, k, j) + w(i - 1, k, j));
          if (i == ide - 2) fqx(i, k) = vel * flux3(w(i - 2, k, j), w(i - 1, k, j), w(i, k, j), w(i + 1, k, j), vel);
        }
    for (int k = d.kts + 1; k <= ktf + 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msftx(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  // radiation conditions of the open boundaries (module_advect_em.F:5689-5841)
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  // the face average and difference of a mass-flux array at level k (k = ktf+1: top extrapolation)
  auto pair_sum = [&](const A3<R>& rr, int ia, int ja, int ib, int jb, int k) -> R {
    if (k <= ktf) return fzm(k) * (rr(ia, k, ja) + rr(ib, k, jb)) + fzp(k) * (rr(ia, k - 1, ja) + rr(ib, k - 1, jb));
    return (R(2.) - fzm(k - 1)) * (rr(ia, k - 1, ja) + rr(ib, k - 1, jb)) - fzp(k - 1) * (rr(ia, k - 2, ja) + rr(ib, k - 2, jb));
  };
  auto pair_dif = [&](const A3<R>& rr, int ia, int ja, int ib, int jb, int k) -> R {  // rr(b) - rr(a)
    if (k <= ktf) return fzm(k) * (rr(ib, k, jb) - rr(ia, k, ja)) + fzp(k) * (rr(ib, k - 1, jb) - rr(ia, k - 1, ja));
    return (R(2.) - fzm(k - 1)) * (rr(ib, k - 1, jb) - rr(ia, k - 1, ja)) - fzp(k - 1) * (rr(ib, k - 2, jb) - rr(ia, k - 2, ja));
  };
  if (cf.open_xs && d.its == ids)
    for (int pass = 0; pass < 2; ++pass)
      for (int j = j_start; j <= j_end; ++j)
        for (int k = pass == 0 ? d.kts + 1 : ktf + 1; k <= (pass == 0 ? ktf : ktf + 1); ++k) {
          const int i = d.its;
          R uw = R(0.5) * pair_sum(ru, i, j, i + 1, j, k);
          R ub = fminr(uw, R(0.));
          tendency(i, k, j) = tendency(i, k, j) -
              rdx * (ub * (w_old(i + 1, k, j) - w_old(i, k, j)) + w(i, k, j) * pair_dif(ru, i, j, i + 1, j, k));
        }
  if (cf.open_xe && d.ite == ide)
    for (int pass = 0; pass < 2; ++pass)
      for (int j = j_start; j <= j_end; ++j)
        for (int k = pass == 0 ? d.kts + 1 : ktf + 1; k <= (pass == 0 ? ktf : ktf + 1); ++k) {
          R uw = R(0.5) * pair_sum(ru, d.ite - 1, j, d.ite, j, k);
          R ub = fmaxr(uw, R(0.));
          tendency(i_end, k, j) = tendency(i_end, k, j) -
              rdx * (ub * (w_old(i_end, k, j) - w_old(i_end - 1, k, j)) + w(i_end, k, j) * pair_dif(ru, d.ite - 1, j, d.ite, j, k));
        }
  if (cf.open_ys && d.jts == jds)
    for (int pass = 0; pass < 2; ++pass)
      for (int i = i_start; i <= i_end; ++i)
        for (int k = pass == 0 ? d.kts + 1 : ktf + 1; k <= (pass == 0 ? ktf : ktf + 1); ++k) {
          const int j = d.jts;
          R vw = R(0.5) * pair_sum(rv, i, j, i, j + 1, k);
          R vb = fminr(vw, R(0.));
          tendency(i, k, j) = tendency(i, k, j) -
              rdy * (vb * (w_old(i, k, j + 1) - w_old(i, k, j)) + w(i, k, j) * pair_dif(rv, i, j, i, j + 1, k));
        }
  if (cf.open_ye && d.jte == jde)
    for (int pass = 0; pass < 2; ++pass)
      for (int i = i_start; i <= i_end; ++i)
        for (int k = pass == 0 ? d.kts + 1 : ktf + 1; k <= (pass == 0 ? ktf : ktf + 1); ++k) {
          R vw = R(0.5) * pair_sum(rv, i, d.jte - 1, i, d.jte, k);
          R vb = fmaxr(vw, R(0.));
          tendency(i, k, j_end) = tendency(i, k, j_end) -
              rdy * (vb * (w_old(i, k, j_end) - w_old(i, k, j_end - 1)) + w(i, k, j_end) * pair_dif(rv, i, d.jte - 1, i, d.jte, k));
        }
  i_start = d.its; i_end = std::min(d.ite, ide - 1); j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  for (int i = i_start; i <= i_end; ++i) { vflux(i, d.kts) = R(0.); vflux(i, d.kte) = R(0.); }
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts + 2; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = R(0.5) * (rom(i, k, j) + rom(i, k - 1, j));
        vflux(i, k) = vel * flux3(w(i, k - 2, j), w(i, k - 1, j), w(i, k, j), w(i, k + 1, j), -vel);
      }
    for (int i = i_start; i <= i_end; ++i) {
      int k = d.kts + 1;
      vflux(i, k) = R(0.25) * (rom(i, k, j) + rom(i, k - 1, j)) * (w(i, k, j) + w(i, k - 1, j));
      k = ktf + 1;
      vflux(i, k) = R(0.25) * (rom(i, k, j) + rom(i, k - 1, j)) * (w(i, k, j) + w(i, k - 1, j));
    }
    for (int k = d.kts + 1; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) - rdzu(k) * (vflux(i, k + 1) - vflux(i, k));
    int k = ktf + 1;
    for (int i = i_start; i <= i_end; ++i)
      tendency(i, k, j) = tendency(i, k, j) + R(2.) * rdzu(k - 1) * (vflux(i, k));
  }
}

// module_advect_em.F:6069-7885 (5th-order horizontal :6505-6779, radiation
// boundary terms :7254-7328, 3rd-order vertical :7595-7645, limiter
// :7681-7781, divergence :7783-7883).
template <typename R>
void advect_scalar_pd(R* field_p, R* field_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p,
                      R* mut_p, R* mub_p, R* mu_old_p, const WrfDynConfig& cf, R* msfux_p, R* msfuy_p,
                      R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p, R* fzm_p, R* fzp_p, R rdx, R rdy,
                      R* rdzw_p, R dt, const Dims& d) {
  (void)msfux_p; (void)msfuy_p; (void)msfvx_p; (void)msfvy_p;
  check_lateral(cf);
  A3<R> field(field_p, d), field_old(field_old_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> mut(mut_p, d), mub(mub_p, d), mu_old(mu_old_p, d), msftx(msftx_p, d), msfty(msfty_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d), fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const R eps = R(1.e-20);
  const int ktf = std::min(d.kte, d.kde - 1), kde = d.kde;
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  // Local flux arrays dimensioned (its-1:ite+2, kts:kte, jts-1:jte+2) in the reference.
  const int li0 = d.its - 1, lj0 = d.jts - 1, lk0 = d.kts;
  const int lnx = d.ite + 2 - li0 + 1, lnk = d.kte - lk0 + 1, lny = d.jte + 2 - lj0 + 1;
  const size_t ln = (size_t)lnx * lnk * lny;
  std::vector<R> s_fqx(ln), s_fqy(ln), s_fqz(ln), s_fqxl(ln), s_fqyl(ln), s_fqzl(ln), s_fo(ln), s_pl(ln);
  auto L = [&](std::vector<R>& s, int i, int k, int j) -> R& {
    return s[(size_t)(i - li0) + (size_t)(k - lk0) * lnx + (size_t)(j - lj0) * lnx * lnk];
  };
  auto fqx = [&](int i, int k, int j) -> R& { return L(s_fqx, i, k, j); };
  auto fqy = [&](int i, int k, int j) -> R& { return L(s_fqy, i, k, j); };
  auto fqz = [&](int i, int k, int j) -> R& { return L(s_fqz, i, k, j); };
  auto fqxl = [&](int i, int k, int j) -> R& { return L(s_fqxl, i, k, j); };
  auto fqyl = [&](int i, int k, int j) -> R& { return L(s_fqyl, i, k, j); };
  auto fqzl = [&](int i, int k, int j) -> R& { return L(s_fqzl, i, k, j); };
  auto flux_out = [&](int i, int k, int j) -> R& { return L(s_fo, i, k, j); };
  auto ph_low = [&](int i, int k, int j) -> R& { return L(s_pl, i, k, j); };
  // module_advect_em.F:6507-6518
  const bool degrade_xs = !(cf.periodic_x || cf.symmetric_xs || d.its > ids + 3);
  const bool degrade_xe = !(cf.periodic_x || cf.symmetric_xe || d.ite < ide - 4);
  const bool degrade_ys = !(cf.periodic_y || cf.symmetric_ys || d.jts > jds + 3);
  const bool degrade_ye = !(cf.periodic_y || cf.symmetric_ye || d.jte < jde - 4);

  // y fluxes
  int i_start = d.its - 1, i_end = std::min(d.ite, ide - 1) + 1;
  int j_start = d.jts - 1, j_end = std::min(d.jte, jde - 1) + 1;
  int j_start_f = j_start, j_end_f = j_end + 1;
  if (degrade_xs) i_start = std::max(d.its - 1, ids);
  if (degrade_xe) i_end = std::min(d.ite + 1, ide - 1);
  if (degrade_ys) { j_start = std::max(d.jts - 1, jds + 1); j_start_f = jds + 3; }
  if (degrade_ye) { j_end = std::min(d.jte + 1, jde - 2); j_end_f = jde - 3; }
  for (int j = j_start; j <= j_end + 1; ++j) {
    const bool full = j >= j_start_f && j <= j_end_f;
    const bool second = !full && (j == jds + 1 || j == jde - 1);
    const bool third = !full && !second && (j == jds + 2 || j == jde - 2);
    if (!full && !second && !third) continue;
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R dy = R(2.) / (msftx(i, j) + msftx(i, j - 1)) / rdy;
        R mu = R(0.5) * ((c1(k) * mut(i, j) + c2(k)) + (c1(k) * mut(i, j - 1) + c2(k)));
        R vel = rv(i, k, j);
        R cr = vel * dt / dy / mu;
        fqyl(i, k, j) = mu * (dy / dt) * flux_upwind(field_old(i, k, j - 1), field_old(i, k, j), cr);
        if (full)
          fqy(i, k, j) = vel * pflux5(field(i, k, j - 3), field(i, k, j - 2), field(i, k, j - 1), field(i, k, j),
                                      field(i, k, j + 1), field(i, k, j + 2), vel);
        else if (second)
          fqy(i, k, j) = R(0.5) * rv(i, k, j) * (field(i, k, j) + field(i, k, j - 1));
        else
          fqy(i, k, j) = vel * pflux3(field(i, k, j - 2), field(i, k, j - 1), field(i, k, j), field(i, k, j + 1), vel);
        fqy(i, k, j) = fqy(i, k, j) - fqyl(i, k, j);
      }
  }
  // x fluxes
  i_start = d.its - 1; i_end = std::min(d.ite, ide - 1) + 1;
  int i_start_f = i_start, i_end_f = i_end + 1;
  j_start = d.jts - 1; j_end = std::min(d.jte, jde - 1) + 1;
  if (degrade_ys) j_start = std::max(d.jts - 1, jds);
  if (degrade_ye) j_end = std::min(d.jte + 1, jde - 1);
  if (degrade_xs) { i_start = std::max(ids + 1, d.its - 1); i_start_f = ids + 3; }
  if (degrade_xe) { i_end = std::min(ide - 2, d.ite + 1); i_end_f = ide - 3; }
  auto xflux = [&](int i, int k, int j, int order) {
    R dx = R(2.) / (msfty(i, j) + msfty(i - 1, j)) / rdx;
    R mu = R(0.5) * ((c1(k) * mut(i, j) + c2(k)) + (c1(k) * mut(i - 1, j) + c2(k)));
    R vel, cr;
    if (order == 1) {  // the second-order face next to the start boundary (:6681-6685)
      vel = ru(i, k, j) / mu;
      cr = vel * dt / dx;
    } else {
      vel = ru(i, k, j);
      cr = vel * dt / dx / mu;
    }
    fqxl(i, k, j) = mu * (dx / dt) * flux_upwind(field_old(i - 1, k, j), field_old(i, k, j), cr);
    if (order == 5)
      fqx(i, k, j) = vel * pflux5(field(i - 3, k, j), field(i - 2, k, j), field(i - 1, k, j), field(i, k, j),
                                  field(i + 1, k, j), field(i + 2, k, j), vel);
    else if (order == 3)
      fqx(i, k, j) = vel * pflux3(field(i - 2, k, j), field(i - 1, k, j), field(i, k, j), field(i + 1, k, j), vel);
    else
      fqx(i, k, j) = R(0.5) * (ru(i, k, j)) * (field(i, k, j) + field(i - 1, k, j));
    fqx(i, k, j) = fqx(i, k, j) - fqxl(i, k, j);
  };
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) xflux(i, k, j, 5);
    if (degrade_xs)
      for (int i = i_start; i <= i_start_f - 1; ++i) {
        if (i == ids + 1) for (int k = d.kts; k <= ktf; ++k) xflux(i, k, j, 1);
        if (i == ids + 2) for (int k = d.kts; k <= ktf; ++k) xflux(i, k, j, 3);
      }
    if (degrade_xe)
      for (int i = i_end_f + 1; i <= i_end + 1; ++i) {
        if (i == ide - 1) for (int k = d.kts; k <= ktf; ++k) xflux(i, k, j, 2);
        if (i == ide - 2) for (int k = d.kts; k <= ktf; ++k) xflux(i, k, j, 3);
      }
  }
  // radiation conditions of the open boundaries, added before the limited
  // flux divergence (no map factors)
  {
    const int ri_end = std::min(d.ite, ide - 1), rj_end = std::min(d.jte, jde - 1);
    if (cf.open_xs && d.its == ids)
      for (int j = d.jts; j <= rj_end; ++j)
        for (int k = d.kts; k <= ktf; ++k) {
          R ub = fminr(R(0.5) * (ru(d.its, k, j) + ru(d.its + 1, k, j)), R(0.));
          tendency(d.its, k, j) = tendency(d.its, k, j) -
              rdx * (ub * (field_old(d.its + 1, k, j) - field_old(d.its, k, j)) +
                     field(d.its, k, j) * (ru(d.its + 1, k, j) - ru(d.its, k, j)));
        }
    if (cf.open_xe && d.ite == ide)
      for (int j = d.jts; j <= rj_end; ++j)
        for (int k = d.kts; k <= ktf; ++k) {
          R ub = fmaxr(R(0.5) * (ru(d.ite - 1, k, j) + ru(d.ite, k, j)), R(0.));
          tendency(ri_end, k, j) = tendency(ri_end, k, j) -
              rdx * (ub * (field_old(ri_end, k, j) - field_old(ri_end - 1, k, j)) +
                     field(ri_end, k, j) * (ru(d.ite, k, j) - ru(d.ite - 1, k, j)));
        }
    if (cf.open_ys && d.jts == jds)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= ri_end; ++i) {
          R vb = fminr(R(0.5) * (rv(i, k, d.jts) + rv(i, k, d.jts + 1)), R(0.));
          tendency(i, k, d.jts) = tendency(i, k, d.jts) -
              rdy * (vb * (field_old(i, k, d.jts + 1) - field_old(i, k, d.jts)) +
                     field(i, k, d.jts) * (rv(i, k, d.jts + 1) - rv(i, k, d.jts)));
        }
    if (cf.open_ye && d.jte == jde)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= ri_end; ++i) {
          R vb = fmaxr(R(0.5) * (rv(i, k, d.jte - 1) + rv(i, k, d.jte)), R(0.));
          tendency(i, k, rj_end) = tendency(i, k, rj_end) -
              rdy * (vb * (field_old(i, k, rj_end) - field_old(i, k, rj_end - 1)) +
                     field(i, k, rj_end) * (rv(i, k, d.jte) - rv(i, k, d.jte - 1)));
        }
  }
  // z fluxes
  i_start = d.its - 1; i_end = std::min(d.ite, ide - 1) + 1;
  j_start = d.jts - 1; j_end = std::min(d.jte, jde - 1) + 1;
  if (degrade_xs) i_start = std::max(d.its - 1, ids);
  if (degrade_xe) i_end = std::min(d.ite + 1, ide - 1);
  if (degrade_ys) j_start = std::max(d.jts - 1, jds);
  if (degrade_ye) j_end = std::min(d.jte + 1, jde - 1);
  for (int j = j_start; j <= j_end; ++j) {
    for (int i = i_start; i <= i_end; ++i) {
      fqz(i, 1, j) = R(0.); fqzl(i, 1, j) = R(0.);
      fqz(i, kde, j) = R(0.); fqzl(i, kde, j) = R(0.);
    }
    for (int k = d.kts + 2; k <= ktf - 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R dz = R(2.) / (rdzw(k) + rdzw(k - 1));
        R mu = R(0.5) * ((c1(k) * mut(i, j) + c2(k)) + (c1(k) * mut(i, j) + c2(k)));
        R vel = rom(i, k, j);
        R cr = vel * dt / dz / mu;
        fqzl(i, k, j) = mu * (dz / dt) * flux_upwind(field_old(i, k - 1, j), field_old(i, k, j), cr);
        fqz(i, k, j) = vel * pflux3(field(i, k - 2, j), field(i, k - 1, j), field(i, k, j), field(i, k + 1, j), -vel);
        fqz(i, k, j) = fqz(i, k, j) - fqzl(i, k, j);
      }
    for (int i = i_start; i <= i_end; ++i) {
      for (int pass = 0; pass < 2; ++pass) {
        int k = pass == 0 ? d.kts + 1 : ktf;
        R dz = R(2.) / (rdzw(k) + rdzw(k - 1));
        R mu = R(0.5) * ((c1(k) * mut(i, j) + c2(k)) + (c1(k) * mut(i, j) + c2(k)));
        R vel = rom(i, k, j);
        R cr = vel * dt / dz / mu;
        fqzl(i, k, j) = mu * (dz / dt) * flux_upwind(field_old(i, k - 1, j), field_old(i, k, j), cr);
        fqz(i, k, j) = rom(i, k, j) * (fzm(k) * field(i, k, j) + fzp(k) * field(i, k - 1, j));
        fqz(i, k, j) = fqz(i, k, j) - fqzl(i, k, j);
      }
    }
  }
  // positive-definite limiter (module_advect_em.F:7681-7781)
  i_start = d.its - 1; i_end = std::min(d.ite, ide - 1) + 1;
  j_start = d.jts - 1; j_end = std::min(d.jte, jde - 1) + 1;
  if (degrade_xs) i_start = std::max(d.its - 1, ids);
  if (degrade_xe) i_end = std::min(d.ite + 1, ide - 1);
  if (degrade_ys) j_start = std::max(d.jts - 1, jds);
  if (degrade_ye) j_end = std::min(d.jte + 1, jde - 1);
  if (cf.open_xs && degrade_xs) i_start = std::max(d.its - 1, ids + 1);
  if (cf.open_xe && degrade_xe) i_end = std::min(d.ite + 1, ide - 2);
  if (cf.open_ys && degrade_ys) j_start = std::max(d.jts - 1, jds + 1);
  if (cf.open_ye && degrade_ye) j_end = std::min(d.jte + 1, jde - 2);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        ph_low(i, k, j) = ((c1(k) * mub(i, j) + c2(k)) + (c1(k) * mu_old(i, j))) * field_old(i, k, j) -
                          dt * (msftx(i, j) * msfty(i, j) *
                                    (rdx * (fqxl(i + 1, k, j) - fqxl(i, k, j)) + rdy * (fqyl(i, k, j + 1) - fqyl(i, k, j))) +
                                msfty(i, j) * rdzw(k) * (fqzl(i, k + 1, j) - fqzl(i, k, j)));
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        flux_out(i, k, j) = dt * ((msftx(i, j) * msfty(i, j)) *
                                      (rdx * (fmaxr(R(0.), fqx(i + 1, k, j)) - fminr(R(0.), fqx(i, k, j))) +
                                       rdy * (fmaxr(R(0.), fqy(i, k, j + 1)) - fminr(R(0.), fqy(i, k, j)))) +
                                  msfty(i, j) * rdzw(k) * (fminr(R(0.), fqz(i, k + 1, j)) - fmaxr(R(0.), fqz(i, k, j))));
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        if (flux_out(i, k, j) > ph_low(i, k, j)) {
          R scale = fmaxr(R(0.), ph_low(i, k, j) / (flux_out(i, k, j) + eps));
          if (fqx(i + 1, k, j) > R(0.)) fqx(i + 1, k, j) = scale * fqx(i + 1, k, j);
          if (fqx(i, k, j) < R(0.)) fqx(i, k, j) = scale * fqx(i, k, j);
          if (fqy(i, k, j + 1) > R(0.)) fqy(i, k, j + 1) = scale * fqy(i, k, j + 1);
          if (fqy(i, k, j) < R(0.)) fqy(i, k, j) = scale * fqy(i, k, j);
          if (fqz(i, k + 1, j) < R(0.)) fqz(i, k + 1, j) = scale * fqz(i, k + 1, j);
          if (fqz(i, k, j) > R(0.)) fqz(i, k, j) = scale * fqz(i, k, j);
        }
  // flux divergence: z, then x, then y
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, jde - 1);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) -
                            rdzw(k) * (fqz(i, k + 1, j) - fqz(i, k, j) + fqzl(i, k + 1, j) - fqzl(i, k, j));
  if (degrade_xs) i_start = std::max(d.its, ids + 1);
  if (degrade_xe) i_end = std::min(d.ite, ide - 2);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) -
                            msftx(i, j) * (rdx * (fqx(i + 1, k, j) - fqx(i, k, j) + fqxl(i + 1, k, j) - fqxl(i, k, j)));
  i_start = d.its; i_end = std::min(d.ite, ide - 1);
  if (degrade_ys) j_start = std::max(d.jts, jds + 1);
  if (degrade_ye) j_end = std::min(d.jte, jde - 2);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) -
                            msftx(i, j) * (rdy * (fqy(i, k, j + 1) - fqy(i, k, j) + fqyl(i, k, j + 1) - fqyl(i, k, j)));
}

}  // namespace wrforacle
