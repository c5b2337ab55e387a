// ORACLE — test infrastructure only (see wrf_oracle.hpp).
// Restatement of dyn_em/module_big_step_utilities_em.F routines on the
// physics-off path and of rk_step_prep (dyn_em/module_em.F:37-186).
#pragma once
#include "wrf_oracle.hpp"

namespace wrforacle {

// module_big_step_utilities_em.F:3587-3636 (called with k range 1:1, i.e. 2-D).
template <typename R>
void calculate_full(R* rfield_p, R* rfieldb_p, R* rfieldp_p, const Dims& d) {
  A2<R> rfield(rfield_p, d), rfieldb(rfieldb_p, d), rfieldp(rfieldp_p, d);
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1);
  for (int j = d.jts - 1; j <= jtf; ++j)
    for (int i = d.its - 1; i <= itf; ++i) rfield(i, j) = rfieldb(i, j) + rfieldp(i, j);
}

// module_big_step_utilities_em.F:26-181.  The three-branch structure reduces
// to one loop with a boundary-point special case; every branch evaluates the
// same expression with im = i-1 (interior) or the periodic/one-sided index.
template <typename R>
void calc_mu_uv(const WrfDynConfig& cf, R* mu_p, R* mub_p, R* muu_p, R* muv_p, const Dims& d) {
  A2<R> MU(mu_p, d), MUB(mub_p, d), MUU(muu_p, d), MUV(muv_p, d);
  int itf = d.ite, jtf = std::min(d.jte, d.jde - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int i = d.its; i <= itf; ++i) {
      if (i == d.ids && d.its == d.ids) {
        int im = cf.periodic_x ? i - 1 : i;
        MUU(i, j) = R(0.5) * (MU(i, j) + MU(im, j) + MUB(i, j) + MUB(im, j));
      } else if (i == d.ide && d.ite == d.ide) {
        int im = cf.periodic_x ? i : i - 1;
        MUU(i, j) = R(0.5) * (MU(i - 1, j) + MU(im, j) + MUB(i - 1, j) + MUB(im, j));
      } else {
        MUU(i, j) = R(0.5) * (MU(i, j) + MU(i - 1, j) + MUB(i, j) + MUB(i - 1, j));
      }
    }
  itf = std::min(d.ite, d.ide - 1); jtf = d.jte;
  for (int j = d.jts; j <= jtf; ++j)
    for (int i = d.its; i <= itf; ++i) {
      if (j == d.jds && d.jts == d.jds) {
        int jm = cf.periodic_y ? j - 1 : j;
        MUV(i, j) = R(0.5) * (MU(i, j) + MU(i, jm) + MUB(i, j) + MUB(i, jm));
      } else if (j == d.jde && d.jte == d.jde) {
        int jm = cf.periodic_y ? j : j - 1;
        MUV(i, j) = R(0.5) * (MU(i, j - 1) + MU(i, jm) + MUB(i, j - 1) + MUB(i, jm));
      } else {
        MUV(i, j) = R(0.5) * (MU(i, j) + MU(i, j - 1) + MUB(i, j) + MUB(i, j - 1));
      }
    }
}

// module_big_step_utilities_em.F:184-326.
template <typename R>
void calc_mu_uv_1(const WrfDynConfig& cf, R* mu_p, R* muu_p, R* muv_p, const Dims& d) {
  A2<R> MU(mu_p, d), MUU(muu_p, d), MUV(muv_p, d);
  int itf = d.ite, jtf = std::min(d.jte, d.jde - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int i = d.its; i <= itf; ++i) {
      if (i == d.ids && d.its == d.ids) {
        int im = cf.periodic_x ? i - 1 : i;
        MUU(i, j) = R(0.5) * (MU(i, j) + MU(im, j));
      } else if (i == d.ide && d.ite == d.ide) {
        int im = cf.periodic_x ? i : i - 1;
        MUU(i, j) = R(0.5) * (MU(i - 1, j) + MU(im, j));
      } else {
        MUU(i, j) = R(0.5) * (MU(i, j) + MU(i - 1, j));
      }
    }
  itf = std::min(d.ite, d.ide - 1); jtf = d.jte;
  for (int j = d.jts; j <= jtf; ++j)
    for (int i = d.its; i <= itf; ++i) {
      if (j == d.jds && d.jts == d.jds) {
        int jm = cf.periodic_y ? j - 1 : j;
        MUV(i, j) = R(0.5) * (MU(i, j) + MU(i, jm));
      } else if (j == d.jde && d.jte == d.jde) {
        int jm = cf.periodic_y ? j : j - 1;
        MUV(i, j) = R(0.5) * (MU(i, j - 1) + MU(i, jm));
      } else {
        MUV(i, j) = R(0.5) * (MU(i, j) + MU(i, j - 1));
      }
    }
}

// module_big_step_utilities_em.F:329-391.
template <typename R>
void couple_momentum(R* muu_p, R* ru_p, R* u_p, R* msfu_p, R* muv_p, R* rv_p, R* v_p, R* msfv_p, R* msfv_inv_p,
                     R* mut_p, R* rw_p, R* w_p, R* msft_p, R* c1h_p, R* c2h_p, R* c1f_p, R* c2f_p, const Dims& d) {
  A2<R> muu(muu_p, d), muv(muv_p, d), mut(mut_p, d), msfu(msfu_p, d), msfv_inv(msfv_inv_p, d), msft(msft_p, d);
  A3<R> ru(ru_p, d), u(u_p, d), rv(rv_p, d), v(v_p, d), rw(rw_p, d), w(w_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), c1f(c1f_p, d), c2f(c2f_p, d);
  (void)msfv_p;
  int ktf = std::min(d.kte, d.kde - 1);
  int itf = d.ite, jtf = std::min(d.jte, d.jde - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= itf; ++i) ru(i, k, j) = u(i, k, j) * (c1h(k) * muu(i, j) + c2h(k)) / msfu(i, j);
  itf = std::min(d.ite, d.ide - 1); jtf = d.jte;
  for (int j = d.jts; j <= jtf; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= itf; ++i) rv(i, k, j) = v(i, k, j) * (c1h(k) * muv(i, j) + c2h(k)) * msfv_inv(i, j);
  itf = std::min(d.ite, d.ide - 1); jtf = std::min(d.jte, d.jde - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int k = d.kts; k <= d.kte; ++k)
      for (int i = d.its; i <= itf; ++i) rw(i, k, j) = w(i, k, j) * (c1f(k) * mut(i, j) + c2f(k)) / msft(i, j);
}

// module_big_step_utilities_em.F:640-784.
template <typename R>
void calc_ww_cp(R* u_p, R* v_p, R* mup_p, R* mub_p, R* c1h_p, R* c2h_p, R* ww_p, R rdx, R rdy, R* msftx_p,
                R* msfty_p, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvx_inv_p, R* msfvy_p, R* dnw_p,
                const Dims& d) {
  A3<R> u(u_p, d), v(v_p, d), ww(ww_p, d);
  A2<R> MUP(mup_p, d), MUB(mub_p, d), msftx(msftx_p, d), msfuy(msfuy_p, d), msfvx_inv(msfvx_inv_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), dnw(dnw_p, d);
  (void)msfty_p; (void)msfux_p; (void)msfvx_p; (void)msfvy_p;
  int nx = d.ime - d.ims + 1, ny = d.jme - d.jms + 1;
  std::vector<R> muu_s((size_t)nx * ny), muv_s((size_t)nx * ny);
  A2<R> MUU(muu_s.data(), d), MUV(muv_s.data(), d);
  int jtf = std::min(d.jte, d.jde - 1), ktf = std::min(d.kte, d.kde - 1), itf = std::min(d.ite, d.ide - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int i = d.its; i <= std::min(d.ite + 1, d.ide); ++i)
      MUU(i, j) = R(0.5) * (MUP(i, j) + MUB(i, j) + MUP(i - 1, j) + MUB(i - 1, j));
  for (int j = d.jts; j <= std::min(d.jte + 1, d.jde); ++j)
    for (int i = d.its; i <= itf; ++i)
      MUV(i, j) = R(0.5) * (MUP(i, j) + MUB(i, j) + MUP(i, j - 1) + MUB(i, j - 1));
  std::vector<R> dmdt((size_t)nx), divv((size_t)nx * (d.kme - d.kms + 1));
  auto DIVV = [&](int i, int k) -> R& { return divv[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  for (int j = d.jts; j <= jtf; ++j) {
    for (int i = d.its; i <= d.ite; ++i) {
      if (i <= itf) dmdt[i - d.ims] = R(0.);
      ww(i, 1, j) = R(0.);
      ww(i, d.kte, j) = R(0.);
    }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= itf; ++i) {
        DIVV(i, k) = msftx(i, j) * dnw(k) *
                     (rdx * ((c1h(k) * MUU(i + 1, j) + c2h(k)) * u(i + 1, k, j) / msfuy(i + 1, j) -
                             (c1h(k) * MUU(i, j) + c2h(k)) * u(i, k, j) / msfuy(i, j)) +
                      rdy * ((c1h(k) * MUV(i, j + 1) + c2h(k)) * v(i, k, j + 1) * msfvx_inv(i, j + 1) -
                             (c1h(k) * MUV(i, j) + c2h(k)) * v(i, k, j) * msfvx_inv(i, j)));
        dmdt[i - d.ims] = dmdt[i - d.ims] + DIVV(i, k);
      }
    for (int k = 2; k <= ktf; ++k)
      for (int i = d.its; i <= itf; ++i)
        ww(i, k, j) = ww(i, k - 1, j) - dnw(k - 1) * c1h(k - 1) * dmdt[i - d.ims] - DIVV(i, k - 1);
  }
}

// module_big_step_utilities_em.F:787-907 (qv is the only moist species on
// the physics-off path; n_moist >= PARAM_FIRST_SCALAR).
template <typename R>
void calc_cq(R* qv_p, R* cqu_p, R* cqv_p, R* cqw_p, int n_moist_species, const Dims& d) {
  A3<R> qv(qv_p, d), cqu(cqu_p, d), cqv(cqv_p, d), cqw(cqw_p, d);
  int ktf = std::min(d.kte, d.kde - 1);
  if (n_moist_species >= 1) {
    int itf = d.ite, jtf = std::min(d.jte, d.jde - 1);
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) {
          R qtot = R(0.) + qv(i, k, j) + qv(i - 1, k, j);
          cqu(i, k, j) = R(1.) / (R(1.) + R(0.5) * qtot);
        }
    itf = std::min(d.ite, d.ide - 1); jtf = d.jte;
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) {
          R qtot = R(0.) + qv(i, k, j) + qv(i, k, j - 1);
          cqv(i, k, j) = R(1.) / (R(1.) + R(0.5) * qtot);
        }
    itf = std::min(d.ite, d.ide - 1); jtf = std::min(d.jte, d.jde - 1);
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts + 1; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) {
          R qtot = R(0.) + qv(i, k, j) + qv(i, k - 1, j);
          cqw(i, k, j) = R(0.5) * qtot;
        }
  } else {
    int itf = d.ite, jtf = std::min(d.jte, d.jde - 1);
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) cqu(i, k, j) = R(1.);
    itf = std::min(d.ite, d.ide - 1); jtf = d.jte;
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) cqv(i, k, j) = R(1.);
    itf = std::min(d.ite, d.ide - 1); jtf = std::min(d.jte, d.jde - 1);
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts + 1; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) cqw(i, k, j) = R(0.);
  }
}

// module_big_step_utilities_em.F:910-950.
template <typename R>
void calc_alt(R* alt_p, R* al_p, R* alb_p, const Dims& d) {
  A3<R> alt(alt_p, d), al(al_p, d), alb(alb_p, d);
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1), ktf = std::min(d.kte, d.kde - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= itf; ++i) alt(i, k, j) = al(i, k, j) + alb(i, k, j);
}

// module_big_step_utilities_em.F:1227-1262.
template <typename R>
void calc_php(R* php_p, R* ph_p, R* phb_p, const Dims& d) {
  A3<R> php(php_p, d), ph(ph_p, d), phb(phb_p, d);
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1), ktf = std::min(d.kte, d.kde - 1);
  for (int j = d.jts; j <= jtf; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= itf; ++i)
        php(i, k, j) = R(0.5) * (phb(i, k, j) + phb(i, k + 1, j) + ph(i, k, j) + ph(i, k + 1, j));
}

// module_em.F:37-186 rk_step_prep (calls in the reference's order).
template <typename R>
void rk_step_prep(const WrfDynConfig& cf, int rk_step, R* u, R* v, R* w, R* t, R* ph, R* mu, R* c1h, R* c2h,
                  R* c1f, R* c2f, R* qv, int n_moist_species, R* ru, R* rv, R* rw, R* ww, R* php, R* alt,
                  R* muu, R* muv, R* mub, R* mut, R* phb, R* pb, R* p, R* al, R* alb, R* cqu, R* cqv, R* cqw,
                  R* msfux, R* msfuy, R* msfvx, R* msfvx_inv, R* msfvy, R* msftx, R* msfty, R* fnm, R* fnp,
                  R* dnw, R rdx, R rdy, const Dims& d) {
  (void)rk_step; (void)t; (void)pb; (void)p; (void)fnm; (void)fnp;
  Dims d2 = d;  // calculate_full is called with k dims 1:2 / 1:1 / 1:1
  calculate_full(mut, mub, mu, d2);
  calc_mu_uv(cf, mu, mub, muu, muv, d);
  couple_momentum(muu, ru, u, msfuy, muv, rv, v, msfvx, msfvx_inv, mut, rw, w, msfty, c1h, c2h, c1f, c2f, d);
  calc_ww_cp(u, v, mu, mub, c1h, c2h, ww, rdx, rdy, msftx, msfty, msfux, msfuy, msfvx, msfvx_inv, msfvy, dnw, d);
  calc_cq(qv, cqu, cqv, cqw, n_moist_species, d);
  calc_alt(alt, al, alb, d);
  calc_php(php, ph, phb, d);
}

// module_big_step_utilities_em.F:4573-4643 zero_tend / zero_tend2d.
template <typename R>
void zero_tend(R* t_p, const Dims& d) {
  A3<R> t(t_p, d);
  for (int j = d.jts; j <= d.jte; ++j)
    for (int k = d.kts; k <= d.kte; ++k)
      for (int i = d.its; i <= d.ite; ++i) t(i, k, j) = R(0.);
}
template <typename R>
void zero_tend2d(R* t_p, const Dims& d) {
  A2<R> t(t_p, d);
  for (int j = d.jts; j <= d.jte; ++j)
    for (int i = d.its; i <= d.ite; ++i) t(i, j) = R(0.);
}

// module_big_step_utilities_em.F:1365-2178 rhs_ph, phi_adv_z 1/2 vertical
// term, "gw" term, the advective_order <= 6 horizontal branch (:1768-1930 y,
// :1930-2075 x; next to an open boundary 4th- and 2nd-order stencils) and the
// open-boundary terms (:2077-2176).
template <typename R>
void rhs_ph(R* ph_tend_p, R* u_p, R* v_p, R* ww_p, R* ph_p, R* ph_old_p, R* phb_p, R* w_p, R* mut_p,
            R* muuf_p, R* muvf_p, R* c1f_p, R* c2f_p, R* fnm_p, R* fnp_p, R* rdnw_p, R cfn, R cfn1, R rdx,
            R rdy, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvx_inv_p, R* msfvy_p, R* msftx_p, R* msfty_p,
            int non_hydrostatic, const WrfDynConfig& cf, const Dims& d) {
  (void)msfuy_p; (void)msfvx_p; (void)msfvx_inv_p;
  A3<R> ph_tend(ph_tend_p, d), u(u_p, d), v(v_p, d), ww(ww_p, d), ph(ph_p, d), ph_old(ph_old_p, d), phb(phb_p, d),
      w(w_p, d);
  A2<R> mut(mut_p, d), muuf(muuf_p, d), muvf(muvf_p, d), msfux(msfux_p, d), msfvy(msfvy_p, d), msftx(msftx_p, d),
      msfty(msfty_p, d);
  A1<R> c1f(c1f_p, d), c2f(c2f_p, d), fnm(fnm_p, d), fnp(fnp_p, d), rdnw(rdnw_p, d);
  const R g = K<R>::g;
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1);
  const int kte = d.kte, kde = d.kde;
  int nx = d.ime - d.ims + 1;
  std::vector<R> wdwn_s((size_t)nx * (d.kme - d.kms + 1));
  auto wdwn = [&](int i, int k) -> R& { return wdwn_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  for (int j = d.jts; j <= jtf; ++j) {
    if (cf.phi_adv_z == 2) {
      for (int k = 2; k <= kte; ++k)
        for (int i = d.its; i <= itf; ++i)
          wdwn(i, k) = rdnw(k - 1) * (ph(i, k, j) - ph(i, k - 1, j) + phb(i, k, j) - phb(i, k - 1, j));
      for (int k = 2; k <= kte - 1; ++k)
        for (int i = d.its; i <= itf; ++i)
          ph_tend(i, k, j) = ph_tend(i, k, j) - ww(i, k, j) * (fnm(k) * wdwn(i, k + 1) + fnp(k) * wdwn(i, k));
    } else {
      for (int k = 2; k <= kte; ++k)
        for (int i = d.its; i <= itf; ++i)
          wdwn(i, k) = R(.5) * (ww(i, k, j) + ww(i, k - 1, j)) * rdnw(k - 1) *
                       (ph(i, k, j) - ph(i, k - 1, j) + phb(i, k, j) - phb(i, k - 1, j));
      for (int k = 2; k <= kte - 1; ++k)
        for (int i = d.its; i <= itf; ++i)
          ph_tend(i, k, j) = ph_tend(i, k, j) - (fnm(k) * wdwn(i, k + 1) + fnp(k) * wdwn(i, k));
    }
  }
  if (non_hydrostatic) {
    for (int j = d.jts; j <= jtf; ++j) {
      for (int i = d.its; i <= itf; ++i) ph_tend(i, kde, j) = R(0.);
      for (int k = 2; k <= kte; ++k)
        for (int i = d.its; i <= itf; ++i)
          ph_tend(i, k, j) = ph_tend(i, k, j) + (c1f(k) * mut(i, j) + c2f(k)) * g * w(i, k, j) / msfty(i, j);
    }
  }
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  // y (v) advection: the 6th-order centred stencil on ph+phb, 4th order two
  // rows and 2nd order one row in from an open boundary.
  auto yterm = [&](int i, int k, int j, int order) {
    const bool top = k == kte;
    auto vv = [&](int jj) -> R {
      return top ? (cfn * v(i, k - 1, jj) + cfn1 * v(i, k - 2, jj)) : (v(i, k, jj) + v(i, k - 1, jj));
    };
    const R cy = (top ? R(0.5) : R(0.25)) * rdy / msfty(i, j);
    const R fp = (c1f(k) * muvf(i, j + 1) + c2f(k)) * vv(j + 1) * msfvy(i, j + 1);
    const R fm = (c1f(k) * muvf(i, j) + c2f(k)) * vv(j) * msfvy(i, j);
    if (order == 6)
      ph_tend(i, k, j) = ph_tend(i, k, j) -
          cy * ((fp + fm) * (R(1.) / R(60.)) *
                (R(45.) * (ph(i, k, j + 1) - ph(i, k, j - 1)) - R(9.) * (ph(i, k, j + 2) - ph(i, k, j - 2)) +
                 (ph(i, k, j + 3) - ph(i, k, j - 3)) + R(45.) * (phb(i, k, j + 1) - phb(i, k, j - 1)) -
                 R(9.) * (phb(i, k, j + 2) - phb(i, k, j - 2)) + (phb(i, k, j + 3) - phb(i, k, j - 3))));
    else if (order == 4)
      ph_tend(i, k, j) = ph_tend(i, k, j) -
          cy * ((fp + fm) * (R(1.) / R(12.)) *
                (R(8.) * (ph(i, k, j + 1) - ph(i, k, j - 1)) - (ph(i, k, j + 2) - ph(i, k, j - 2)) +
                 R(8.) * (phb(i, k, j + 1) - phb(i, k, j - 1)) - (phb(i, k, j + 2) - phb(i, k, j - 2))));
    else
      ph_tend(i, k, j) = ph_tend(i, k, j) -
          cy * (fp * (phb(i, k, j + 1) - phb(i, k, j) + ph(i, k, j + 1) - ph(i, k, j)) +
                fm * (phb(i, k, j) - phb(i, k, j - 1) + ph(i, k, j) - ph(i, k, j - 1)));
  };
  auto xterm = [&](int i, int k, int j, int order) {
    const bool top = k == kte;
    auto uu = [&](int ii) -> R {
      return top ? (cfn * u(ii, k - 1, j) + cfn1 * u(ii, k - 2, j)) : (u(ii, k, j) + u(ii, k - 1, j));
    };
    const R cx = (top ? R(0.5) : R(0.25)) * rdx / msfty(i, j);
    const R fp = (c1f(k) * muuf(i + 1, j) + c2f(k)) * uu(i + 1) * msfux(i + 1, j);
    const R fm = (c1f(k) * muuf(i, j) + c2f(k)) * uu(i) * msfux(i, j);
    if (order == 6)
      ph_tend(i, k, j) = ph_tend(i, k, j) -
          cx * ((fp + fm) * (R(1.) / R(60.)) *
                (R(45.) * (ph(i + 1, k, j) - ph(i - 1, k, j)) - R(9.) * (ph(i + 2, k, j) - ph(i - 2, k, j)) +
                 (ph(i + 3, k, j) - ph(i - 3, k, j)) + R(45.) * (phb(i + 1, k, j) - phb(i - 1, k, j)) -
                 R(9.) * (phb(i + 2, k, j) - phb(i - 2, k, j)) + (phb(i + 3, k, j) - phb(i - 3, k, j))));
    else if (order == 4)
      ph_tend(i, k, j) = ph_tend(i, k, j) -
          cx * ((fp + fm) * (R(1.) / R(12.)) *
                (R(8.) * (ph(i + 1, k, j) - ph(i - 1, k, j)) - (ph(i + 2, k, j) - ph(i - 2, k, j)) +
                 R(8.) * (phb(i + 1, k, j) - phb(i - 1, k, j)) - (phb(i + 2, k, j) - phb(i - 2, k, j))));
    else
      ph_tend(i, k, j) = ph_tend(i, k, j) -
          cx * (fp * (phb(i + 1, k, j) - phb(i, k, j) + ph(i + 1, k, j) - ph(i, k, j)) +
                fm * (phb(i, k, j) - phb(i - 1, k, j) + ph(i, k, j) - ph(i - 1, k, j)));
  };
  itf = std::min(d.ite, ide - 1); jtf = std::min(d.jte, jde - 1);
  {
    int j_start = d.jts, jtf_y = jtf;
    if (cf.open_ys) j_start = std::max(d.jts, jds + 3);
    if (cf.open_ye) jtf_y = std::min(jtf_y, jde - 4);
    for (int j = j_start; j <= jtf_y; ++j)
      for (int k = 2; k <= kte; ++k)
        for (int i = d.its; i <= itf; ++i) yterm(i, k, j, 6);
    auto row = [&](int j, int order) {
      for (int k = 2; k <= kte; ++k)
        for (int i = d.its; i <= itf; ++i) yterm(i, k, j, order);
    };
    if (cf.open_ys && d.jts <= jds + 2 && jds + 2 <= d.jte) row(jds + 2, 4);
    if (cf.open_ye && d.jts <= jde - 3 && jde - 3 <= d.jte) row(jde - 3, 4);
    if (cf.open_ys && d.jts <= jds + 1 && jds + 1 <= d.jte) row(jds + 1, 2);
    if (cf.open_ye && d.jts <= jde - 2 && jde - 2 <= d.jte) row(jde - 2, 2);
  }
  // x (u) advection.
  {
    int i_start = d.its, itf_x = itf;
    if (cf.open_xs) i_start = std::max(d.its, ids + 3);
    if (cf.open_xe) itf_x = std::min(itf_x, ide - 4);
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = 2; k <= kte; ++k)
        for (int i = i_start; i <= itf_x; ++i) xterm(i, k, j, 6);
    auto col = [&](int i, int order) {
      for (int j = d.jts; j <= jtf; ++j)
        for (int k = 2; k <= kte; ++k) xterm(i, k, j, order);
    };
    if (cf.open_xs && d.its <= ids + 2 && ids + 2 <= d.ite) col(ids + 2, 4);
    if (cf.open_xe && d.its <= ide - 3 && ide - 3 <= d.ite) col(ide - 3, 4);
    if (cf.open_xs && d.its <= ids + 1 && ids + 1 <= d.ite) col(ids + 1, 2);
    if (cf.open_xe && d.its <= ide - 2 && ide - 2 <= d.ite) col(ide - 2, 2);
  }
  // lateral open boundary conditions: north and south, then east and west
  if (cf.open_ys && d.jts == jds) {
    const int j = d.jts;
    for (int k = 2; k <= kde; ++k) {
      const int kz = std::min(k, kde - 1);
      for (int i = d.its; i <= itf; ++i) {
        R vb = R(.5) * (fnm(kz) * (v(i, kz, j + 1) + v(i, kz, j)) + fnp(kz) * (v(i, kz - 1, j + 1) + v(i, kz - 1, j)));
        R vl = fminr(vb, R(0.));
        ph_tend(i, k, j) = ph_tend(i, k, j) - rdy * (c1f(k) * mut(i, j) + c2f(k)) * (vl * (ph_old(i, k, j + 1) - ph_old(i, k, j)));
      }
    }
  }
  if (cf.open_ye && d.jte == jde) {
    const int j = d.jte - 1;
    for (int k = 2; k <= kde; ++k) {
      const int kz = std::min(k, kde - 1);
      for (int i = d.its; i <= itf; ++i) {
        R vb = R(.5) * (fnm(kz) * (v(i, kz, j + 1) + v(i, kz, j)) + fnp(kz) * (v(i, kz - 1, j + 1) + v(i, kz - 1, j)));
        R vr = fmaxr(vb, R(0.));
        ph_tend(i, k, j) = ph_tend(i, k, j) - rdy * (c1f(k) * mut(i, j) + c2f(k)) * (vr * (ph_old(i, k, j) - ph_old(i, k, j - 1)));
      }
    }
  }
  if (cf.open_xs && d.its == ids) {
    const int i = d.its;
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = 2; k <= kde; ++k) {
        const int kz = k;  // the top level too (module_big_step_utilities_em.F:2137-2139)
        R ub = R(.5) * (fnm(kz) * (u(i + 1, kz, j) + u(i, kz, j)) + fnp(kz) * (u(i + 1, kz - 1, j) + u(i, kz - 1, j)));
        R ul = fminr(ub, R(0.));
        ph_tend(i, k, j) = ph_tend(i, k, j) - (msftx(i, j) / msfty(i, j)) * rdx * (c1f(k) * mut(i, j) + c2f(k)) *
                                                  (ul * (ph_old(i + 1, k, j) - ph_old(i, k, j)));
      }
  }
  if (cf.open_xe && d.ite == ide) {
    const int i = d.ite - 1;
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = 2; k <= kde; ++k) {
        const int kz = k < kde ? k : kde - 1;  // :2163-2164
        R ub = R(.5) * (fnm(kz) * (u(i + 1, kz, j) + u(i, kz, j)) + fnp(kz) * (u(i + 1, kz - 1, j) + u(i, kz - 1, j)));
        R ur = fmaxr(ub, R(0.));
        ph_tend(i, k, j) = ph_tend(i, k, j) - (msftx(i, j) / msfty(i, j)) * rdx * (c1f(k) * mut(i, j) + c2f(k)) *
                                                  (ur * (ph_old(i, k, j) - ph_old(i - 1, k, j)));
      }
  }
}

// module_big_step_utilities_em.F:2183-2418 (non-hydrostatic branch).
template <typename R>
void horizontal_pressure_gradient(R* ru_tend_p, R* rv_tend_p, R* ph_p, R* alt_p, R* p_p, R* pb_p, R* al_p,
                                  R* php_p, R* cqu_p, R* cqv_p, R* muu_p, R* muv_p, R* mu_p, R* c1h_p, R* c2h_p,
                                  R* fnm_p, R* fnp_p, R* rdnw_p, R cf1, R cf2, R cf3, R cfn, R cfn1, R rdx, R rdy,
                                  R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
                                  const WrfDynConfig& cf, int non_hydrostatic, int top_lid, const Dims& d) {
  (void)msftx_p; (void)msfty_p;
  A3<R> ru_tend(ru_tend_p, d), rv_tend(rv_tend_p, d), ph(ph_p, d), alt(alt_p, d), p(p_p, d), pb(pb_p, d),
      al(al_p, d), php(php_p, d), cqu(cqu_p, d), cqv(cqv_p, d);
  A2<R> muu(muu_p, d), muv(muv_p, d), mu(mu_p, d), msfux(msfux_p, d), msfuy(msfuy_p, d), msfvx(msfvx_p, d),
      msfvy(msfvy_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), fnm(fnm_p, d), fnp(fnp_p, d), rdnw(rdnw_p, d);
  A1<R> c1 = c1h;
  if (!non_hydrostatic) throw std::runtime_error("hydrostatic not supported");
  int nx = d.ime - d.ims + 1;
  std::vector<R> dpn_s((size_t)nx * (d.kme - d.kms + 1));
  auto dpn = [&](int i, int k) -> R& { return dpn_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  const int kde = d.kde;
  int itf = std::min(d.ite, d.ide - 1), jtf = d.jte, ktf = std::min(d.kte, d.kde - 1);
  int i_start = d.its, j_start = d.jts;
  // module_big_step_utilities_em.F:2273-2276
  if (cf.open_ys && d.jts == d.jds) j_start = d.jts + 1;
  if (cf.open_ye && d.jte == d.jde) jtf = jtf - 1;
  for (int j = j_start; j <= jtf; ++j) {
    int k = 1;
    for (int i = i_start; i <= itf; ++i) {
      dpn(i, k) = R(.5) * (cf1 * (p(i, k, j - 1) + p(i, k, j)) + cf2 * (p(i, k + 1, j - 1) + p(i, k + 1, j)) +
                           cf3 * (p(i, k + 2, j - 1) + p(i, k + 2, j)));
      dpn(i, kde) = R(0.);
    }
    if (top_lid)
      for (int i = i_start; i <= itf; ++i)
        dpn(i, kde) = R(.5) * (cfn * (p(i, kde - 1, j - 1) + p(i, kde - 1, j)) + cfn1 * (p(i, kde - 2, j - 1) + p(i, kde - 2, j)));
    for (k = 2; k <= ktf; ++k)
      for (int i = i_start; i <= itf; ++i)
        dpn(i, k) = R(.5) * (fnm(k) * (p(i, k, j - 1) + p(i, k, j)) + fnp(k) * (p(i, k - 1, j - 1) + p(i, k - 1, j)));
    for (k = 1; k <= ktf; ++k)
      for (int i = i_start; i <= itf; ++i) {
        R dpy = (msfvy(i, j) / msfvx(i, j)) * R(.5) * rdy * (c1h(k) * muv(i, j) + c2h(k)) *
                ((ph(i, k + 1, j) - ph(i, k + 1, j - 1) + ph(i, k, j) - ph(i, k, j - 1)) +
                 (alt(i, k, j) + alt(i, k, j - 1)) * (p(i, k, j) - p(i, k, j - 1)) +
                 (al(i, k, j) + al(i, k, j - 1)) * (pb(i, k, j) - pb(i, k, j - 1)));
        dpy = dpy + (msfvy(i, j) / msfvx(i, j)) * rdy * (php(i, k, j) - php(i, k, j - 1)) *
                        (rdnw(k) * (dpn(i, k + 1) - dpn(i, k)) - R(.5) * ((c1(k) * mu(i, j - 1)) + (c1(k) * mu(i, j))));
        rv_tend(i, k, j) = rv_tend(i, k, j) - cqv(i, k, j) * dpy;
      }
  }
  itf = d.ite; jtf = std::min(d.jte, d.jde - 1);
  i_start = d.its; j_start = d.jts;
  // :2346-2351
  if (cf.open_xs && d.its == d.ids) i_start = d.its + 1;
  if (cf.open_xe && d.ite == d.ide) itf = itf - 1;
  if (cf.periodic_x) { i_start = d.its; itf = d.ite; }
  for (int j = j_start; j <= jtf; ++j) {
    int k = 1;
    for (int i = i_start; i <= itf; ++i) {
      dpn(i, k) = R(.5) * (cf1 * (p(i - 1, k, j) + p(i, k, j)) + cf2 * (p(i - 1, k + 1, j) + p(i, k + 1, j)) +
                           cf3 * (p(i - 1, k + 2, j) + p(i, k + 2, j)));
      dpn(i, kde) = R(0.);
    }
    if (top_lid)
      for (int i = i_start; i <= itf; ++i)
        dpn(i, kde) = R(.5) * (cfn * (p(i - 1, kde - 1, j) + p(i, kde - 1, j)) + cfn1 * (p(i - 1, kde - 2, j) + p(i, kde - 2, j)));
    for (k = 2; k <= ktf; ++k)
      for (int i = i_start; i <= itf; ++i)
        dpn(i, k) = R(.5) * (fnm(k) * (p(i - 1, k, j) + p(i, k, j)) + fnp(k) * (p(i - 1, k - 1, j) + p(i, k - 1, j)));
    for (k = 1; k <= ktf; ++k)
      for (int i = i_start; i <= itf; ++i) {
        R dpx = (msfux(i, j) / msfuy(i, j)) * R(.5) * rdx * (c1h(k) * muu(i, j) + c2h(k)) *
                ((ph(i, k + 1, j) - ph(i - 1, k + 1, j) + ph(i, k, j) - ph(i - 1, k, j)) +
                 (alt(i, k, j) + alt(i - 1, k, j)) * (p(i, k, j) - p(i - 1, k, j)) +
                 (al(i, k, j) + al(i - 1, k, j)) * (pb(i, k, j) - pb(i - 1, k, j)));
        dpx = dpx + (msfux(i, j) / msfuy(i, j)) * rdx * (php(i, k, j) - php(i - 1, k, j)) *
                        (rdnw(k) * (dpn(i, k + 1) - dpn(i, k)) - R(.5) * ((c1(k) * mu(i - 1, j)) + (c1(k) * mu(i, j))));
        ru_tend(i, k, j) = ru_tend(i, k, j) - cqu(i, k, j) * dpx;
      }
  }
}

// module_big_step_utilities_em.F:2419-2502.  Overwrites cqw with 1/(1+cqw).
template <typename R>
void pg_buoy_w(R* rw_tend_p, R* p_p, R* cqw_p, R* muf_p, R* mubf_p, R* c1f_p, R* c2f_p, R* rdnw_p, R* rdn_p,
               R g, R* msftx_p, R* msfty_p, const Dims& d) {
  (void)msftx_p;
  A3<R> rw_tend(rw_tend_p, d), p(p_p, d), cqw(cqw_p, d);
  A2<R> muf(muf_p, d), mubf(mubf_p, d), msfty(msfty_p, d);
  A1<R> c1f(c1f_p, d), c2f(c2f_p, d), rdnw(rdnw_p, d), rdn(rdn_p, d);
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1);
  const int kde = d.kde;
  for (int j = d.jts; j <= jtf; ++j) {
    int k = kde;
    for (int i = d.its; i <= itf; ++i) {
      R cq1 = R(1.) / (R(1.) + cqw(i, k - 1, j));
      R cq2 = cqw(i, k - 1, j) * cq1;
      rw_tend(i, k, j) = rw_tend(i, k, j) + (R(1.) / msfty(i, j)) * g *
                                                (cq1 * R(2.) * rdnw(k - 1) * (-p(i, k - 1, j)) - (c1f(k) * muf(i, j)) -
                                                 cq2 * (c1f(k) * mubf(i, j) + c2f(k)));
    }
    for (k = 2; k <= kde - 1; ++k)
      for (int i = d.its; i <= itf; ++i) {
        R cq1 = R(1.) / (R(1.) + cqw(i, k, j));
        R cq2 = cqw(i, k, j) * cq1;
        cqw(i, k, j) = cq1;
        rw_tend(i, k, j) = rw_tend(i, k, j) + (R(1.) / msfty(i, j)) * g *
                                                  (cq1 * rdn(k) * (p(i, k, j) - p(i, k - 1, j)) - (c1f(k) * muf(i, j)) -
                                                   cq2 * (c1f(k) * mubf(i, j) + c2f(k)));
      }
  }
}

// module_big_step_utilities_em.F:2503-2712 w_damp: the CFL diagnostics, and
// with w_damping = 1 the damping of rw_tend where the vertical Courant
// number exceeds w_beta (:2689; zadvect_implicit = 0 on this path, so the
// activation number is w_beta, module_model_constants.F:88-89).
template <typename R>
void w_damp_cfl(R* rw_tend_p, R* u_p, R* v_p, R* ww_p, R* w_p, R* mut_p, R* c1f_p, R* c2f_p, R* rdnw_p, R rdx,
                R rdy, R* msfux_p, R* msfvy_p, R dt, const WrfDynConfig& cf, R* max_vert_cfl, R* max_horiz_cfl,
                const Dims& d) {
  A3<R> rw_tend(rw_tend_p, d), u(u_p, d), v(v_p, d), ww(ww_p, d), w(w_p, d);
  A2<R> mut(mut_p, d), msfux(msfux_p, d), msfvy(msfvy_p, d);
  A1<R> c1f(c1f_p, d), c2f(c2f_p, d), rdnw(rdnw_p, d);
  const R w_alpha = R(0.3), w_beta = R(1.0);
  const R w_crit_cfl = (R)cf.w_crit_cfl;
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1);
  R mv = 0, mh = 0;
  for (int j = d.jts; j <= jtf; ++j)
    for (int k = 2; k <= d.kde - 1; ++k)
      for (int i = d.its; i <= itf; ++i) {
        R vert_cfl = std::fabs(ww(i, k, j) / (c1f(k) * mut(i, j) + c2f(k)) * rdnw(k) * dt);
        if (vert_cfl > mv) mv = vert_cfl;
        R horiz_cfl = fmaxr(std::fabs(u(i, k, j) * rdx * msfux(i, j) * dt), std::fabs(v(i, k, j) * rdy * msfvy(i, j) * dt));
        if (horiz_cfl > mh) mh = horiz_cfl;
        if (vert_cfl > w_beta && cf.w_damping == 1)
          rw_tend(i, k, j) = rw_tend(i, k, j) - std::copysign(R(1.), w(i, k, j)) * w_alpha * (vert_cfl - w_crit_cfl) *
                                                    (c1f(k) * mut(i, j) + c2f(k));
      }
  *max_vert_cfl = mv; *max_horiz_cfl = mh;
}

// module_big_step_utilities_em.F:3640-3853.
template <typename R>
void coriolis(R* ru_p, R* rv_p, R* rw_p, R* ru_tend_p, R* rv_tend_p, R* rw_tend_p, const WrfDynConfig& cf,
              R* msftx_p, R* msfty_p, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* f_p, R* e_p, R* sina_p,
              R* cosa_p, R* fzm_p, R* fzp_p, const Dims& d) {
  A3<R> ru(ru_p, d), rv(rv_p, d), rw(rw_p, d), ru_tend(ru_tend_p, d), rv_tend(rv_tend_p, d), rw_tend(rw_tend_p, d);
  A2<R> msftx(msftx_p, d), msfty(msfty_p, d), msfux(msfux_p, d), msfuy(msfuy_p, d), msfvx(msfvx_p, d),
      msfvy(msfvy_p, d), f(f_p, d), e(e_p, d), sina(sina_p, d), cosa(cosa_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d);
  int ktf = std::min(d.kte, d.kde - 1);
  int i_start = d.its, i_end = d.ite;
  // module_big_step_utilities_em.F:3710-3717
  if (cf.open_xs) i_start = std::max(d.ids + 1, d.its);
  if (cf.open_xe) i_end = std::min(d.ide - 1, d.ite);
  if (cf.periodic_x) { i_start = d.its; i_end = d.ite; }
  for (int j = d.jts; j <= std::min(d.jte, d.jde - 1); ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        ru_tend(i, k, j) = ru_tend(i, k, j) +
                           (msfux(i, j) / msfuy(i, j)) * R(0.5) * (f(i, j) + f(i - 1, j)) * R(0.25) *
                               (rv(i - 1, k, j + 1) + rv(i, k, j + 1) + rv(i - 1, k, j) + rv(i, k, j)) -
                           R(0.5) * (e(i, j) + e(i - 1, j)) * R(0.5) * (cosa(i, j) + cosa(i - 1, j)) * R(0.25) *
                               (rw(i - 1, k + 1, j) + rw(i - 1, k, j) + rw(i, k + 1, j) + rw(i, k, j));
  int j_start = d.jts, j_end = d.jte;
  // :3765-3768
  if (cf.open_ys) j_start = std::max(d.jds + 1, d.jts);
  if (cf.open_ye) j_end = std::min(d.jde - 1, d.jte);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= std::min(d.ide - 1, d.ite); ++i)
        rv_tend(i, k, j) = rv_tend(i, k, j) -
                           (msfvy(i, j) / msfvx(i, j)) * R(0.5) * (f(i, j) + f(i, j - 1)) * R(0.25) *
                               (ru(i, k, j) + ru(i + 1, k, j) + ru(i, k, j - 1) + ru(i + 1, k, j - 1)) +
                           (msfvy(i, j) / msfvx(i, j)) * R(0.5) * (e(i, j) + e(i, j - 1)) * R(0.5) *
                               (sina(i, j) + sina(i, j - 1)) * R(0.25) *
                               (rw(i, k + 1, j - 1) + rw(i, k, j - 1) + rw(i, k + 1, j) + rw(i, k, j));
  for (int j = d.jts; j <= std::min(d.jte, d.jde - 1); ++j)
    for (int k = d.kts + 1; k <= ktf; ++k)
      for (int i = d.its; i <= std::min(d.ite, d.ide - 1); ++i)
        rw_tend(i, k, j) = rw_tend(i, k, j) +
                           e(i, j) * (cosa(i, j) * R(0.5) *
                                          (fzm(k) * (ru(i, k, j) + ru(i + 1, k, j)) + fzp(k) * (ru(i, k - 1, j) + ru(i + 1, k - 1, j))) -
                                      (msftx(i, j) / msfty(i, j)) * sina(i, j) * R(0.5) *
                                          (fzm(k) * (rv(i, k, j) + rv(i, k, j + 1)) + fzp(k) * (rv(i, k - 1, j) + rv(i, k - 1, j + 1))));
}

// module_big_step_utilities_em.F:4175-4469 (map_proj /= 6, not polar).
template <typename R>
void curvature(R* ru_p, R* rv_p, R* rw_p, R* u_p, R* v_p, R* w_p, R* ru_tend_p, R* rv_tend_p, R* rw_tend_p,
               const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
               R* xlat_p, R* fzm_p, R* fzp_p, R rdx, R rdy, const Dims& d) {
  (void)w_p; (void)xlat_p; (void)msfux_p;
  A3<R> ru(ru_p, d), rv(rv_p, d), rw(rw_p, d), u(u_p, d), v(v_p, d), ru_tend(ru_tend_p, d),
      rv_tend(rv_tend_p, d), rw_tend(rw_tend_p, d);
  A2<R> msfuy(msfuy_p, d), msfvx(msfvx_p, d), msfvy(msfvy_p, d), msftx(msftx_p, d), msfty(msfty_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d);
  const R reradius = K<R>::reradius;
  int ktf = std::min(d.kte, d.kde - 1);
  int nx = d.ime - d.ims + 1;
  // vxgm is a local (ims:ime, kms:kme, jms:jme) array in the reference.
  std::vector<R> vx_s((size_t)nx * (d.kme - d.kms + 1) * (d.jme - d.jms + 1));
  A3<R> vxgm(vx_s.data(), d);
  int i_start = d.its - 1, i_end = d.ite, j_start = d.jts - 1, j_end = d.jte;
  // module_big_step_utilities_em.F:4262-4271
  if (cf.open_xs && d.its == d.ids) i_start = d.its;
  if (cf.open_xe && d.ite == d.ide) i_end = d.ite - 1;
  if (cf.open_ys && d.jts == d.jds) j_start = d.jts;
  if (cf.open_ye && d.jte == d.jde) j_end = d.jte - 1;
  if (cf.periodic_x) { i_start = d.its - 1; i_end = d.ite; }
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        vxgm(i, k, j) = R(0.5) * (u(i, k, j) + u(i + 1, k, j)) * (msfvx(i, j + 1) - msfvx(i, j)) * rdy -
                        R(0.5) * (v(i, k, j) + v(i, k, j + 1)) * (msfuy(i + 1, j) - msfuy(i, j)) * rdx;
  // :4292-4298 (i_end keeps the vxgm bound unless open_xe narrows it)
  i_start = d.its;
  if (cf.open_xs) i_start = std::max(d.ids + 1, d.its);
  if (cf.open_xe) i_end = std::min(d.ide - 1, d.ite);
  if (cf.periodic_x) { i_start = d.its; i_end = d.ite; }
  for (int j = d.jts; j <= std::min(d.jde - 1, d.jte); ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        ru_tend(i, k, j) = ru_tend(i, k, j) +
                           R(0.5) * (vxgm(i, k, j) + vxgm(i - 1, k, j)) * R(0.25) *
                               (rv(i - 1, k, j + 1) + rv(i, k, j + 1) + rv(i - 1, k, j) + rv(i, k, j)) -
                           u(i, k, j) * reradius * R(0.25) *
                               (rw(i - 1, k + 1, j) + rw(i - 1, k, j) + rw(i, k + 1, j) + rw(i, k, j));
  // :4352-4356 (j_end keeps the vxgm bound unless open_ye narrows it)
  j_start = d.jts;
  if (cf.open_ys) j_start = std::max(d.jds + 1, d.jts);
  if (cf.open_ye) j_end = std::min(d.jde - 1, d.jte);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = d.its; i <= std::min(d.ite, d.ide - 1); ++i)
        rv_tend(i, k, j) = rv_tend(i, k, j) -
                           R(0.5) * (vxgm(i, k, j) + vxgm(i, k, j - 1)) * R(0.25) *
                               (ru(i, k, j) + ru(i + 1, k, j) + ru(i, k, j - 1) + ru(i + 1, k, j - 1)) -
                           (msfvy(i, j) / msfvx(i, j)) * v(i, k, j) * reradius * R(0.25) *
                               (rw(i, k + 1, j - 1) + rw(i, k, j - 1) + rw(i, k + 1, j) + rw(i, k, j));
  for (int j = d.jts; j <= std::min(d.jte, d.jde - 1); ++j)
    for (int k = std::max(2, d.kts); k <= ktf; ++k)
      for (int i = d.its; i <= std::min(d.ite, d.ide - 1); ++i)
        rw_tend(i, k, j) = rw_tend(i, k, j) +
                           reradius * (R(0.5) * (fzm(k) * (ru(i, k, j) + ru(i + 1, k, j)) + fzp(k) * (ru(i, k - 1, j) + ru(i + 1, k - 1, j))) *
                                           R(0.5) * (fzm(k) * (u(i, k, j) + u(i + 1, k, j)) + fzp(k) * (u(i, k - 1, j) + u(i + 1, k - 1, j))) +
                                       (msftx(i, j) / msfty(i, j)) * R(0.5) *
                                           (fzm(k) * (rv(i, k, j) + rv(i, k, j + 1)) + fzp(k) * (rv(i, k - 1, j) + rv(i, k - 1, j + 1))) *
                                           R(0.5) * (fzm(k) * (v(i, k, j) + v(i, k, j + 1)) + fzp(k) * (v(i, k - 1, j) + v(i, k - 1, j + 1))));
}

// Elementary functions of calc_p_rho_phi.  The reference calls the platform
// libm (LOG, and x**y through vspow / vpow); any libm within 1 ulp is a valid
// build of it, and they disagree in the last bit (glibc's logf is not
// correctly rounded for a few percent of these arguments).  The oracle pins
// the canonical value: the correctly rounded result, taken from the double
// libm and rounded once.  -DORACLE_PLATFORM_LIBM selects logf/powf instead.
template <typename R> static inline R olog(R x) { return std::log(x); }
template <typename R> static inline R opow(R x, R y) { return std::pow(x, y); }
#ifndef ORACLE_PLATFORM_LIBM
template <> inline float olog<float>(float x) { return (float)std::log((double)x); }
template <> inline float opow<float>(float x, float y) { return (float)std::pow((double)x, (double)y); }
#endif

// module_big_step_utilities_em.F:953-1226 calc_p_rho_phi, non-hydrostatic
// branch; VPOW is vspow (real*4 x**y) in the default build and vpow
// (real*8) under -r8 (module_big_step_utilities_em.F:4-10, frame/libmassv.F:375-390).
template <typename R>
void calc_p_rho_phi(R* qv_p, int n_moist_species, int hypsometric_opt, R* al_p, R* alb_p, R* mu_p, R* muts_p,
                    R* c1_p, R* c2_p, R* c3h_p, R* c4h_p, R* c3f_p, R* c4f_p, R* ph_p, R* phb_p, R* p_p, R* pb_p,
                    R* t_p, R p0, R t0, R ptop, R* znu_p, R* znw_p, R* dnw_p, R* rdnw_p, R* rdn_p,
                    int non_hydrostatic, int use_theta_m, const Dims& d) {
  (void)znu_p; (void)znw_p; (void)dnw_p; (void)rdn_p;
  A3<R> qv(qv_p, d), al(al_p, d), alb(alb_p, d), ph(ph_p, d), phb(phb_p, d), p(p_p, d), pb(pb_p, d), t(t_p, d);
  A2<R> mu(mu_p, d), muts(muts_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d), c3h(c3h_p, d), c4h(c4h_p, d), c3f(c3f_p, d), c4f(c4f_p, d), rdnw(rdnw_p, d);
  if (!non_hydrostatic) throw std::runtime_error("hydrostatic not supported");
  const R r_d = K<R>::r_d, cpovcv = K<R>::cpovcv, rvovrd = K<R>::rvovrd;
  int itf = std::min(d.ite, d.ide - 1), jtf = std::min(d.jte, d.jde - 1), ktf = std::min(d.kte, d.kde - 1);
  if (hypsometric_opt == 1) {
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i)
          al(i, k, j) = -R(1.) / (c1(k) * muts(i, j) + c2(k)) * (alb(i, k, j) * (c1(k) * mu(i, j)) + rdnw(k) * (ph(i, k + 1, j) - ph(i, k, j)));
  } else if (hypsometric_opt == 2) {
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i) {
          R pfu = c3f(k + 1) * muts(i, j) + c4f(k + 1) + ptop;
          R pfd = c3f(k) * muts(i, j) + c4f(k) + ptop;
          R phm = c3h(k) * muts(i, j) + c4h(k) + ptop;
          al(i, k, j) = (ph(i, k + 1, j) - ph(i, k, j) + phb(i, k + 1, j) - phb(i, k, j)) / phm / olog(pfd / pfu) - alb(i, k, j);
        }
  } else {
    throw std::runtime_error("calc_p_rho_phi: hypsometric_opt should be 1 or 2");
  }
  if (n_moist_species >= 1) {
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k) {
        for (int i = d.its; i <= itf; ++i) {
          R temp;
          if (use_theta_m == 1) {
            temp = (r_d * (t0 + t(i, k, j))) / (p0 * (al(i, k, j) + alb(i, k, j)));
          } else {
            R qvf = R(1.) + rvovrd * qv(i, k, j);
            temp = (r_d * (t0 + t(i, k, j)) * qvf) / (p0 * (al(i, k, j) + alb(i, k, j)));
          }
          p(i, k, j) = opow(temp, cpovcv);
        }
        for (int i = d.its; i <= itf; ++i) p(i, k, j) = p(i, k, j) * p0 - pb(i, k, j);
      }
  } else {
    for (int j = d.jts; j <= jtf; ++j)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = d.its; i <= itf; ++i)
          p(i, k, j) = p0 * opow((r_d * (t0 + t(i, k, j))) / (p0 * (al(i, k, j) + alb(i, k, j))), cpovcv) - pb(i, k, j);
  }
}

// module_big_step_utilities_em.F:6220-6636 sixth_order_diffusion: Xue's
// sixth-order flux, dropped where it runs up-gradient (diff_6th_opt = 2),
// tapered over steep terrain (diff_6th_slopeopt >= 1), weighted by the column
// mass, added to `tendency`.  name: 'u', 'v', 'w' or 'm' (mass-point
// scalars).  The loop limits of :6330-6443 (without the specified branch).
template <typename R>
void sixth_order_diffusion(char name, R* field_p, R* tendency_p, R* mut_p, R dt, const WrfDynConfig& cf, R* c1_p,
                           R* c2_p, R* phb_p, R rdx, R rdy, R* msftx_p, R* msfty_p, R* msfux_p, R* msfuy_p,
                           R* msfvx_p, R* msfvy_p, const Dims& d) {
  A3<R> field(field_p, d), tendency(tendency_p, d), phb(phb_p, d);
  A2<R> mut(mut_p, d), msftx(msftx_p, d), msfty(msfty_p, d), msfux(msfux_p, d), msfuy(msfuy_p, d),
      msfvx(msfvx_p, d), msfvy(msfvy_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const R coef = R(cf.diff_6th_factor) * R(0.015625) / (R(2.0) * dt);
  const int ktf = std::min(d.kte, d.kde - 1);
  int i_start = d.its, j_start = d.jts;
  int i_end = std::min(d.ide - 1, d.ite), j_end = std::min(d.jde - 1, d.jte), k_start = d.kts;
  if (name == 'u') i_end = d.ite;
  if (name == 'v') j_end = d.jte;
  if (name == 'w') k_start = d.kts + 1;
  // next to open boundaries (:6336-6443)
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  if (cf.open_xs) i_start = std::max(d.its, ids + 3);
  if (cf.open_ys) j_start = std::max(d.jts, jds + 3);
  if (name == 'u') {
    if (cf.open_xe) i_end = std::min(d.ite, ide - 3);
    if (cf.open_ye) j_end = std::min(d.jte, jde - 4);
  } else if (name == 'v') {
    if (cf.open_xe) i_end = std::min(d.ite, ide - 4);
    if (cf.open_ye) j_end = std::min(d.jte, jde - 3);
    if (cf.open_xs) {  // :6383-6388: all four limits on open_xs
      i_start = std::max(d.its, ids + 3); i_end = std::min(d.ite, ide - 4);
      j_start = std::max(d.jts, jds + 3); j_end = std::min(d.jte, jde - 3);
    }
  } else {
    if (cf.open_xe) i_end = std::min(d.ite, ide - 4);
    if (cf.open_ye) j_end = std::min(d.jte, jde - 4);
  }
  auto mass = [&](int k, int i, int j) { return c1(k) * mut(i, j) + c2(k); };
  // the sixth-order flux through the face between f(-1) and f(0) of a row
  auto flux6 = [](R fm3, R fm2, R fm1, R f0, R fp1, R fp2) {
    return R(10.0) * (f0 - fm1) - R(5.0) * (fp1 - fm2) + (fp2 - fm3);
  };
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        // x
        R fx0 = flux6(field(i - 3, k, j), field(i - 2, k, j), field(i - 1, k, j), field(i, k, j), field(i + 1, k, j),
                      field(i + 2, k, j));
        R fx1 = flux6(field(i - 2, k, j), field(i - 1, k, j), field(i, k, j), field(i + 1, k, j), field(i + 2, k, j),
                      field(i + 3, k, j));
        if (cf.diff_6th_opt == 2) {
          if (fx0 * (field(i, k, j) - field(i - 1, k, j)) <= R(0.)) fx0 = R(0.);
          if (fx1 * (field(i + 1, k, j) - field(i, k, j)) <= R(0.)) fx1 = R(0.);
        }
        R sd0 = R(1.), sd1 = R(1.);
        if (cf.diff_6th_slopeopt >= 1) {
          const R dx = R(1.) / rdx;
          const R thresh = R(cf.diff_6th_thresh) * R(9.81) * dx;
          R z0, z1;
          if (name == 'u') {
            z0 = std::max(std::fabs(phb(i, k, j) - phb(i - 1, k, j)) * msfux(i, j),
                          std::fabs(phb(i - 1, k, j) - phb(i - 2, k, j)) * msfux(i - 1, j));
            z1 = std::max(std::fabs(phb(i + 1, k, j) - phb(i, k, j)) * msfux(i + 1, j),
                          std::fabs(phb(i, k, j) - phb(i - 1, k, j)) * msfux(i, j));
          } else if (name == 'v') {
            z0 = std::max(std::fabs(phb(i, k, j) - phb(i - 1, k, j)) * msfux(i, j),
                          std::fabs(phb(i, k, j - 1) - phb(i - 1, k, j - 1)) * msfux(i, j - 1));
            z1 = std::max(std::fabs(phb(i + 1, k, j) - phb(i, k, j)) * msfux(i + 1, j),
                          std::fabs(phb(i + 1, k, j - 1) - phb(i, k, j - 1)) * msfux(i + 1, j - 1));
          } else {
            z0 = std::fabs(phb(i, k, j) - phb(i - 1, k, j)) * msfux(i, j);
            z1 = std::fabs(phb(i + 1, k, j) - phb(i, k, j)) * msfux(i + 1, j);
          }
          sd0 = std::max(R(1.) - (z0 / thresh), R(0.));
          sd1 = std::max(R(1.) - (z1 / thresh), R(0.));
        }
        R m0, m1, msf;
        if (name == 'u') {
          m0 = mass(k, i - 1, j); m1 = mass(k, i, j); msf = msfux(i, j);
        } else if (name == 'v') {
          m0 = R(0.25) * (mass(k, i - 1, j - 1) + mass(k, i, j - 1) + mass(k, i - 1, j) + mass(k, i, j));
          m1 = R(0.25) * (mass(k, i, j - 1) + mass(k, i + 1, j - 1) + mass(k, i, j) + mass(k, i + 1, j));
          msf = msfvx(i, j);
        } else {
          m0 = R(0.5) * (mass(k, i - 1, j) + mass(k, i, j));
          m1 = R(0.5) * (mass(k, i, j) + mass(k, i + 1, j));
          msf = msftx(i, j);
        }
        const R tx = coef * msf * ((sd1 * m1 * fx1) - (sd0 * m0 * fx0));
        // y
        R fy0 = flux6(field(i, k, j - 3), field(i, k, j - 2), field(i, k, j - 1), field(i, k, j), field(i, k, j + 1),
                      field(i, k, j + 2));
        R fy1 = flux6(field(i, k, j - 2), field(i, k, j - 1), field(i, k, j), field(i, k, j + 1), field(i, k, j + 2),
                      field(i, k, j + 3));
        if (cf.diff_6th_opt == 2) {
          if (fy0 * (field(i, k, j) - field(i, k, j - 1)) <= R(0.)) fy0 = R(0.);
          if (fy1 * (field(i, k, j + 1) - field(i, k, j)) <= R(0.)) fy1 = R(0.);
        }
        sd0 = R(1.); sd1 = R(1.);
        if (cf.diff_6th_slopeopt >= 1) {
          const R dy = R(1.) / rdy;
          const R thresh = R(cf.diff_6th_thresh) * R(9.81) * dy;
          R z0, z1;
          if (name == 'u') {
            z0 = std::max(std::fabs(phb(i, k, j) - phb(i, k, j - 1)) * msfvy(i, j),
                          std::fabs(phb(i - 1, k, j) - phb(i - 1, k, j - 1)) * msfvy(i - 1, j));
            z1 = std::max(std::fabs(phb(i, k, j + 1) - phb(i, k, j)) * msfvy(i, j + 1),
                          std::fabs(phb(i - 1, k, j + 1) - phb(i - 1, k, j)) * msfvy(i - 1, j + 1));
          } else if (name == 'v') {
            z0 = std::max(std::fabs(phb(i, k, j) - phb(i, k, j - 1)) * msfvy(i, j),
                          std::fabs(phb(i, k, j - 1) - phb(i, k, j - 2)) * msfvy(i, j - 1));
            z1 = std::max(std::fabs(phb(i, k, j + 1) - phb(i, k, j)) * msfvy(i, j + 1),
                          std::fabs(phb(i, k, j) - phb(i, k, j - 1)) * msfvy(i, j));
          } else {
            z0 = std::fabs(phb(i, k, j) - phb(i, k, j - 1)) * msfvy(i, j);
            z1 = std::fabs(phb(i, k, j + 1) - phb(i, k, j)) * msfvy(i, j + 1);
          }
          sd0 = std::max(R(1.) - (z0 / thresh), R(0.));
          sd1 = std::max(R(1.) - (z1 / thresh), R(0.));
        }
        if (name == 'u') {
          m0 = R(0.25) * (mass(k, i - 1, j - 1) + mass(k, i, j - 1) + mass(k, i - 1, j) + mass(k, i, j));
          m1 = R(0.25) * (mass(k, i - 1, j) + mass(k, i, j) + mass(k, i - 1, j + 1) + mass(k, i, j + 1));
          msf = msfuy(i, j);
        } else if (name == 'v') {
          m0 = mass(k, i, j - 1); m1 = mass(k, i, j); msf = msfvy(i, j);
        } else {
          m0 = R(0.5) * (mass(k, i, j - 1) + mass(k, i, j));
          m1 = R(0.5) * (mass(k, i, j) + mass(k, i, j + 1));
          msf = msfty(i, j);
        }
        const R ty = coef * msf * ((sd1 * m1 * fy1) - (sd0 * m0 * fy0));
        tendency(i, k, j) = tendency(i, k, j) + tx + ty;
      }
}

// ---------------------------------------------------------------------------
// Explicit diffusion (diff_opt = 1) with constant coefficients (km_opt = 1:
// isotropic_km, module_diffusion_em.F, fills xkmh with khdif and xkhh with
// khdif / prandtl everywhere, so each coefficient access below reads that
// one value `xk`; every expression keeps the reference's order).
// ---------------------------------------------------------------------------
// The loop limits of horizontal_diffusion / horizontal_diffusion_3dmp next to
// open boundaries (:2786-2790 u, :2834-2839 v, :2874-2879 w, :2919-2924 and
// :3026-3031 mass points; a periodic x keeps its limits).
inline void hdiff_open_limits(const WrfDynConfig& cf, char name, const Dims& d, int* i_start, int* i_end,
                              int* j_start, int* j_end) {
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  const int xe = name == 'u' ? ide - 1 : ide - 2, ye = name == 'v' ? jde - 1 : jde - 2;
  if (cf.open_xs) *i_start = std::max(ids + 1, d.its);
  if (cf.open_xe) *i_end = std::min(xe, d.ite);
  if (cf.open_ys) *j_start = std::max(jds + 1, d.jts);
  if (cf.open_ye) *j_end = std::min(ye, d.jte);
  if (cf.periodic_x) {
    *i_start = d.its;
    *i_end = name == 'u' ? d.ite : std::min(d.ite, d.ide - 1);
  }
}

// module_big_step_utilities_em.F:2715-2950 horizontal_diffusion
template <typename R>
void horizontal_diffusion(const WrfDynConfig& cf, char name, R* field_p, R* tendency_p, R* mut_p, R* c1_p, R* c2_p,
                          R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvx_inv_p, R* msfvy_p, R* msftx_p, R* msfty_p, R xk,
                          R rdx, R rdy, const Dims& d) {
  A3<R> field(field_p, d), tendency(tendency_p, d);
  A2<R> MUT(mut_p, d), msfux(msfux_p, d), msfuy(msfuy_p, d), msfvx(msfvx_p, d), msfvx_inv(msfvx_inv_p, d),
      msfvy(msfvy_p, d), msftx(msftx_p, d), msfty(msfty_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  int i_end = std::min(d.ite, d.ide - 1), j_end = std::min(d.jte, d.jde - 1), k_start = d.kts;
  if (name == 'u') i_end = d.ite;
  if (name == 'v') j_end = d.jte;
  if (name == 'w') k_start = d.kts + 1;
  int i_start = d.its, j_start = d.jts;
  hdiff_open_limits(cf, name, d, &i_start, &i_end, &j_start, &j_end);
  auto M = [&](int k, int i, int j) { return c1(k) * MUT(i, j) + c2(k); };
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mkrdxm, mkrdxp, mrdx, mkrdym, mkrdyp, mrdy;
        if (name == 'u') {
          mkrdxm = (msftx(i - 1, j) / msfty(i - 1, j)) * M(k, i - 1, j) * xk * rdx;
          mkrdxp = (msftx(i, j) / msfty(i, j)) * M(k, i, j) * xk * rdx;
          mrdx = msfux(i, j) * msfuy(i, j) * rdx;
          mkrdym = ((msfuy(i, j) + msfuy(i, j - 1)) / (msfux(i, j) + msfux(i, j - 1))) * R(0.25) *
                   (M(k, i, j) + M(k, i, j - 1) + M(k, i - 1, j - 1) + M(k, i - 1, j)) * R(0.25) *
                   (xk + xk + xk + xk) * rdy;
          mkrdyp = ((msfuy(i, j) + msfuy(i, j + 1)) / (msfux(i, j) + msfux(i, j + 1))) * R(0.25) *
                   (M(k, i, j) + M(k, i, j + 1) + M(k, i - 1, j + 1) + M(k, i - 1, j)) * R(0.25) *
                   (xk + xk + xk + xk) * rdy;
          mrdy = msfux(i, j) * msfuy(i, j) * rdy;
        } else if (name == 'v') {
          mkrdxm = ((msfvx(i, j) + msfvx(i - 1, j)) / (msfvy(i, j) + msfvy(i - 1, j))) * R(0.25) *
                   (M(k, i, j) + M(k, i, j - 1) + M(k, i - 1, j - 1) + M(k, i - 1, j)) * R(0.25) *
                   (xk + xk + xk + xk) * rdx;
          mkrdxp = ((msfvx(i, j) + msfvx(i + 1, j)) / (msfvy(i, j) + msfvy(i + 1, j))) * R(0.25) *
                   (M(k, i, j) + M(k, i, j - 1) + M(k, i + 1, j - 1) + M(k, i + 1, j)) * R(0.25) *
                   (xk + xk + xk + xk) * rdx;
          mrdx = msfvx(i, j) * msfvy(i, j) * rdx;
          mkrdym = (msfty(i, j - 1) / msftx(i, j - 1)) * xk * rdy;
          mkrdyp = (msfty(i, j) / msftx(i, j)) * xk * rdy;
          mrdy = msfvx(i, j) * msfvy(i, j) * rdy;
        } else if (name == 'w') {
          mkrdxm = (msfux(i, j) / msfuy(i, j)) * R(0.25) *
                   (M(k, i, j) + M(k, i - 1, j) + M(k, i, j) + M(k, i - 1, j)) * R(0.25) * (xk + xk + xk + xk) * rdx;
          mkrdxp = (msfux(i + 1, j) / msfuy(i + 1, j)) * R(0.25) *
                   (M(k, i + 1, j) + M(k, i, j) + M(k, i + 1, j) + M(k, i, j)) * R(0.25) * (xk + xk + xk + xk) * rdx;
          mrdx = msftx(i, j) * msfty(i, j) * rdx;
          mkrdym = (msfvy(i, j) * msfvx_inv(i, j)) * R(0.25) *
                   (M(k, i, j) + M(k, i, j - 1) + M(k, i, j) + M(k, i, j - 1)) * R(0.25) * (xk + xk + xk + xk) * rdy;
          mkrdyp = (msfvy(i, j + 1) * msfvx_inv(i, j + 1)) * R(0.25) *
                   (M(k, i, j + 1) + M(k, i, j) + M(k, i, j + 1) + M(k, i, j)) * R(0.25) * (xk + xk + xk + xk) * rdy;
          mrdy = msftx(i, j) * msfty(i, j) * rdy;
        } else {
          mkrdxm = (msfux(i, j) / msfuy(i, j)) * R(0.5) * (xk + xk) * R(0.5) * (M(k, i, j) + M(k, i - 1, j)) * rdx;
          mkrdxp = (msfux(i + 1, j) / msfuy(i + 1, j)) * R(0.5) * (xk + xk) * R(0.5) * (M(k, i + 1, j) + M(k, i, j)) * rdx;
          mrdx = msftx(i, j) * msfty(i, j) * rdx;
          mkrdym = (msfvy(i, j) * msfvx_inv(i, j)) * R(0.5) * (xk + xk) * R(0.5) * (M(k, i, j) + M(k, i, j - 1)) * rdy;
          mkrdyp = (msfvy(i, j + 1) * msfvx_inv(i, j + 1)) * R(0.5) * (xk + xk) * R(0.5) *
                   (M(k, i, j + 1) + M(k, i, j)) * rdy;
          mrdy = msftx(i, j) * msfty(i, j) * rdy;
        }
        tendency(i, k, j) = tendency(i, k, j) + (mrdx * (mkrdxp * (field(i + 1, k, j) - field(i, k, j)) -
                                                         mkrdxm * (field(i, k, j) - field(i - 1, k, j))) +
                                                 mrdy * (mkrdyp * (field(i, k, j + 1) - field(i, k, j)) -
                                                         mkrdym * (field(i, k, j) - field(i, k, j - 1))));
      }
}

// :2953-3060 horizontal_diffusion_3dmp: mass-point field minus its base state
template <typename R>
void horizontal_diffusion_3dmp(const WrfDynConfig& cf, R* field_p, R* tendency_p, R* mut_p, R* c1_p, R* c2_p,
                               R* base_p, R* msfux_p, R* msfuy_p, R* msfvx_inv_p, R* msfvy_p, R* msftx_p, R* msfty_p,
                               R xk, R rdx, R rdy, const Dims& d) {
  A3<R> field(field_p, d), tendency(tendency_p, d), base(base_p, d);
  A2<R> MUT(mut_p, d), msfux(msfux_p, d), msfuy(msfuy_p, d), msfvx_inv(msfvx_inv_p, d), msfvy(msfvy_p, d),
      msftx(msftx_p, d), msfty(msfty_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  auto M = [&](int k, int i, int j) { return c1(k) * MUT(i, j) + c2(k); };
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  hdiff_open_limits(cf, 'm', d, &i_start, &i_end, &j_start, &j_end);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        const R mkrdxm = (msfux(i, j) / msfuy(i, j)) * R(0.5) * (xk + xk) * R(0.5) * (M(k, i, j) + M(k, i - 1, j)) * rdx;
        const R mkrdxp =
            (msfux(i + 1, j) / msfuy(i + 1, j)) * R(0.5) * (xk + xk) * R(0.5) * (M(k, i + 1, j) + M(k, i, j)) * rdx;
        const R mrdx = msftx(i, j) * msfty(i, j) * rdx;
        const R mkrdym =
            (msfvy(i, j) * msfvx_inv(i, j)) * R(0.5) * (xk + xk) * R(0.5) * (M(k, i, j) + M(k, i, j - 1)) * rdy;
        const R mkrdyp = (msfvy(i, j + 1) * msfvx_inv(i, j + 1)) * R(0.5) * (xk + xk) * R(0.5) *
                         (M(k, i, j + 1) + M(k, i, j)) * rdy;
        const R mrdy = msftx(i, j) * msfty(i, j) * rdy;
        tendency(i, k, j) =
            tendency(i, k, j) +
            (mrdx * (mkrdxp * (field(i + 1, k, j) - field(i, k, j) - base(i + 1, k, j) + base(i, k, j)) -
                     mkrdxm * (field(i, k, j) - field(i - 1, k, j) - base(i, k, j) + base(i - 1, k, j))) +
             mrdy * (mkrdyp * (field(i, k, j + 1) - field(i, k, j) - base(i, k, j + 1) + base(i, k, j)) -
                     mkrdym * (field(i, k, j) - field(i, k, j - 1) - base(i, k, j) + base(i, k, j - 1))));
      }
}

// :3064-3581 vertical diffusion.  kind 'u' / 'v': vertical_diffusion_u / _v
// (the wind minus its base profile, levels kts..ktf-1); 'w': vertical_diffusion
// 'w' (levels kts+1..ktf); 'm': vertical_diffusion 'm' (no base); 'p':
// vertical_diffusion_mp (a 1-D base profile, qv); 't': vertical_diffusion_3dmp
// (a 3-D base state, theta).  mass: mut (u: muu, v: muv).
template <typename R>
void vertical_diffusion(const WrfDynConfig& cf, char kind, R* field_p, R* tendency_p, R* base1_p, R* base3_p, R* c1_p,
                        R* c2_p, R* alt_p, R* mass_p, R* rdn_p, R* rdnw_p, R kvdif, const Dims& d) {
  A3<R> field(field_p, d), tendency(tendency_p, d), alt(alt_p, d), base3(base3_p, d);
  A2<R> MASS(mass_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d), rdn(rdn_p, d), rdnw(rdnw_p, d), base1(base1_p, d);
  const R g = K<R>::g;
  const int ktf = std::min(d.kte, d.kde - 1);
  int i_start = d.its, i_end = kind == 'u' ? d.ite : std::min(d.ite, d.ide - 1);
  int j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  // next to open boundaries: vertical_diffusion_u leaves the boundary u out
  // (:3443-3446), vertical_diffusion_v the boundary v (:3545-3546)
  if (kind == 'u') {
    if (cf.open_xs) i_start = std::max(d.ids + 1, d.its);
    if (cf.open_xe) i_end = std::min(d.ide - 1, d.ite);
    if (cf.periodic_x) { i_start = d.its; i_end = d.ite; }
  }
  if (kind == 'v') {
    if (cf.open_ys) j_start = std::max(d.jds + 1, d.jts);
    if (cf.open_ye) j_end = std::min(d.jde - 1, d.jte);
  }
  std::vector<R> vf(d.kme - d.kms + 3);
  auto V = [&](int k) -> R& { return vf[k - d.kms + 1]; };  // vflux(0:kte+1)
  for (int j = j_start; j <= j_end; ++j)
    for (int i = i_start; i <= i_end; ++i) {
      if (kind == 'w') {
        for (int k = d.kts; k <= ktf - 1; ++k) V(k) = (kvdif / alt(i, k, j)) * rdnw(k) * (field(i, k + 1, j) - field(i, k, j));
        V(ktf) = R(0.);
        for (int k = d.kts + 1; k <= ktf; ++k)
          tendency(i, k, j) = tendency(i, k, j) + rdn(k) * g * g / (c1(k) * MASS(i, j) + c2(k)) /
                                                      (R(0.5) * (alt(i, k, j) + alt(i, k - 1, j))) * (V(k) - V(k - 1));
        continue;
      }
      for (int k = d.kts; k <= ktf - 1; ++k) {
        if (kind == 'u')
          V(k) = kvdif * rdn(k + 1) / (R(0.25) * (alt(i, k, j) + alt(i - 1, k, j) + alt(i, k + 1, j) + alt(i - 1, k + 1, j))) *
                 (field(i, k + 1, j) - field(i, k, j) - base1(k + 1) + base1(k));
        else if (kind == 'v')
          V(k) = kvdif * rdn(k + 1) / (R(0.25) * (alt(i, k, j) + alt(i, k, j - 1) + alt(i, k + 1, j) + alt(i, k + 1, j - 1))) *
                 (field(i, k + 1, j) - field(i, k, j) - base1(k + 1) + base1(k));
        else if (kind == 'm')
          V(k) = kvdif * rdn(k + 1) / (R(0.5) * (alt(i, k, j) + alt(i, k + 1, j))) * (field(i, k + 1, j) - field(i, k, j));
        else if (kind == 'p')
          V(k) = kvdif * rdn(k + 1) / (R(0.5) * (alt(i, k, j) + alt(i, k + 1, j))) *
                 (field(i, k + 1, j) - field(i, k, j) - base1(k + 1) + base1(k));
        else
          V(k) = kvdif * rdn(k + 1) / (R(0.5) * (alt(i, k, j) + alt(i, k + 1, j))) *
                 (field(i, k + 1, j) - field(i, k, j) - base3(i, k + 1, j) + base3(i, k, j));
      }
      V(d.kts - 1) = V(d.kts);
      V(ktf) = R(0.);
      if (kind == 'u' || kind == 'v') {
        for (int k = d.kts; k <= ktf - 1; ++k) {
          const R a = kind == 'u' ? R(0.5) * (alt(i - 1, k, j) + alt(i, k, j)) : R(0.5) * (alt(i, k, j - 1) + alt(i, k, j));
          tendency(i, k, j) = tendency(i, k, j) + g * g * rdnw(k) / (c1(k) * MASS(i, j) + c2(k)) / a * (V(k) - V(k - 1));
        }
      } else {
        for (int k = d.kts; k <= ktf; ++k)
          tendency(i, k, j) = tendency(i, k, j) + g * g / (c1(k) * MASS(i, j) + c2(k)) / alt(i, k, j) * rdnw(k) *
                                                      (V(k) - V(k - 1));
      }
    }
}

// module_big_step_utilities_em.F:5836-6110 rk_rayleigh_damp (damp_opt = 2):
// relaxation of u, v, w and theta toward the base-state profiles (u_base,
// v_base, t_base interpolated linearly in height z_base to the column's
// current level heights; w toward 0) in the top zdamp metres, with weight
// sin^2(pi/2 (1 - (ztop - z)/zdamp)) dampcoef times the column mass, added to
// the forward tendencies ru_tendf .. t_tendf.  The level searches stop at the
// first level (the reference's loops assume zdamp lies inside the model
// column).  sin in the working precision, correctly rounded (FP64 sine
// rounded once for the FP32 restatement).
template <typename R>
void rk_rayleigh_damp(R* ru_tendf_p, R* rv_tendf_p, R* rw_tendf_p, R* t_tendf_p, R* u_p, R* v_p, R* w_p, R* t_p,
                      R* c1h_p, R* c2h_p, R* c1f_p, R* c2f_p, R* mut_p, R* muu_p, R* muv_p, R* ph_p, R* phb_p,
                      R* u_base_p, R* v_base_p, R* t_base_p, R* z_base_p, R dampcoef, R zdamp, const Dims& d) {
  A3<R> ru_tendf(ru_tendf_p, d), rv_tendf(rv_tendf_p, d), rw_tendf(rw_tendf_p, d), t_tendf(t_tendf_p, d);
  A3<R> u(u_p, d), v(v_p, d), w(w_p, d), t(t_p, d), ph(ph_p, d), phb(phb_p, d);
  A2<R> mut(mut_p, d), muu(muu_p, d), muv(muv_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), c1f(c1f_p, d), c2f(c2f_p, d), u_base(u_base_p, d), v_base(v_base_p, d),
      t_base(t_base_p, d), z_base(z_base_p, d);
  const R g = K<R>::g;
  const R pii = R(2.0) * std::asin(R(1.0));
  const int ktf = std::min(d.kte, d.kde - 1);
  std::vector<R> z00(d.kme - d.kms + 2), q00(d.kme - d.kms + 2);
  auto Z = [&](int k) -> R& { return z00[k - d.kms]; };
  auto Q = [&](int k) -> R& { return q00[k - d.kms]; };
  auto weight = [&](R ztop, R z) {
    R dcoef = R(1.0) - std::min(R(1.0), (ztop - z) / zdamp);
    const R s = (R)std::sin((double)(R(0.5) * pii * dcoef));
    return s * s;
  };
  // level heights of the top layer of a column (the search of :5903-5913),
  // the profile interpolated to them (:5915-5930); returns the first level
  auto top_layer = [&](R ztop, auto height, const A1<R>& prof) {
    int k1 = ktf;
    R z = ztop;
    while (z >= ztop - zdamp && k1 >= d.kts) {
      z = height(k1);
      Z(k1) = z;
      k1 = k1 - 1;
    }
    k1 = k1 + 2;
    for (int k = k1; k <= ktf; ++k) {
      int k2 = ktf;
      while (z_base(k2) > Z(k) && k2 > d.kts) k2 = k2 - 1;
      if (k2 + 1 > ktf)
        Q(k) = prof(k2) + (prof(k2) - prof(k2 - 1)) * (Z(k) - z_base(k2)) / (z_base(k2) - z_base(k2 - 1));
      else
        Q(k) = prof(k2) + (prof(k2 + 1) - prof(k2)) * (Z(k) - z_base(k2)) / (z_base(k2 + 1) - z_base(k2));
    }
    return k1;
  };
  // u (:5897-5945)
  for (int j = d.jts; j <= std::min(d.jte, d.jde - 1); ++j)
    for (int i = d.its; i <= std::min(d.ite, d.ide); ++i) {
      const R ztop = R(0.5) * (phb(i, d.kde, j) + phb(i - 1, d.kde, j) + ph(i, d.kde, j) + ph(i - 1, d.kde, j)) / g;
      const int k1 = top_layer(ztop, [&](int k) {
        return R(0.25) * (phb(i, k, j) + phb(i, k + 1, j) + phb(i - 1, k, j) + phb(i - 1, k + 1, j) + ph(i, k, j) +
                          ph(i, k + 1, j) + ph(i - 1, k, j) + ph(i - 1, k + 1, j)) / g;
      }, u_base);
      for (int k = k1; k <= ktf; ++k)
        ru_tendf(i, k, j) = ru_tendf(i, k, j) - (c1h(k) * muu(i, j) + c2h(k)) * (weight(ztop, Z(k)) * dampcoef) *
                                                    (u(i, k, j) - Q(k));
    }
  // v (:5947-5995)
  for (int j = d.jts; j <= std::min(d.jte, d.jde); ++j)
    for (int i = d.its; i <= std::min(d.ite, d.ide - 1); ++i) {
      const R ztop = R(0.5) * (phb(i, d.kde, j) + phb(i, d.kde, j - 1) + ph(i, d.kde, j) + ph(i, d.kde, j - 1)) / g;
      const int k1 = top_layer(ztop, [&](int k) {
        return R(0.25) * (phb(i, k, j) + phb(i, k + 1, j) + phb(i, k, j - 1) + phb(i, k + 1, j - 1) + ph(i, k, j) +
                          ph(i, k + 1, j) + ph(i, k, j - 1) + ph(i, k + 1, j - 1)) / g;
      }, v_base);
      for (int k = k1; k <= ktf; ++k)
        rv_tendf(i, k, j) = rv_tendf(i, k, j) - (c1h(k) * muv(i, j) + c2h(k)) * (weight(ztop, Z(k)) * dampcoef) *
                                                    (v(i, k, j) - Q(k));
    }
  // w (:5997-6013) and theta (:6015-6062)
  for (int j = d.jts; j <= std::min(d.jte, d.jde - 1); ++j)
    for (int i = d.its; i <= std::min(d.ite, d.ide - 1); ++i) {
      const R ztop = (phb(i, d.kde, j) + ph(i, d.kde, j)) / g;
      for (int k = d.kts; k <= std::min(d.kte, d.kde); ++k) {
        const R z = (phb(i, k, j) + ph(i, k, j)) / g;
        if (z >= ztop - zdamp)
          rw_tendf(i, k, j) = rw_tendf(i, k, j) - (c1f(k) * mut(i, j) + c2f(k)) * (weight(ztop, z) * dampcoef) * w(i, k, j);
      }
      const int k1 = top_layer(
          ztop, [&](int k) { return R(0.5) * (phb(i, k, j) + phb(i, k + 1, j) + ph(i, k, j) + ph(i, k + 1, j)) / g; },
          t_base);
      for (int k = k1; k <= ktf; ++k)
        t_tendf(i, k, j) = t_tendf(i, k, j) - (c1h(k) * mut(i, j) + c2h(k)) * (weight(ztop, Z(k)) * dampcoef) *
                                                  (t(i, k, j) - Q(k));
    }
}

// module_em.F:959-1092 rk_addtend_dry for the forward-in-time tendencies this
// path forms (ru_tendf .. t_tendf: the sixth-order diffusion).  With physics
// off the saved tendencies (u_save .. t_save, ph_save), h_diabatic, ph_tendf
// and mu_tendf are zero: the stage-1 "tendf + save * msf" steps add +0 to a
// tendency that is never -0, and the ph / mu additions are left out; the
// h_diabatic term of theta is kept, as it can turn a -0 sum into +0.
template <typename R>
void rk_addtend_dry(R* ru_tend_p, R* rv_tend_p, R* rw_tend_p, R* t_tend_p, R* ru_tendf_p, R* rv_tendf_p,
                    R* rw_tendf_p, R* t_tendf_p, R* c1_p, R* c2_p, R* mut_p, R* msfty_p, R* msfuy_p,
                    R* msfvx_inv_p, const Dims& d) {
  A3<R> ru_tend(ru_tend_p, d), rv_tend(rv_tend_p, d), rw_tend(rw_tend_p, d), t_tend(t_tend_p, d),
      ru_tendf(ru_tendf_p, d), rv_tendf(rv_tendf_p, d), rw_tendf(rw_tendf_p, d), t_tendf(t_tendf_p, d);
  A2<R> mut(mut_p, d), msfty(msfty_p, d), msfuy(msfuy_p, d), msfvx_inv(msfvx_inv_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const int i_end = std::min(d.ite, d.ide - 1), j_end = std::min(d.jte, d.jde - 1);
  for (int j = d.jts; j <= j_end; ++j)
    for (int k = d.kts; k <= d.kte - 1; ++k)
      for (int i = d.its; i <= d.ite; ++i) ru_tend(i, k, j) = ru_tend(i, k, j) + ru_tendf(i, k, j) / msfuy(i, j);
  for (int j = d.jts; j <= d.jte; ++j)
    for (int k = d.kts; k <= d.kte - 1; ++k)
      for (int i = d.its; i <= i_end; ++i) rv_tend(i, k, j) = rv_tend(i, k, j) + rv_tendf(i, k, j) * msfvx_inv(i, j);
  for (int j = d.jts; j <= j_end; ++j)
    for (int k = d.kts; k <= d.kte; ++k)
      for (int i = d.its; i <= i_end; ++i) rw_tend(i, k, j) = rw_tend(i, k, j) + rw_tendf(i, k, j) / msfty(i, j);
  for (int j = d.jts; j <= j_end; ++j)
    for (int k = d.kts; k <= d.kte - 1; ++k)
      for (int i = d.its; i <= i_end; ++i)
        t_tend(i, k, j) = t_tend(i, k, j) + t_tendf(i, k, j) / msfty(i, j) +
                          (c1(k) * mut(i, j) + c2(k)) * R(0.) / msfty(i, j);
}

// module_em.F:959-1092 rk_addtend_dry, every term (the routine-level form):
// at stage 1 the saved tendencies join the forward ones, and every stage adds
// the forward ones to the large-step tendencies, theta's with its h_diabatic
// term; mu_tend += mu_tendf.
template <typename R>
void rk_addtend_dry_full(R* ru_tend_p, R* rv_tend_p, R* rw_tend_p, R* ph_tend_p, R* t_tend_p, R* ru_tendf_p,
                         R* rv_tendf_p, R* rw_tendf_p, R* ph_tendf_p, R* t_tendf_p, R* u_save_p, R* v_save_p,
                         R* w_save_p, R* ph_save_p, R* t_save_p, R* mu_tend_p, R* mu_tendf_p, int rk_step, R* c1_p,
                         R* c2_p, R* h_diabatic_p, R* mut_p, R* msfty_p, R* msfuy_p, R* msfvx_p, R* msfvx_inv_p,
                         const Dims& d) {
  A3<R> ru_tend(ru_tend_p, d), rv_tend(rv_tend_p, d), rw_tend(rw_tend_p, d), ph_tend(ph_tend_p, d),
      t_tend(t_tend_p, d), ru_tendf(ru_tendf_p, d), rv_tendf(rv_tendf_p, d), rw_tendf(rw_tendf_p, d),
      ph_tendf(ph_tendf_p, d), t_tendf(t_tendf_p, d), u_save(u_save_p, d), v_save(v_save_p, d),
      w_save(w_save_p, d), ph_save(ph_save_p, d), t_save(t_save_p, d), h_diabatic(h_diabatic_p, d);
  A2<R> mu_tend(mu_tend_p, d), mu_tendf(mu_tendf_p, d), mut(mut_p, d), msfty(msfty_p, d), msfuy(msfuy_p, d),
      msfvx(msfvx_p, d), msfvx_inv(msfvx_inv_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const int i_end = std::min(d.ite, d.ide - 1), j_end = std::min(d.jte, d.jde - 1);
  for (int j = d.jts; j <= j_end; ++j)
    for (int k = d.kts; k <= d.kte - 1; ++k)
      for (int i = d.its; i <= d.ite; ++i) {
        if (rk_step == 1) ru_tendf(i, k, j) = ru_tendf(i, k, j) + u_save(i, k, j) * msfuy(i, j);
        ru_tend(i, k, j) = ru_tend(i, k, j) + ru_tendf(i, k, j) / msfuy(i, j);
      }
  for (int j = d.jts; j <= d.jte; ++j)
    for (int k = d.kts; k <= d.kte - 1; ++k)
      for (int i = d.its; i <= i_end; ++i) {
        if (rk_step == 1) rv_tendf(i, k, j) = rv_tendf(i, k, j) + v_save(i, k, j) * msfvx(i, j);
        rv_tend(i, k, j) = rv_tend(i, k, j) + rv_tendf(i, k, j) * msfvx_inv(i, j);
      }
  for (int j = d.jts; j <= j_end; ++j)
    for (int k = d.kts; k <= d.kte; ++k)
      for (int i = d.its; i <= i_end; ++i) {
        if (rk_step == 1) rw_tendf(i, k, j) = rw_tendf(i, k, j) + w_save(i, k, j) * msfty(i, j);
        rw_tend(i, k, j) = rw_tend(i, k, j) + rw_tendf(i, k, j) / msfty(i, j);
        if (rk_step == 1) ph_tendf(i, k, j) = ph_tendf(i, k, j) + ph_save(i, k, j);
        ph_tend(i, k, j) = ph_tend(i, k, j) + ph_tendf(i, k, j) / msfty(i, j);
      }
  for (int j = d.jts; j <= j_end; ++j)
    for (int k = d.kts; k <= d.kte - 1; ++k)
      for (int i = d.its; i <= i_end; ++i) {
        if (rk_step == 1) t_tendf(i, k, j) = t_tendf(i, k, j) + t_save(i, k, j);
        t_tend(i, k, j) = t_tend(i, k, j) + t_tendf(i, k, j) / msfty(i, j) +
                          (c1(k) * mut(i, j) + c2(k)) * h_diabatic(i, k, j) / msfty(i, j);
      }
  for (int j = d.jts; j <= j_end; ++j)
    for (int i = d.its; i <= i_end; ++i) mu_tend(i, j) = mu_tend(i, j) + mu_tendf(i, j);
}

}  // namespace wrforacle
