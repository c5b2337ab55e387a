// ORACLE — test infrastructure only (see wrf_oracle.hpp).
// Restatement of dyn_em/module_small_step_em.F: small_step_prep (:16-290),
// small_step_finish (:295-434), calc_p_rho (:438-568), calc_coef_w
// (:570-652), advance_uv (:654-967), advance_mu_t (:969-1175), advance_w
// (:1178-1469) and sumflux (:1473-1633); periodic/symmetric boundaries.
#pragma once
#include "wrf_oracle.hpp"

namespace wrforacle {

template <typename R>
void small_step_prep(R* u_1_p, R* u_2_p, R* v_1_p, R* v_2_p, R* w_1_p, R* w_2_p, R* t_1_p, R* t_2_p, R* ph_1_p,
                     R* ph_2_p, R* mub_p, R* mu_1_p, R* mu_2_p, R* muu_p, R* muus_p, R* muv_p, R* muvs_p,
                     R* mut_p, R* muts_p, R* mudf_p, R* c1h_p, R* c2h_p, R* c1f_p, R* c2f_p, R* u_save_p,
                     R* v_save_p, R* w_save_p, R* t_save_p, R* ph_save_p, R* mu_save_p, R* ww_p, R* ww_save_p,
                     R* c2a_p, R* pb_p, R* p_p, R* alt_p, R* msfuy_p, R* msfvx_inv_p, R* msfty_p, int rk_step,
                     const Dims& d) {
  A3<R> u_1(u_1_p, d), u_2(u_2_p, d), v_1(v_1_p, d), v_2(v_2_p, d), w_1(w_1_p, d), w_2(w_2_p, d), t_1(t_1_p, d),
      t_2(t_2_p, d), ph_1(ph_1_p, d), ph_2(ph_2_p, d), u_save(u_save_p, d), v_save(v_save_p, d),
      w_save(w_save_p, d), t_save(t_save_p, d), ph_save(ph_save_p, d), ww(ww_p, d), ww_save(ww_save_p, d),
      c2a(c2a_p, d), pb(pb_p, d), p(p_p, d), alt(alt_p, d);
  A2<R> mub(mub_p, d), MU_1(mu_1_p, d), MU_2(mu_2_p, d), MUU(muu_p, d), MUUS(muus_p, d), MUV(muv_p, d),
      MUVS(muvs_p, d), mut(mut_p, d), MUTS(muts_p, d), MUDF(mudf_p, d), MU_SAVE(mu_save_p, d),
      msfuy(msfuy_p, d), msfvx_inv(msfvx_inv_p, d), msfty(msfty_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), c1f(c1f_p, d), c2f(c2f_p, d);
  const R cpovcv = K<R>::cpovcv;
  const int kde = d.kde;
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int k_start = d.kts, k_end = std::min(d.kte, d.kde - 1), i_endu = d.ite, j_endv = d.jte;
  if (rk_step == 1) {
    for (int j = j_start; j <= j_end; ++j)
      for (int i = i_start; i <= i_end; ++i) {
        MU_1(i, j) = MU_2(i, j);
        ww_save(i, kde, j) = R(0.);
        ww_save(i, 1, j) = R(0.);
        MUDF(i, j) = R(0.);
      }
    for (int j = j_start; j <= j_end; ++j)
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_endu; ++i) u_1(i, k, j) = u_2(i, k, j);
    for (int j = j_start; j <= j_endv; ++j)
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i) v_1(i, k, j) = v_2(i, k, j);
    for (int j = j_start; j <= j_end; ++j)
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i) t_1(i, k, j) = t_2(i, k, j);
    for (int j = j_start; j <= j_end; ++j)
      for (int k = k_start; k <= std::min(kde, d.kte); ++k)
        for (int i = i_start; i <= i_end; ++i) { w_1(i, k, j) = w_2(i, k, j); ph_1(i, k, j) = ph_2(i, k, j); }
    for (int j = j_start; j <= j_end; ++j) {
      for (int i = i_start; i <= i_end; ++i) MUTS(i, j) = mub(i, j) + MU_2(i, j);
      for (int i = i_start; i <= i_endu; ++i) MUUS(i, j) = MUU(i, j);
    }
    for (int j = j_start; j <= j_endv; ++j)
      for (int i = i_start; i <= i_end; ++i) MUVS(i, j) = MUV(i, j);
    for (int j = j_start; j <= j_end; ++j)
      for (int i = i_start; i <= i_end; ++i) { MU_SAVE(i, j) = MU_2(i, j); MU_2(i, j) = R(0.); }
  } else {
    for (int j = j_start; j <= j_end; ++j) {
      for (int i = i_start; i <= i_end; ++i) MUTS(i, j) = mub(i, j) + MU_1(i, j);
      for (int i = i_start; i <= i_endu; ++i)
        MUUS(i, j) = R(0.5) * (mub(i, j) + MU_1(i, j) + mub(i - 1, j) + MU_1(i - 1, j));
    }
    for (int j = j_start; j <= j_endv; ++j)
      for (int i = i_start; i <= i_end; ++i)
        MUVS(i, j) = R(0.5) * (mub(i, j) + MU_1(i, j) + mub(i, j - 1) + MU_1(i, j - 1));
    for (int j = j_start; j <= j_end; ++j)
      for (int i = i_start; i <= i_end; ++i) { MU_SAVE(i, j) = MU_2(i, j); MU_2(i, j) = MU_1(i, j) - MU_2(i, j); }
  }
  for (int j = j_start; j <= j_end; ++j)
    for (int i = i_start; i <= i_end; ++i) { ww_save(i, kde, j) = R(0.); ww_save(i, 1, j) = R(0.); }
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) c2a(i, k, j) = cpovcv * (pb(i, k, j) + p(i, k, j)) / alt(i, k, j);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_endu; ++i) {
        u_save(i, k, j) = u_2(i, k, j);
        u_2(i, k, j) = ((c1h(k) * MUUS(i, j) + c2h(k)) * u_1(i, k, j) - (c1h(k) * MUU(i, j) + c2h(k)) * u_2(i, k, j)) / msfuy(i, j);
      }
  for (int j = j_start; j <= j_endv; ++j)
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        v_save(i, k, j) = v_2(i, k, j);
        v_2(i, k, j) = ((c1h(k) * MUVS(i, j) + c2h(k)) * v_1(i, k, j) - (c1h(k) * MUV(i, j) + c2h(k)) * v_2(i, k, j)) * msfvx_inv(i, j);
      }
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        t_save(i, k, j) = t_2(i, k, j);
        t_2(i, k, j) = (c1h(k) * MUTS(i, j) + c2h(k)) * t_1(i, k, j) - (c1h(k) * mut(i, j) + c2h(k)) * t_2(i, k, j);
      }
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= kde; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        w_save(i, k, j) = w_2(i, k, j);
        w_2(i, k, j) = ((c1f(k) * MUTS(i, j) + c2f(k)) * w_1(i, k, j) - (c1f(k) * mut(i, j) + c2f(k)) * w_2(i, k, j)) / msfty(i, j);
        ph_save(i, k, j) = ph_2(i, k, j);
        ph_2(i, k, j) = ph_1(i, k, j) - ph_2(i, k, j);
      }
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= kde; ++k)
      for (int i = i_start; i <= i_end; ++i) ww_save(i, k, j) = ww(i, k, j);
}

template <typename R>
void small_step_finish(R* u_2_p, R* u_1_p, R* v_2_p, R* v_1_p, R* w_2_p, R* w_1_p, R* t_2_p, R* t_1_p, R* ph_2_p,
                       R* ph_1_p, R* ww_p, R* ww1_p, R* mu_2_p, R* mu_1_p, R* mut_p, R* muts_p, R* muu_p,
                       R* muus_p, R* muv_p, R* muvs_p, R* c1h_p, R* c2h_p, R* c1f_p, R* c2f_p, R* u_save_p,
                       R* v_save_p, R* w_save_p, R* t_save_p, R* ph_save_p, R* mu_save_p, R* msfuy_p, R* msfvx_p,
                       R* msfty_p, R* h_diabatic_p, int number_of_small_timesteps, R dts, int rk_step,
                       int rk_order, const Dims& d) {
  (void)u_1_p; (void)v_1_p; (void)w_1_p; (void)t_1_p; (void)ph_1_p; (void)mu_1_p;
  A3<R> u_2(u_2_p, d), v_2(v_2_p, d), w_2(w_2_p, d), t_2(t_2_p, d), ph_2(ph_2_p, d), ww(ww_p, d), ww1(ww1_p, d),
      u_save(u_save_p, d), v_save(v_save_p, d), w_save(w_save_p, d), t_save(t_save_p, d), ph_save(ph_save_p, d);
  A2<R> mu_2(mu_2_p, d), mut(mut_p, d), muts(muts_p, d), muu(muu_p, d), muus(muus_p, d), muv(muv_p, d),
      muvs(muvs_p, d), mu_save(mu_save_p, d), msfuy(msfuy_p, d), msfvx(msfvx_p, d), msfty(msfty_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), c1f(c1f_p, d), c2f(c2f_p, d);
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int i_endu = d.ite, j_endv = d.jte;
  for (int j = j_start; j <= j_endv; ++j)
    for (int k = d.kds; k <= d.kde - 1; ++k)
      for (int i = i_start; i <= i_end; ++i)
        v_2(i, k, j) = (msfvx(i, j) * v_2(i, k, j) + v_save(i, k, j) * (c1h(k) * muv(i, j) + c2h(k))) / (c1h(k) * muvs(i, j) + c2h(k));
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kds; k <= d.kde - 1; ++k)
      for (int i = i_start; i <= i_endu; ++i)
        u_2(i, k, j) = (msfuy(i, j) * u_2(i, k, j) + u_save(i, k, j) * (c1h(k) * muu(i, j) + c2h(k))) / (c1h(k) * muus(i, j) + c2h(k));
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kds; k <= d.kde; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        w_2(i, k, j) = (msfty(i, j) * w_2(i, k, j) + w_save(i, k, j) * (c1f(k) * mut(i, j) + c2f(k))) / (c1f(k) * muts(i, j) + c2f(k));
        ph_2(i, k, j) = ph_2(i, k, j) + ph_save(i, k, j);
        ww(i, k, j) = ww(i, k, j) + ww1(i, k, j);
      }
  if (rk_step < rk_order) {
    for (int j = j_start; j <= j_end; ++j)
      for (int k = d.kds; k <= d.kde - 1; ++k)
        for (int i = i_start; i <= i_end; ++i)
          t_2(i, k, j) = (t_2(i, k, j) + t_save(i, k, j) * (c1h(k) * mut(i, j) + c2h(k))) / (c1h(k) * muts(i, j) + c2h(k));
  } else {
    A3<R> h_diabatic(h_diabatic_p, d);
    for (int j = j_start; j <= j_end; ++j)
      for (int k = d.kds; k <= d.kde - 1; ++k)
        for (int i = i_start; i <= i_end; ++i)
          t_2(i, k, j) = (t_2(i, k, j) - dts * R(number_of_small_timesteps) * (c1h(k) * mut(i, j) + c2h(k)) * h_diabatic(i, k, j) +
                          t_save(i, k, j) * (c1h(k) * mut(i, j) + c2h(k))) / (c1h(k) * muts(i, j) + c2h(k));
  }
  for (int j = j_start; j <= j_end; ++j)
    for (int i = i_start; i <= i_end; ++i) mu_2(i, j) = mu_2(i, j) + mu_save(i, j);
}

template <typename R>
void calc_p_rho(R* al_p, R* p_p, R* ph_p, R* alt_p, R* t_2_p, R* t_1_p, R* c2a_p, R* pm1_p, R* mu_p, R* mut_p,
                R* c1h_p, R* c2h_p, R t0, R* rdnw_p, R smdiv, int non_hydrostatic, int step, const Dims& d) {
  A3<R> al(al_p, d), p(p_p, d), ph(ph_p, d), alt(alt_p, d), t_2(t_2_p, d), t_1(t_1_p, d), c2a(c2a_p, d), pm1(pm1_p, d);
  A2<R> mu(mu_p, d), Mut(mut_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), rdnw(rdnw_p, d);
  if (!non_hydrostatic) throw std::runtime_error("hydrostatic not supported");
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int k_start = d.kts, k_end = std::min(d.kte, d.kde - 1);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        al(i, k, j) = -R(1.) / (c1h(k) * Mut(i, j) + c2h(k)) * (alt(i, k, j) * (c1h(k) * mu(i, j)) + rdnw(k) * (ph(i, k + 1, j) - ph(i, k, j)));
        p(i, k, j) = c2a(i, k, j) * (alt(i, k, j) * (t_2(i, k, j) - (c1h(k) * mu(i, j)) * t_1(i, k, j)) /
                                         ((c1h(k) * Mut(i, j) + c2h(k)) * (t0 + t_1(i, k, j))) - al(i, k, j));
      }
  if (step == 0) {
    for (int j = j_start; j <= j_end; ++j)
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i) pm1(i, k, j) = p(i, k, j);
  } else {
    for (int j = j_start; j <= j_end; ++j)
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R ptmp = p(i, k, j);
          p(i, k, j) = p(i, k, j) + smdiv * (p(i, k, j) - pm1(i, k, j));
          pm1(i, k, j) = ptmp;
        }
  }
}

template <typename R>
void calc_coef_w(R* a_p, R* alpha_p, R* gamma_p, R* mut_p, R* c1h_p, R* c2h_p, R* c1f_p, R* c2f_p, R* cqw_p,
                 R* rdn_p, R* rdnw_p, R* c2a_p, R dts, R g, R epssm, int top_lid, const Dims& d) {
  A3<R> a(a_p, d), alpha(alpha_p, d), gamma(gamma_p, d), cqw(cqw_p, d), c2a(c2a_p, d);
  A2<R> MUT(mut_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), c1f(c1f_p, d), c2f(c2f_p, d), rdn(rdn_p, d), rdnw(rdnw_p, d);
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  const int kde = d.kde;
  int lid_flag = top_lid ? 0 : 1;
  std::vector<R> cof_s(d.ime - d.ims + 1);
  auto cof = [&](int i) -> R& { return cof_s[i - d.ims]; };
  for (int j = j_start; j <= j_end; ++j) {
    int k = kde - 1;
    for (int i = i_start; i <= i_end; ++i) {
      R t = (R(.5) * dts * g * (R(1.) + epssm));
      cof(i) = t * t;
      a(i, 2, j) = R(0.);
      a(i, kde, j) = -R(2.) * cof(i) * (rdnw(kde - 1) * rdnw(kde - 1)) * c2a(i, kde - 1, j) * R(lid_flag) /
                     ((c1h(k) * MUT(i, j) + c2h(k)) * (c1f(k) * MUT(i, j) + c2f(k)));
      gamma(i, 1, j) = R(0.);
    }
    for (int kk = 3; kk <= kde - 1; ++kk) {
      k = kk - 1;
      for (int i = i_start; i <= i_end; ++i)
        a(i, kk, j) = -cqw(i, kk, j) * cof(i) * rdn(kk) * rdnw(kk - 1) * c2a(i, kk - 1, j) /
                      ((c1h(k) * MUT(i, j) + c2h(k)) * (c1f(k) * MUT(i, j) + c2f(k)));
    }
    for (k = 2; k <= kde - 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R b = R(1.) + cqw(i, k, j) * cof(i) * rdn(k) *
                          (rdnw(k) * c2a(i, k, j) / ((c1h(k) * MUT(i, j) + c2h(k)) * (c1f(k) * MUT(i, j) + c2f(k))) +
                           rdnw(k - 1) * c2a(i, k - 1, j) / ((c1h(k - 1) * MUT(i, j) + c2h(k - 1)) * (c1f(k) * MUT(i, j) + c2f(k))));
        R c = -cqw(i, k, j) * cof(i) * rdn(k) * rdnw(k) * c2a(i, k, j) /
              ((c1h(k) * MUT(i, j) + c2h(k)) * (c1f(k + 1) * MUT(i, j) + c2f(k + 1)));
        alpha(i, k, j) = R(1.) / (b - a(i, k, j) * gamma(i, k - 1, j));
        gamma(i, k, j) = c * alpha(i, k, j);
      }
    k = kde;
    for (int i = i_start; i <= i_end; ++i) {
      R b = R(1.) + R(2.) * cof(i) * (rdnw(kde - 1) * rdnw(kde - 1)) * c2a(i, kde - 1, j) /
                        ((c1h(k - 1) * MUT(i, j) + c2h(k - 1)) * (c1f(k) * MUT(i, j) + c2f(k)));
      R c = R(0.);
      alpha(i, kde, j) = R(1.) / (b - a(i, kde, j) * gamma(i, kde - 1, j));
      gamma(i, kde, j) = c * alpha(i, kde, j);
    }
  }
}

template <typename R>
void advance_uv(R* u_p, R* ru_tend_p, R* v_p, R* rv_tend_p, R* p_p, R* pb_p, R* ph_p, R* php_p, R* alt_p, R* al_p,
                R* mu_p, R* muu_p, R* cqu_p, R* muv_p, R* cqv_p, R* mudf_p, R* c1h_p, R* c2h_p, R* msfux_p,
                R* msfuy_p, R* msfvx_p, R* msfvx_inv_p, R* msfvy_p, R rdx, R rdy, R dts, R cf1, R cf2, R cf3,
                R* fnm_p, R* fnp_p, R emdiv, R* rdnw_p, const WrfDynConfig& cf, int non_hydrostatic, int top_lid,
                const Dims& d) {
  A3<R> u(u_p, d), ru_tend(ru_tend_p, d), v(v_p, d), rv_tend(rv_tend_p, d), p(p_p, d), pb(pb_p, d), ph(ph_p, d),
      php(php_p, d), alt(alt_p, d), al(al_p, d), cqu(cqu_p, d), cqv(cqv_p, d);
  A2<R> mu(mu_p, d), muu(muu_p, d), muv(muv_p, d), MUDF(mudf_p, d), msfux(msfux_p, d), msfuy(msfuy_p, d),
      msfvx(msfvx_p, d), msfvx_inv(msfvx_inv_p, d), msfvy(msfvy_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), fnm(fnm_p, d), fnp(fnp_p, d), rdnw(rdnw_p, d);
  if (!non_hydrostatic) throw std::runtime_error("hydrostatic not supported");
  const int kde = d.kde;
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int k_start = d.kts, k_end = d.kte - 1, i_endu = d.ite, j_endv = d.jte;
  int i_start_up = i_start, i_end_up = i_endu, j_start_vp = i_start * 0 + j_start, j_end_vp = j_endv;
  (void)j_end;
  if ((cf.open_xs || cf.symmetric_xs) && d.its == d.ids) i_start_up = i_start_up + 1;
  if ((cf.open_xe || cf.symmetric_xe) && d.ite == d.ide) i_end_up = i_end_up - 1;
  if ((cf.open_ys || cf.symmetric_ys || cf.polar) && d.jts == d.jds) j_start_vp = j_start_vp + 1;
  if ((cf.open_ye || cf.symmetric_ye || cf.polar) && d.jte == d.jde) j_end_vp = j_end_vp - 1;
  int i_start_u_tend = i_start, i_end_u_tend = i_endu, j_start_v_tend = j_start, j_end_v_tend = j_endv;
  if (cf.symmetric_xs && d.its == d.ids) i_start_u_tend = i_start_u_tend + 1;
  if (cf.symmetric_xe && d.ite == d.ide) i_end_u_tend = i_end_u_tend - 1;
  if (cf.symmetric_ys && d.jts == d.jds) j_start_v_tend = j_start_v_tend + 1;
  if (cf.symmetric_ye && d.jte == d.jde) j_end_v_tend = j_end_v_tend - 1;
  R dx = R(1.) / rdx, dy = R(1.) / rdy;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> dpn_s((size_t)nx * nk), dpxy_s((size_t)nx * nk), mxy_s(nx);
  auto dpn = [&](int i, int k) -> R& { return dpn_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto dpxy = [&](int i, int k) -> R& { return dpxy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto MUDF_XY = [&](int i) -> R& { return mxy_s[i - d.ims]; };
  for (int j = j_start; j <= std::min(d.jte, d.jde - 1); ++j) {
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start_u_tend; i <= i_end_u_tend; ++i) u(i, k, j) = u(i, k, j) + dts * ru_tend(i, k, j);
    for (int i = i_start_up; i <= i_end_up; ++i) MUDF_XY(i) = -emdiv * dx * (MUDF(i, j) - MUDF(i - 1, j)) / msfuy(i, j);
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start_up; i <= i_end_up; ++i)
        dpxy(i, k) = (msfux(i, j) / msfuy(i, j)) * R(.5) * rdx * (c1h(k) * muu(i, j) + c2h(k)) *
                     (((ph(i, k + 1, j) - ph(i - 1, k + 1, j)) + (ph(i, k, j) - ph(i - 1, k, j))) +
                      (alt(i, k, j) + alt(i - 1, k, j)) * (p(i, k, j) - p(i - 1, k, j)) +
                      (al(i, k, j) + al(i - 1, k, j)) * (pb(i, k, j) - pb(i - 1, k, j)));
    for (int i = i_start_up; i <= i_end_up; ++i) {
      dpn(i, 1) = R(.5) * (cf1 * (p(i, 1, j) + p(i - 1, 1, j)) + cf2 * (p(i, 2, j) + p(i - 1, 2, j)) + cf3 * (p(i, 3, j) + p(i - 1, 3, j)));
      dpn(i, kde) = R(0.);
    }
    if (top_lid)
      for (int i = i_start_up; i <= i_end_up; ++i)
        dpn(i, kde) = R(.5) * (cf1 * (p(i - 1, kde - 1, j) + p(i, kde - 1, j)) + cf2 * (p(i - 1, kde - 2, j) + p(i, kde - 2, j)) +
                               cf3 * (p(i - 1, kde - 3, j) + p(i, kde - 3, j)));
    for (int k = k_start + 1; k <= k_end; ++k)
      for (int i = i_start_up; i <= i_end_up; ++i)
        dpn(i, k) = R(.5) * (fnm(k) * (p(i, k, j) + p(i - 1, k, j)) + fnp(k) * (p(i, k - 1, j) + p(i - 1, k - 1, j)));
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start_up; i <= i_end_up; ++i)
        dpxy(i, k) = dpxy(i, k) + (msfux(i, j) / msfuy(i, j)) * rdx * (php(i, k, j) - php(i - 1, k, j)) *
                                      (rdnw(k) * (dpn(i, k + 1) - dpn(i, k)) - R(.5) * ((c1h(k) * mu(i - 1, j)) + (c1h(k) * mu(i, j))));
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start_up; i <= i_end_up; ++i)
        u(i, k, j) = u(i, k, j) - dts * cqu(i, k, j) * dpxy(i, k) + (c1h(k) * MUDF_XY(i));
  }
  for (int j = j_start_v_tend; j <= j_end_v_tend; ++j) {
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) v(i, k, j) = v(i, k, j) + dts * rv_tend(i, k, j);
    for (int i = i_start; i <= i_end; ++i) MUDF_XY(i) = -emdiv * dy * (MUDF(i, j) - MUDF(i, j - 1)) * msfvx_inv(i, j);
    if (j >= j_start_vp && j <= j_end_vp) {
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          dpxy(i, k) = (msfvy(i, j) / msfvx(i, j)) * R(.5) * rdy * (c1h(k) * muv(i, j) + c2h(k)) *
                       (((ph(i, k + 1, j) - ph(i, k + 1, j - 1)) + (ph(i, k, j) - ph(i, k, j - 1))) +
                        (alt(i, k, j) + alt(i, k, j - 1)) * (p(i, k, j) - p(i, k, j - 1)) +
                        (al(i, k, j) + al(i, k, j - 1)) * (pb(i, k, j) - pb(i, k, j - 1)));
      for (int i = i_start; i <= i_end; ++i) {
        dpn(i, 1) = R(.5) * (cf1 * (p(i, 1, j) + p(i, 1, j - 1)) + cf2 * (p(i, 2, j) + p(i, 2, j - 1)) + cf3 * (p(i, 3, j) + p(i, 3, j - 1)));
        dpn(i, kde) = R(0.);
      }
      if (top_lid)
        for (int i = i_start; i <= i_end; ++i)
          dpn(i, kde) = R(.5) * (cf1 * (p(i, kde - 1, j - 1) + p(i, kde - 1, j)) + cf2 * (p(i, kde - 2, j - 1) + p(i, kde - 2, j)) +
                                 cf3 * (p(i, kde - 3, j - 1) + p(i, kde - 3, j)));
      for (int k = k_start + 1; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          dpn(i, k) = R(.5) * (fnm(k) * (p(i, k, j) + p(i, k, j - 1)) + fnp(k) * (p(i, k - 1, j) + p(i, k - 1, j - 1)));
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          dpxy(i, k) = dpxy(i, k) + (msfvy(i, j) / msfvx(i, j)) * rdy * (php(i, k, j) - php(i, k, j - 1)) *
                                        (rdnw(k) * (dpn(i, k + 1) - dpn(i, k)) - R(.5) * ((c1h(k) * mu(i, j - 1)) + (c1h(k) * mu(i, j))));
      for (int k = k_start; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          v(i, k, j) = v(i, k, j) - dts * cqv(i, k, j) * dpxy(i, k) + (c1h(k) * MUDF_XY(i));
    }
  }
}

template <typename R>
void advance_mu_t(R* ww_p, R* ww_1_p, R* u_p, R* u_1_p, R* v_p, R* v_1_p, R* mu_p, R* mut_p, R* muave_p,
                  R* muts_p, R* muu_p, R* muv_p, R* mudf_p, R* c1h_p, R* c2h_p, R* t_p, R* t_1_p, R* t_ave_p,
                  R* ft_p, R* mu_tend_p, R rdx, R rdy, R dts, R epssm, R* dnw_p, R* fnm_p, R* fnp_p, R* rdnw_p,
                  R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvx_inv_p, R* msfvy_p, R* msftx_p, R* msfty_p,
                  const WrfDynConfig& cf, const Dims& d) {
  (void)msfux_p; (void)msfvx_p; (void)msfvy_p; (void)cf;
  A3<R> ww(ww_p, d), ww_1(ww_1_p, d), u(u_p, d), u_1(u_1_p, d), v(v_p, d), v_1(v_1_p, d), t(t_p, d), t_1(t_1_p, d),
      t_ave(t_ave_p, d), ft(ft_p, d);
  A2<R> MU(mu_p, d), MUT(mut_p, d), MUAVE(muave_p, d), MUTS(muts_p, d), muu(muu_p, d), muv(muv_p, d),
      MUDF(mudf_p, d), MU_TEND(mu_tend_p, d), msfuy(msfuy_p, d), msfvx_inv(msfvx_inv_p, d), msftx(msftx_p, d),
      msfty(msfty_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), dnw(dnw_p, d), fnm(fnm_p, d), fnp(fnp_p, d), rdnw(rdnw_p, d);
  const int kde = d.kde;
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int k_start = d.kts, k_end = d.kte - 1;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> dv_s((size_t)nx * nk), wd_s((size_t)nx * nk), dm_s(nx);
  auto dvdxi = [&](int i, int k) -> R& { return dv_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto wdtn = [&](int i, int k) -> R& { return wd_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto DMDT = [&](int i) -> R& { return dm_s[i - d.ims]; };
  for (int j = j_start; j <= j_end; ++j) {
    for (int i = i_start; i <= i_end; ++i) DMDT(i) = R(0.);
    for (int k = k_start; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        dvdxi(i, k) = msftx(i, j) * msfty(i, j) *
                      (rdy * ((v(i, k, j + 1) + (c1h(k) * muv(i, j + 1) + c2h(k)) * v_1(i, k, j + 1) * msfvx_inv(i, j + 1)) -
                              (v(i, k, j) + (c1h(k) * muv(i, j) + c2h(k)) * v_1(i, k, j) * msfvx_inv(i, j))) +
                       rdx * ((u(i + 1, k, j) + (c1h(k) * muu(i + 1, j) + c2h(k)) * u_1(i + 1, k, j) / msfuy(i + 1, j)) -
                              (u(i, k, j) + (c1h(k) * muu(i, j) + c2h(k)) * u_1(i, k, j) / msfuy(i, j))));
        DMDT(i) = DMDT(i) + dnw(k) * dvdxi(i, k);
      }
    for (int i = i_start; i <= i_end; ++i) {
      MUAVE(i, j) = MU(i, j);
      MU(i, j) = MU(i, j) + dts * (DMDT(i) + MU_TEND(i, j));
      MUDF(i, j) = (DMDT(i) + MU_TEND(i, j));
      MUTS(i, j) = MUT(i, j) + MU(i, j);
      MUAVE(i, j) = R(.5) * ((R(1.) + epssm) * MU(i, j) + (R(1.) - epssm) * MUAVE(i, j));
    }
    for (int kk = 2; kk <= k_end; ++kk) {
      int k = kk - 1;
      for (int i = i_start; i <= i_end; ++i)
        ww(i, kk, j) = ww(i, kk - 1, j) - dnw(kk - 1) * ((c1h(k) * DMDT(i)) + dvdxi(i, kk - 1) + (c1h(k) * MU_TEND(i, j))) / msfty(i, j);
    }
    for (int k = 1; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) ww(i, k, j) = ww(i, k, j) - ww_1(i, k, j);
  }
  for (int j = j_start; j <= j_end; ++j)
    for (int k = 1; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        t_ave(i, k, j) = t(i, k, j);
        t(i, k, j) = t(i, k, j) + msfty(i, j) * dts * ft(i, k, j);
      }
  for (int j = j_start; j <= j_end; ++j) {
    for (int i = i_start; i <= i_end; ++i) { wdtn(i, 1) = R(0.); wdtn(i, kde) = R(0.); }
    for (int k = 2; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) wdtn(i, k) = ww(i, k, j) * (fnm(k) * t_1(i, k, j) + fnp(k) * t_1(i, k - 1, j));
    for (int k = 1; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i)
        t(i, k, j) = t(i, k, j) - dts * msfty(i, j) *
                                      (msftx(i, j) * (R(.5) * rdy * (v(i, k, j + 1) * (t_1(i, k, j + 1) + t_1(i, k, j)) - v(i, k, j) * (t_1(i, k, j) + t_1(i, k, j - 1))) +
                                                      R(.5) * rdx * (u(i + 1, k, j) * (t_1(i + 1, k, j) + t_1(i, k, j)) - u(i, k, j) * (t_1(i, k, j) + t_1(i - 1, k, j)))) +
                                       rdnw(k) * (wdtn(i, k + 1) - wdtn(i, k)));
  }
}

template <typename R>
void advance_w(R* w_p, R* rw_tend_p, R* ww_p, R* w_save_p, R* u_p, R* v_p, R* mu1_p, R* mut_p, R* muave_p,
               R* muts_p, R* c1h_p, R* c2h_p, R* c1f_p, R* c2f_p, R* t_2ave_p, R* t_2_p, R* t_1_p, R* ph_p,
               R* ph_1_p, R* phb_p, R* ph_tend_p, R* ht_p, R* c2a_p, R* cqw_p, R* alt_p, R* alb_p, R* a_p,
               R* alpha_p, R* gamma_p, R rdx, R rdy, R dts, R t0, R epssm, R* dnw_p, R* fnm_p, R* fnp_p,
               R* rdnw_p, R* rdn_p, R cf1, R cf2, R cf3, R* msftx_p, R* msfty_p, const WrfDynConfig& cf,
               int top_lid, const Dims& d) {
  (void)mu1_p; (void)alb_p; (void)dnw_p;
  A3<R> w(w_p, d), rw_tend(rw_tend_p, d), ww(ww_p, d), u(u_p, d), v(v_p, d), t_2ave(t_2ave_p, d), t_2(t_2_p, d),
      t_1(t_1_p, d), ph(ph_p, d), ph_1(ph_1_p, d), phb(phb_p, d), ph_tend(ph_tend_p, d), c2a(c2a_p, d),
      cqw(cqw_p, d), alt(alt_p, d), a(a_p, d), alpha(alpha_p, d), gamma(gamma_p, d), w_save(w_save_p, d);
  A2<R> mut(mut_p, d), muave(muave_p, d), muts(muts_p, d), ht(ht_p, d), msftx(msftx_p, d), msfty(msfty_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d), c1f(c1f_p, d), c2f(c2f_p, d), fnm(fnm_p, d), fnp(fnp_p, d),
      rdnw(rdnw_p, d), rdn(rdn_p, d);
  const R g = K<R>::g;
  // damp_opt = 3 (:1283-1285): pi = 4 atan(1) in the working precision
  const R pi = R(4.) * std::atan(R(1.));
  const R dampmag = dts * (R)cf.dampcoef, hdepth = (R)cf.zdamp;
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1), j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int k_end = d.kte - 1;
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> rhs_s((size_t)nx * nk), wdwn_s((size_t)nx * nk), mi_s(nx);
  auto rhs = [&](int i, int k) -> R& { return rhs_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto wdwn = [&](int i, int k) -> R& { return wdwn_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto msft_inv = [&](int i) -> R& { return mi_s[i - d.ims]; };
  for (int i = i_start; i <= i_end; ++i) rhs(i, 1) = R(0.);
  for (int j = j_start; j <= j_end; ++j) {
    for (int i = i_start; i <= i_end; ++i) msft_inv(i) = R(1.) / msfty(i, j);
    for (int k = 1; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        t_2ave(i, k, j) = R(.5) * ((R(1.) + epssm) * t_2(i, k, j) + (R(1.) - epssm) * t_2ave(i, k, j));
        t_2ave(i, k, j) = (t_2ave(i, k, j) + (c1h(k) * muave(i, j)) * t0) / ((c1h(k) * muts(i, j) + c2h(k)) * (t0 + t_1(i, k, j)));
        rhs(i, k + 1) = dts * (ph_tend(i, k + 1, j) + R(.5) * g * (R(1.) - epssm) * w(i, k + 1, j));
      }
    if (cf.phi_adv_z == 2) {
      for (int k = 1; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          wdwn(i, k + 1) = rdnw(k) * (ph_1(i, k + 1, j) - ph_1(i, k, j) + phb(i, k + 1, j) - phb(i, k, j));
      for (int k = 2; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          rhs(i, k) = rhs(i, k) - dts * ww(i, k, j) * (fnm(k) * wdwn(i, k + 1) + fnp(k) * wdwn(i, k));
    } else {
      for (int k = 1; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          wdwn(i, k + 1) = R(.5) * (ww(i, k + 1, j) + ww(i, k, j)) * rdnw(k) *
                           (ph_1(i, k + 1, j) - ph_1(i, k, j) + phb(i, k + 1, j) - phb(i, k, j));
      for (int k = 2; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i)
          rhs(i, k) = rhs(i, k) - dts * (fnm(k) * wdwn(i, k + 1) + fnp(k) * wdwn(i, k));
    }
    for (int k = 2; k <= k_end + 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        rhs(i, k) = ph(i, k, j) + msfty(i, j) * rhs(i, k) / (c1f(k) * mut(i, j) + c2f(k));
        if (top_lid && k == k_end + 1) rhs(i, k) = R(0.);
      }
    for (int i = i_start; i <= i_end; ++i)
      w(i, 1, j) = msfty(i, j) * R(.5) * rdy *
                       ((ht(i, j + 1) - ht(i, j)) * (cf1 * v(i, 1, j + 1) + cf2 * v(i, 2, j + 1) + cf3 * v(i, 3, j + 1)) +
                        (ht(i, j) - ht(i, j - 1)) * (cf1 * v(i, 1, j) + cf2 * v(i, 2, j) + cf3 * v(i, 3, j))) +
                   msftx(i, j) * R(.5) * rdx *
                       ((ht(i + 1, j) - ht(i, j)) * (cf1 * u(i + 1, 1, j) + cf2 * u(i + 1, 2, j) + cf3 * u(i + 1, 3, j)) +
                        (ht(i, j) - ht(i - 1, j)) * (cf1 * u(i, 1, j) + cf2 * u(i, 2, j) + cf3 * u(i, 3, j)));
    for (int k = 2; k <= k_end; ++k)
      for (int i = i_start; i <= i_end; ++i)
        w(i, k, j) = w(i, k, j) + dts * rw_tend(i, k, j) +
                     msft_inv(i) * cqw(i, k, j) *
                         (+R(.5) * dts * g * rdn(k) *
                          (c2a(i, k, j) * rdnw(k) / (c1h(k) * mut(i, j) + c2h(k)) *
                               ((R(1.) + epssm) * (rhs(i, k + 1) - rhs(i, k)) + (R(1.) - epssm) * (ph(i, k + 1, j) - ph(i, k, j))) -
                           c2a(i, k - 1, j) * rdnw(k - 1) / (c1h(k - 1) * mut(i, j) + c2h(k - 1)) *
                               ((R(1.) + epssm) * (rhs(i, k) - rhs(i, k - 1)) + (R(1.) - epssm) * (ph(i, k, j) - ph(i, k - 1, j))))) +
                     dts * g * msft_inv(i) *
                         (rdn(k) * (c2a(i, k, j) * alt(i, k, j) * t_2ave(i, k, j) - c2a(i, k - 1, j) * alt(i, k - 1, j) * t_2ave(i, k - 1, j)) -
                          (c1f(k) * muave(i, j)));
    int k = k_end + 1;
    for (int i = i_start; i <= i_end; ++i) {
      w(i, k, j) = w(i, k, j) + dts * rw_tend(i, k, j) +
                   msft_inv(i) * (-R(.5) * dts * g / (c1h(k - 1) * mut(i, j) + c2h(k - 1)) * (rdnw(k - 1) * rdnw(k - 1)) * R(2.) * c2a(i, k - 1, j) *
                                      ((R(1.) + epssm) * (rhs(i, k) - rhs(i, k - 1)) + (R(1.) - epssm) * (ph(i, k, j) - ph(i, k - 1, j))) -
                                  dts * g * (R(2.) * rdnw(k - 1) * c2a(i, k - 1, j) * alt(i, k - 1, j) * t_2ave(i, k - 1, j) + (c1f(k) * muave(i, j))));
      if (top_lid) w(i, k, j) = R(0.);
    }
    for (k = 2; k <= k_end + 1; ++k)
      for (int i = i_start; i <= i_end; ++i) w(i, k, j) = (w(i, k, j) - a(i, k, j) * w(i, k - 1, j)) * alpha(i, k, j);
    for (k = k_end; k >= 2; --k)
      for (int i = i_start; i <= i_end; ++i) w(i, k, j) = w(i, k, j) - gamma(i, k, j) * w(i, k + 1, j);
    // implicit Rayleigh damping of w toward w_save in the top zdamp metres
    // (:1445-1458); sin in the working precision, correctly rounded (FP64
    // sine rounded once for the FP32 restatement)
    if (cf.damp_opt == 3) {
      for (k = k_end + 1; k >= 2; --k)
        for (int i = i_start; i <= i_end; ++i) {
          const R htop = (ph_1(i, k_end + 1, j) + phb(i, k_end + 1, j)) / g;
          const R hk = (ph_1(i, k, j) + phb(i, k, j)) / g;
          const R hbot = htop - hdepth;
          R dampwt = R(0.);
          if (hk >= hbot) {
            const R s = (R)std::sin((double)(R(.5) * pi * (hk - hbot) / hdepth));
            dampwt = dampmag * s * s;
          }
          w(i, k, j) = (w(i, k, j) - dampwt * (c1f(k) * mut(i, j) + c2f(k)) * w_save(i, k, j)) / (R(1.) + dampwt);
        }
    }
    for (k = k_end + 1; k >= 2; --k)
      for (int i = i_start; i <= i_end; ++i)
        ph(i, k, j) = rhs(i, k) + msfty(i, j) * R(.5) * dts * g * (R(1.) + epssm) * w(i, k, j) / (c1f(k) * muts(i, j) + c2f(k));
  }
}

template <typename R>
void sumflux(R* ru_p, R* rv_p, R* ww_p, R* u_lin_p, R* v_lin_p, R* ww_lin_p, R* muu_p, R* muv_p, R* c1h_p, R* c2h_p,
             R* ru_m_p, R* rv_m_p, R* ww_m_p, R* msfuy_p, R* msfvx_inv_p, int iteration,
             int number_of_small_timesteps, const Dims& d) {
  A3<R> ru(ru_p, d), rv(rv_p, d), ww(ww_p, d), u_lin(u_lin_p, d), v_lin(v_lin_p, d), ww_lin(ww_lin_p, d),
      ru_m(ru_m_p, d), rv_m(rv_m_p, d), ww_m(ww_m_p, d);
  A2<R> muu(muu_p, d), muv(muv_p, d), msfuy(msfuy_p, d), msfvx_inv(msfvx_inv_p, d);
  A1<R> c1h(c1h_p, d), c2h(c2h_p, d);
  if (iteration == 1)
    for (int j = d.jts; j <= d.jte; ++j)
      for (int k = d.kts; k <= d.kte; ++k)
        for (int i = d.its; i <= d.ite; ++i) { ru_m(i, k, j) = R(0.); rv_m(i, k, j) = R(0.); ww_m(i, k, j) = R(0.); }
  int mini = std::min(d.ide - 1, d.ite), minj = std::min(d.jde - 1, d.jte), mink = std::min(d.kde - 1, d.kte);
  for (int j = d.jts; j <= minj; ++j)
    for (int k = d.kts; k <= mink; ++k)
      for (int i = d.its; i <= mini; ++i) {
        ru_m(i, k, j) = ru_m(i, k, j) + ru(i, k, j);
        rv_m(i, k, j) = rv_m(i, k, j) + rv(i, k, j);
        ww_m(i, k, j) = ww_m(i, k, j) + ww(i, k, j);
      }
  if (d.ite > mini)
    for (int j = d.jts; j <= minj; ++j)
      for (int k = d.kts; k <= mink; ++k)
        for (int i = mini + 1; i <= d.ite; ++i) ru_m(i, k, j) = ru_m(i, k, j) + ru(i, k, j);
  if (d.jte > minj)
    for (int j = minj + 1; j <= d.jte; ++j)
      for (int k = d.kts; k <= mink; ++k)
        for (int i = d.its; i <= mini; ++i) rv_m(i, k, j) = rv_m(i, k, j) + rv(i, k, j);
  if (d.kte > mink)
    for (int j = d.jts; j <= minj; ++j)
      for (int k = mink + 1; k <= d.kte; ++k)
        for (int i = d.its; i <= mini; ++i) ww_m(i, k, j) = ww_m(i, k, j) + ww(i, k, j);
  if (iteration == number_of_small_timesteps) {
    const R ns = R(number_of_small_timesteps);
    for (int j = d.jts; j <= minj; ++j)
      for (int k = d.kts; k <= mink; ++k)
        for (int i = d.its; i <= mini; ++i) {
          ru_m(i, k, j) = ru_m(i, k, j) / ns + (c1h(k) * muu(i, j) + c2h(k)) * u_lin(i, k, j) / msfuy(i, j);
          rv_m(i, k, j) = rv_m(i, k, j) / ns + (c1h(k) * muv(i, j) + c2h(k)) * v_lin(i, k, j) * msfvx_inv(i, j);
          ww_m(i, k, j) = ww_m(i, k, j) / ns + ww_lin(i, k, j);
        }
    if (d.ite > mini)
      for (int j = d.jts; j <= minj; ++j)
        for (int k = d.kts; k <= mink; ++k)
          for (int i = mini + 1; i <= d.ite; ++i)
            ru_m(i, k, j) = ru_m(i, k, j) / ns + (c1h(k) * muu(i, j) + c2h(k)) * u_lin(i, k, j) / msfuy(i, j);
    if (d.jte > minj)
      for (int j = minj + 1; j <= d.jte; ++j)
        for (int k = d.kts; k <= mink; ++k)
          for (int i = d.its; i <= mini; ++i)
            rv_m(i, k, j) = rv_m(i, k, j) / ns + (c1h(k) * muv(i, j) + c2h(k)) * v_lin(i, k, j) * msfvx_inv(i, j);
    if (d.kte > mink)
      for (int j = d.jts; j <= minj; ++j)
        for (int k = mink + 1; k <= d.kte; ++k)
          for (int i = d.its; i <= mini; ++i) ww_m(i, k, j) = ww_m(i, k, j) / ns + ww_lin(i, k, j);
  }
}

}  // namespace wrforacle
