// ORACLE — test infrastructure only (see wrf_oracle.hpp).
// Restatement of dyn_em/module_advect_em.F advect_u/v/w/scalar/scalar_pd for
// h_*_adv_order=5, v_*_adv_order=3 with periodic or symmetric lateral
// boundaries, where the reference's degrade_xs/xe/ys/ye are all .false.
// (module_advect_em.F:500-515) and every horizontal flux uses the full
// 6-point stencil.
#pragma once
#include "wrf_oracle.hpp"

namespace wrforacle {

inline void check_no_degrade(const WrfDynConfig& cf) {
  bool px = cf.periodic_x || (cf.symmetric_xs && cf.symmetric_xe);
  bool py = cf.periodic_y || (cf.symmetric_ys && cf.symmetric_ye);
  if (!px || !py) throw std::runtime_error("advection restatement needs periodic or symmetric boundaries");
}

// module_advect_em.F:126-1526 (5th-order horizontal :486-745, 3rd-order vertical :1470-1497).
template <typename R>
void advect_u(R* u_p, R* u_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p, R* mut_p,
              const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
              R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzw_p, const Dims& d) {
  (void)u_old_p; (void)c1_p; (void)c2_p; (void)mut_p; (void)msfuy_p; (void)msfvx_p; (void)msfvy_p;
  (void)msftx_p; (void)msfty_p;
  check_no_degrade(cf);
  A3<R> u(u_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msfux(msfux_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  // y flux divergence
  int i_start = d.its, i_end = d.ite;
  int j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = R(0.5) * (rv(i, k, j) + rv(i - 1, k, j));
        fqy(i, k, jp1) = vel * flux5(u(i, k, j - 3), u(i, k, j - 2), u(i, k, j - 1), u(i, k, j), u(i, k, j + 1), u(i, k, j + 2), vel);
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
  j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
  int i_start_f = i_start, i_end_f = i_end + 1;
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = R(0.5) * (ru(i, k, j) + ru(i - 1, k, j));
        fqx(i, k) = vel * flux5(u(i - 3, k, j), u(i - 2, k, j), u(i - 1, k, j), u(i, k, j), u(i + 1, k, j), u(i + 2, k, j), vel);
      }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msfux(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  // vertical
  i_start = d.its; i_end = d.ite; j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
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

// module_advect_em.F:1530-3024 (5th-order horizontal :1904-2171, 3rd-order vertical :2961-2995).
template <typename R>
void advect_v(R* v_p, R* v_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p, R* mut_p,
              const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
              R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzw_p, const Dims& d) {
  (void)v_old_p; (void)c1_p; (void)c2_p; (void)mut_p; (void)msfux_p; (void)msfuy_p; (void)msftx_p; (void)msfty_p;
  check_no_degrade(cf);
  A3<R> v(v_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msfvx(msfvx_p, d), msfvy(msfvy_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1);
  int j_start = d.jts, j_end = d.jte;
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = R(0.5) * (rv(i, k, j) + rv(i, k, j - 1));
        fqy(i, k, jp1) = vel * flux5(v(i, k, j - 3), v(i, k, j - 2), v(i, k, j - 1), v(i, k, j), v(i, k, j + 1), v(i, k, j + 2), vel);
      }
    if (j > j_start)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msfvy(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1);
  j_start = d.jts; j_end = d.jte;
  int i_start_f = i_start, i_end_f = i_end + 1;
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = R(0.5) * (ru(i, k, j) + ru(i, k, j - 1));
        fqx(i, k) = vel * flux5(v(i - 3, k, j), v(i - 2, k, j), v(i - 1, k, j), v(i, k, j), v(i + 1, k, j), v(i + 2, k, j), vel);
      }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msfvy(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1); j_start = d.jts; j_end = d.jte;
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

// module_advect_em.F:3029-4359 (5th-order horizontal :3394-3650, 3rd-order vertical :4306-4333).
template <typename R>
void advect_scalar(R* field_p, R* field_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p,
                   R* mut_p, const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p,
                   R* msfty_p, R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzw_p, const Dims& d) {
  (void)field_old_p; (void)c1_p; (void)c2_p; (void)mut_p; (void)msfux_p; (void)msfuy_p; (void)msfvx_p;
  (void)msfvy_p; (void)msfty_p;
  check_no_degrade(cf);
  A3<R> field(field_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msftx(msftx_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1);
  int j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = rv(i, k, j);
        fqy(i, k, jp1) = vel * flux5(field(i, k, j - 3), field(i, k, j - 2), field(i, k, j - 1), field(i, k, j),
                                     field(i, k, j + 1), field(i, k, j + 2), vel);
      }
    if (j > j_start)
      for (int k = d.kts; k <= ktf; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msftx(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
  int i_start_f = i_start, i_end_f = i_end + 1;
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = ru(i, k, j);
        fqx(i, k) = vel * flux5(field(i - 3, k, j), field(i - 2, k, j), field(i - 1, k, j), field(i, k, j),
                                field(i + 1, k, j), field(i + 2, k, j), vel);
      }
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msftx(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1); j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
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

// module_advect_em.F:4364-6064 (5th-order horizontal :4784-5096, 3rd-order vertical :5996-6031).
template <typename R>
void advect_w(R* w_p, R* w_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p, R* mut_p,
              const WrfDynConfig& cf, R* msfux_p, R* msfuy_p, R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p,
              R* fzm_p, R* fzp_p, R rdx, R rdy, R* rdzu_p, const Dims& d) {
  (void)w_old_p; (void)c1_p; (void)c2_p; (void)mut_p; (void)msfux_p; (void)msfuy_p; (void)msfvx_p;
  (void)msfvy_p; (void)msfty_p;
  check_no_degrade(cf);
  A3<R> w(w_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> msftx(msftx_p, d);
  A1<R> fzm(fzm_p, d), fzp(fzp_p, d), rdzu(rdzu_p, d);
  const int ktf = std::min(d.kte, d.kde - 1);
  const int nx = d.ime - d.ims + 1, nk = d.kme - d.kms + 1;
  std::vector<R> fqy_s((size_t)nx * nk * 2), fqx_s((size_t)nx * nk), vf_s((size_t)nx * nk);
  auto fqy = [&](int i, int k, int s) -> R& { return fqy_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx + (size_t)(s - 1) * nx * nk]; };
  auto fqx = [&](int i, int k) -> R& { return fqx_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  auto vflux = [&](int i, int k) -> R& { return vf_s[(size_t)(i - d.ims) + (size_t)(k - d.kms) * nx]; };
  int i_start = d.its, i_end = std::min(d.ite, d.ide - 1);
  int j_start = d.jts, j_end = std::min(d.jte, d.jde - 1);
  int jp1 = 2, jp0 = 1;
  for (int j = j_start; j <= j_end + 1; ++j) {
    for (int k = d.kts + 1; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R vel = fzm(k) * rv(i, k, j) + fzp(k) * rv(i, k - 1, j);
        fqy(i, k, jp1) = vel * flux5(w(i, k, j - 3), w(i, k, j - 2), w(i, k, j - 1), w(i, k, j), w(i, k, j + 1), w(i, k, j + 2), vel);
      }
    {
      int k = ktf + 1;
      for (int i = i_start; i <= i_end; ++i) {
        R vel = (R(2.) - fzm(k - 1)) * rv(i, k - 1, j) - fzp(k - 1) * rv(i, k - 2, j);
        fqy(i, k, jp1) = vel * flux5(w(i, k, j - 3), w(i, k, j - 2), w(i, k, j - 1), w(i, k, j), w(i, k, j + 1), w(i, k, j + 2), vel);
      }
    }
    if (j > j_start)
      for (int k = d.kts + 1; k <= ktf + 1; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          R mrdy = msftx(i, j - 1) * rdy;
          tendency(i, k, j - 1) = tendency(i, k, j - 1) - mrdy * (fqy(i, k, jp1) - fqy(i, k, jp0));
        }
    std::swap(jp1, jp0);
  }
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
  int i_start_f = i_start, i_end_f = i_end + 1;
  for (int j = j_start; j <= j_end; ++j) {
    for (int k = d.kts + 1; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = fzm(k) * ru(i, k, j) + fzp(k) * ru(i, k - 1, j);
        fqx(i, k) = vel * flux5(w(i - 3, k, j), w(i - 2, k, j), w(i - 1, k, j), w(i, k, j), w(i + 1, k, j), w(i + 2, k, j), vel);
      }
    {
      int k = ktf + 1;
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R vel = (R(2.) - fzm(k - 1)) * ru(i, k - 1, j) - fzp(k - 1) * ru(i, k - 2, j);
        fqx(i, k) = vel * flux5(w(i - 3, k, j), w(i - 2, k, j), w(i - 1, k, j), w(i, k, j), w(i + 1, k, j), w(i + 2, k, j), vel);
      }
    }
    for (int k = d.kts + 1; k <= ktf + 1; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R mrdx = msftx(i, j) * rdx;
        tendency(i, k, j) = tendency(i, k, j) - mrdx * (fqx(i + 1, k) - fqx(i, k));
      }
  }
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1); j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
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

// module_advect_em.F:6069-7885 (5th-order horizontal :6505-6779, 3rd-order
// vertical :7595-7645, limiter :7681-7781, divergence :7783-7883).
template <typename R>
void advect_scalar_pd(R* field_p, R* field_old_p, R* tend_p, R* ru_p, R* rv_p, R* rom_p, R* c1_p, R* c2_p,
                      R* mut_p, R* mub_p, R* mu_old_p, const WrfDynConfig& cf, R* msfux_p, R* msfuy_p,
                      R* msfvx_p, R* msfvy_p, R* msftx_p, R* msfty_p, R* fzm_p, R* fzp_p, R rdx, R rdy,
                      R* rdzw_p, R dt, const Dims& d) {
  (void)msfux_p; (void)msfuy_p; (void)msfvx_p; (void)msfvy_p;
  check_no_degrade(cf);
  A3<R> field(field_p, d), field_old(field_old_p, d), tendency(tend_p, d), ru(ru_p, d), rv(rv_p, d), rom(rom_p, d);
  A2<R> mut(mut_p, d), mub(mub_p, d), mu_old(mu_old_p, d), msftx(msftx_p, d), msfty(msfty_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d), fzm(fzm_p, d), fzp(fzp_p, d), rdzw(rdzw_p, d);
  const R eps = R(1.e-20);
  const int ktf = std::min(d.kte, d.kde - 1), kde = d.kde;
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

  // y fluxes (bounds for periodic and symmetric b.c.)
  int i_start = d.its - 1, i_end = std::min(d.ite, d.ide - 1) + 1;
  int j_start = d.jts - 1, j_end = std::min(d.jte, d.jde - 1) + 1;
  for (int j = j_start; j <= j_end + 1; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i) {
        R dy = R(2.) / (msftx(i, j) + msftx(i, j - 1)) / rdy;
        R mu = R(0.5) * ((c1(k) * mut(i, j) + c2(k)) + (c1(k) * mut(i, j - 1) + c2(k)));
        R vel = rv(i, k, j);
        R cr = vel * dt / dy / mu;
        fqyl(i, k, j) = mu * (dy / dt) * flux_upwind(field_old(i, k, j - 1), field_old(i, k, j), cr);
        fqy(i, k, j) = vel * pflux5(field(i, k, j - 3), field(i, k, j - 2), field(i, k, j - 1), field(i, k, j),
                                    field(i, k, j + 1), field(i, k, j + 2), vel);
        fqy(i, k, j) = fqy(i, k, j) - fqyl(i, k, j);
      }
  // x fluxes
  i_start = d.its - 1; i_end = std::min(d.ite, d.ide - 1) + 1;
  int i_start_f = i_start, i_end_f = i_end + 1;
  j_start = d.jts - 1; j_end = std::min(d.jte, d.jde - 1) + 1;
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start_f; i <= i_end_f; ++i) {
        R dx = R(2.) / (msfty(i, j) + msfty(i - 1, j)) / rdx;
        R mu = R(0.5) * ((c1(k) * mut(i, j) + c2(k)) + (c1(k) * mut(i - 1, j) + c2(k)));
        R vel = ru(i, k, j);
        R cr = vel * dt / dx / mu;
        fqxl(i, k, j) = mu * (dx / dt) * flux_upwind(field_old(i - 1, k, j), field_old(i, k, j), cr);
        fqx(i, k, j) = vel * pflux5(field(i - 3, k, j), field(i - 2, k, j), field(i - 1, k, j), field(i, k, j),
                                    field(i + 1, k, j), field(i + 2, k, j), vel);
        fqx(i, k, j) = fqx(i, k, j) - fqxl(i, k, j);
      }
  // z fluxes
  i_start = d.its - 1; i_end = std::min(d.ite, d.ide - 1) + 1;
  j_start = d.jts - 1; j_end = std::min(d.jte, d.jde - 1) + 1;
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
  // positive-definite limiter
  i_start = d.its - 1; i_end = std::min(d.ite, d.ide - 1) + 1;
  j_start = d.jts - 1; j_end = std::min(d.jte, d.jde - 1) + 1;
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
  i_start = d.its; i_end = std::min(d.ite, d.ide - 1);
  j_start = d.jts; j_end = std::min(d.jte, d.jde - 1);
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) -
                            rdzw(k) * (fqz(i, k + 1, j) - fqz(i, k, j) + fqzl(i, k + 1, j) - fqzl(i, k, j));
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) -
                            msftx(i, j) * (rdx * (fqx(i + 1, k, j) - fqx(i, k, j) + fqxl(i + 1, k, j) - fqxl(i, k, j)));
  for (int j = j_start; j <= j_end; ++j)
    for (int k = d.kts; k <= ktf; ++k)
      for (int i = i_start; i <= i_end; ++i)
        tendency(i, k, j) = tendency(i, k, j) -
                            msftx(i, j) * (rdy * (fqy(i, k, j + 1) - fqy(i, k, j) + fqyl(i, k, j + 1) - fqyl(i, k, j)));
}

}  // namespace wrforacle
