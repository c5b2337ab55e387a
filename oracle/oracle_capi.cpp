// ORACLE — test infrastructure only (see wrf_oracle.hpp).
// extern "C" surface of the CPU restatement, mirroring the coarse domain API
// of include/wrfgpu.h with an "oracle_f32_" / "oracle_f64_" prefix, plus a
// routine runner used by the kernel-level parity tests.
#include <cstdio>
#include <exception>
#include "oracle_solve.hpp"
#include "oracle_routines.h"

using namespace wrforacle;

namespace {
template <typename R>
int run_routine(Domain<R>& D, int routine, int rk_step, int iteration, int species) {
  using KR = K<R>;
  const R dt = R(D.sc.dt), rdx = R(D.sc.rdx), rdy = R(D.sc.rdy);
  const R cf1 = R(D.sc.cf1), cf2 = R(D.sc.cf2), cf3 = R(D.sc.cf3), cfn = R(D.sc.cfn), cfn1 = R(D.sc.cfn1);
  const R epssm = R(D.sc.epssm), smdiv = R(D.sc.smdiv), emdiv = R(D.sc.emdiv), p_top = R(D.sc.p_top);
  const int ns_total = D.num_sound_steps();
  const R dts = dt / R(ns_total);
  R dt_rk, dts_rk; int nsmall;
  if (rk_step == 1) { dt_rk = dt / R(3.); dts_rk = dt_rk; nsmall = 1; }
  else if (rk_step == 2) { dt_rk = R(0.5) * dt; dts_rk = dts; nsmall = ns_total / 2; }
  else { dt_rk = dt; dts_rk = dts; nsmall = ns_total; }
  const WrfDynConfig& cf = D.cf;
  auto p3 = [&](int id) { return D.p3(id); };
  auto p2 = [&](int id) { return D.p2(id); };
  auto p1 = [&](int id) { return D.p1(id); };
  const Dims td = D.d;
  switch (routine) {
    case ORACLE_R_RK_STEP_PREP:
      rk_step_prep(cf, rk_step, p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_W_2), p3(WRFGPU_T_2), p3(WRFGPU_PH_2),
                   p2(WRFGPU_MU_2), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F), p1(WRFGPU_C2F), D.q(0), D.n_moist,
                   p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_RW), p3(WRFGPU_WW), p3(WRFGPU_PHP), p3(WRFGPU_ALT),
                   p2(WRFGPU_MUU), p2(WRFGPU_MUV), p2(WRFGPU_MUB), p2(WRFGPU_MUT), p3(WRFGPU_PHB), p3(WRFGPU_PB),
                   p3(WRFGPU_P), p3(WRFGPU_AL), p3(WRFGPU_ALB), p3(WRFGPU_CQU), p3(WRFGPU_CQV), p3(WRFGPU_CQW),
                   p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY),
                   p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_DNW), rdx, rdy, td);
      return 0;
    case ORACLE_R_ZERO_TEND:
      zero_tend(p3(WRFGPU_RU_TEND), td); zero_tend(p3(WRFGPU_RV_TEND), td); zero_tend(p3(WRFGPU_RW_TEND), td);
      zero_tend(p3(WRFGPU_T_TEND), td); zero_tend(p3(WRFGPU_PH_TEND), td);
      zero_tend(p3(WRFGPU_U_SAVE), td); zero_tend(p3(WRFGPU_V_SAVE), td); zero_tend(p3(WRFGPU_W_SAVE), td);
      zero_tend(p3(WRFGPU_PH_SAVE), td); zero_tend(p3(WRFGPU_T_SAVE), td);
      zero_tend2d(p2(WRFGPU_MU_TEND), td); zero_tend2d(p2(WRFGPU_MU_SAVE), td);
      return 0;
    case ORACLE_R_ADVECT_U:
      advect_u(p3(WRFGPU_U_2), p3(WRFGPU_U_2), p3(WRFGPU_RU_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
               p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
               p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy,
               p1(WRFGPU_RDNW), td);
      return 0;
    case ORACLE_R_ADVECT_V:
      advect_v(p3(WRFGPU_V_2), p3(WRFGPU_V_2), p3(WRFGPU_RV_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
               p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
               p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy,
               p1(WRFGPU_RDNW), td);
      return 0;
    case ORACLE_R_ADVECT_W:
      advect_w(p3(WRFGPU_W_2), p3(WRFGPU_W_2), p3(WRFGPU_RW_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
               p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
               p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy,
               p1(WRFGPU_RDN), td);
      return 0;
    case ORACLE_R_ADVECT_T:
      advect_scalar(p3(WRFGPU_T_2), p3(WRFGPU_T_2), p3(WRFGPU_T_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
                    p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                    p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM),
                    p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW), td);
      return 0;
    case ORACLE_R_RHS_PH:
      rhs_ph(p3(WRFGPU_PH_TEND), p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_WW), p3(WRFGPU_PH_2), p3(WRFGPU_PH_2),
             p3(WRFGPU_PHB), p3(WRFGPU_W_2), p2(WRFGPU_MUT), p2(WRFGPU_MUU), p2(WRFGPU_MUV), p1(WRFGPU_C1F),
             p1(WRFGPU_C2F), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW), cfn, cfn1, rdx, rdy, p2(WRFGPU_MSFUX),
             p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX),
             p2(WRFGPU_MSFTY), cf.non_hydrostatic, cf, td);
      return 0;
    case ORACLE_R_HPG:
      horizontal_pressure_gradient(p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_PH_2), p3(WRFGPU_ALT),
                                   p3(WRFGPU_P), p3(WRFGPU_PB), p3(WRFGPU_AL), p3(WRFGPU_PHP), p3(WRFGPU_CQU),
                                   p3(WRFGPU_CQV), p2(WRFGPU_MUU), p2(WRFGPU_MUV), p2(WRFGPU_MU_2), p1(WRFGPU_C1H),
                                   p1(WRFGPU_C2H), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW), cf1, cf2, cf3, cfn,
                                   cfn1, rdx, rdy, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
                                   p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), cf, cf.non_hydrostatic,
                                   cf.top_lid, td);
      return 0;
    case ORACLE_R_PG_BUOY_W:
      pg_buoy_w(p3(WRFGPU_RW_TEND), p3(WRFGPU_P), p3(WRFGPU_CQW), p2(WRFGPU_MU_2), p2(WRFGPU_MUB), p1(WRFGPU_C1F),
                p1(WRFGPU_C2F), p1(WRFGPU_RDNW), p1(WRFGPU_RDN), KR::g, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), td);
      return 0;
    case ORACLE_R_CORIOLIS:
      coriolis(p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_RW), p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_RW_TEND),
               cf, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
               p2(WRFGPU_MSFVY), p2(WRFGPU_F), p2(WRFGPU_E), p2(WRFGPU_SINA), p2(WRFGPU_COSA), p1(WRFGPU_FNM),
               p1(WRFGPU_FNP), td);
      return 0;
    case ORACLE_R_CURVATURE:
      curvature(p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_RW), p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_W_2),
                p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_RW_TEND), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), (R*)nullptr, p1(WRFGPU_FNM),
                p1(WRFGPU_FNP), rdx, rdy, td);
      return 0;
    case ORACLE_R_SMALL_STEP_PREP:
      small_step_prep(p3(WRFGPU_U_1), p3(WRFGPU_U_2), p3(WRFGPU_V_1), p3(WRFGPU_V_2), p3(WRFGPU_W_1), p3(WRFGPU_W_2),
                      p3(WRFGPU_T_1), p3(WRFGPU_T_2), p3(WRFGPU_PH_1), p3(WRFGPU_PH_2), p2(WRFGPU_MUB), p2(WRFGPU_MU_1),
                      p2(WRFGPU_MU_2), p2(WRFGPU_MUU), p2(WRFGPU_MUUS), p2(WRFGPU_MUV), p2(WRFGPU_MUVS), p2(WRFGPU_MUT),
                      p2(WRFGPU_MUTS), p2(WRFGPU_MUDF), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F), p1(WRFGPU_C2F),
                      p3(WRFGPU_U_SAVE), p3(WRFGPU_V_SAVE), p3(WRFGPU_W_SAVE), p3(WRFGPU_T_SAVE), p3(WRFGPU_PH_SAVE),
                      p2(WRFGPU_MU_SAVE), p3(WRFGPU_WW), p3(WRFGPU_WW1), p3(WRFGPU_C2A), p3(WRFGPU_PB), p3(WRFGPU_P),
                      p3(WRFGPU_ALT), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFTY), rk_step, td);
      return 0;
    case ORACLE_R_CALC_P_RHO:
      calc_p_rho(p3(WRFGPU_AL), p3(WRFGPU_P), p3(WRFGPU_PH_2), p3(WRFGPU_ALT), p3(WRFGPU_T_2), p3(WRFGPU_T_SAVE),
                 p3(WRFGPU_C2A), p3(WRFGPU_PM1), p2(WRFGPU_MU_2), p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H), KR::t0,
                 p1(WRFGPU_RDNW), smdiv, cf.non_hydrostatic, iteration, td);
      return 0;
    case ORACLE_R_CALC_COEF_W:
      calc_coef_w(p3(WRFGPU_A), p3(WRFGPU_ALPHA), p3(WRFGPU_GAMMA), p2(WRFGPU_MUT), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                  p1(WRFGPU_C1F), p1(WRFGPU_C2F), p3(WRFGPU_CQW), p1(WRFGPU_RDN), p1(WRFGPU_RDNW), p3(WRFGPU_C2A), dts_rk,
                  KR::g, epssm, cf.top_lid, td);
      return 0;
    case ORACLE_R_ADVANCE_UV:
      advance_uv(p3(WRFGPU_U_2), p3(WRFGPU_RU_TEND), p3(WRFGPU_V_2), p3(WRFGPU_RV_TEND), p3(WRFGPU_P), p3(WRFGPU_PB),
                 p3(WRFGPU_PH_2), p3(WRFGPU_PHP), p3(WRFGPU_ALT), p3(WRFGPU_AL), p2(WRFGPU_MU_2), p2(WRFGPU_MUU),
                 p3(WRFGPU_CQU), p2(WRFGPU_MUV), p3(WRFGPU_CQV), p2(WRFGPU_MUDF), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                 p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY), rdx, rdy,
                 dts_rk, cf1, cf2, cf3, p1(WRFGPU_FNM), p1(WRFGPU_FNP), emdiv, p1(WRFGPU_RDNW), cf, cf.non_hydrostatic,
                 cf.top_lid, td);
      return 0;
    case ORACLE_R_ADVANCE_MU_T:
      advance_mu_t(p3(WRFGPU_WW), p3(WRFGPU_WW1), p3(WRFGPU_U_2), p3(WRFGPU_U_SAVE), p3(WRFGPU_V_2), p3(WRFGPU_V_SAVE),
                   p2(WRFGPU_MU_2), p2(WRFGPU_MUT), p2(WRFGPU_MUAVE), p2(WRFGPU_MUTS), p2(WRFGPU_MUU), p2(WRFGPU_MUV),
                   p2(WRFGPU_MUDF), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p3(WRFGPU_T_2), p3(WRFGPU_T_SAVE), p3(WRFGPU_T_2SAVE),
                   p3(WRFGPU_T_TEND), p2(WRFGPU_MU_TEND), rdx, rdy, dts_rk, epssm, p1(WRFGPU_DNW), p1(WRFGPU_FNM),
                   p1(WRFGPU_FNP), p1(WRFGPU_RDNW), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
                   p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), cf, td);
      return 0;
    case ORACLE_R_ADVANCE_W:
      advance_w(p3(WRFGPU_W_2), p3(WRFGPU_RW_TEND), p3(WRFGPU_WW), p3(WRFGPU_W_SAVE), p3(WRFGPU_U_2), p3(WRFGPU_V_2),
                p2(WRFGPU_MU_2), p2(WRFGPU_MUT), p2(WRFGPU_MUAVE), p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                p1(WRFGPU_C1F), p1(WRFGPU_C2F), p3(WRFGPU_T_2SAVE), p3(WRFGPU_T_2), p3(WRFGPU_T_SAVE), p3(WRFGPU_PH_2),
                p3(WRFGPU_PH_SAVE), p3(WRFGPU_PHB), p3(WRFGPU_PH_TEND), p2(WRFGPU_HT), p3(WRFGPU_C2A), p3(WRFGPU_CQW),
                p3(WRFGPU_ALT), p3(WRFGPU_ALB), p3(WRFGPU_A), p3(WRFGPU_ALPHA), p3(WRFGPU_GAMMA), rdx, rdy, dts_rk,
                KR::t0, epssm, p1(WRFGPU_DNW), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW), p1(WRFGPU_RDN), cf1, cf2,
                cf3, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), cf, cf.top_lid, td);
      return 0;
    case ORACLE_R_SUMFLUX:
      sumflux(p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_WW), p3(WRFGPU_U_SAVE), p3(WRFGPU_V_SAVE), p3(WRFGPU_WW1),
              p2(WRFGPU_MUU), p2(WRFGPU_MUV), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p3(WRFGPU_RU_M), p3(WRFGPU_RV_M),
              p3(WRFGPU_WW_M), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX_INV), iteration, nsmall, td);
      return 0;
    case ORACLE_R_SMALL_STEP_FINISH:
      calc_mu_uv_1(cf, p2(WRFGPU_MUTS), p2(WRFGPU_MUUS), p2(WRFGPU_MUVS), td);
      small_step_finish(p3(WRFGPU_U_2), p3(WRFGPU_U_1), p3(WRFGPU_V_2), p3(WRFGPU_V_1), p3(WRFGPU_W_2), p3(WRFGPU_W_1),
                        p3(WRFGPU_T_2), p3(WRFGPU_T_1), p3(WRFGPU_PH_2), p3(WRFGPU_PH_1), p3(WRFGPU_WW), p3(WRFGPU_WW1),
                        p2(WRFGPU_MU_2), p2(WRFGPU_MU_1), p2(WRFGPU_MUT), p2(WRFGPU_MUTS), p2(WRFGPU_MUU),
                        p2(WRFGPU_MUUS), p2(WRFGPU_MUV), p2(WRFGPU_MUVS), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F),
                        p1(WRFGPU_C2F), p3(WRFGPU_U_SAVE), p3(WRFGPU_V_SAVE), p3(WRFGPU_W_SAVE), p3(WRFGPU_T_SAVE),
                        p3(WRFGPU_PH_SAVE), p2(WRFGPU_MU_SAVE), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFTY),
                        p3(WRFGPU_H_DIABATIC), nsmall, dts_rk, rk_step, D.cf.rk_ord, td);
      return 0;
    case ORACLE_R_UPDATE_SCALAR_PD:
      rk_update_scalar_pd(D.qold(species), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MU_1), p2(WRFGPU_MU_1),
                          p2(WRFGPU_MUB), dt_rk, (R*)nullptr, td);
      return 0;
    case ORACLE_R_UPDATE_SCALAR_PD_ARGS:
      rk_update_scalar_pd(D.qold(species), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MU_1), p2(WRFGPU_MU_2),
                          p2(WRFGPU_MUB), dt_rk, p3(WRFGPU_H_DIABATIC), td);
      return 0;
    case ORACLE_R_UPDATE_SCALAR_ARGS:
      rk_update_scalar(D.qold(species), D.q(species), p3(WRFGPU_ADVECT_TEND), p2(WRFGPU_MSFTY), p1(WRFGPU_C1H),
                       p1(WRFGPU_C2H), p2(WRFGPU_MU_1), p2(WRFGPU_MU_2), p2(WRFGPU_MUB), rk_step, dt_rk,
                       p3(WRFGPU_H_DIABATIC), td);
      return 0;
    case ORACLE_R_FORWARD_TERMS:
      if (D.tendf.empty()) return -1;
      D.forward_terms(D.tendf[0].data(), D.tendf[1].data(), D.tendf[2].data(), D.tendf[3].data(), R(D.sc.dt), td);
      return 0;
    case ORACLE_R_ADDTEND_DRY_ARGS:
      if (D.tendf.empty()) return -1;
      rk_addtend_dry_full(p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_RW_TEND), p3(WRFGPU_PH_TEND),
                          p3(WRFGPU_T_TEND), D.tendf[0].data(), D.tendf[1].data(), D.tendf[2].data(),
                          p3(WRFGPU_ADVECT_TEND), D.tendf[3].data(), p3(WRFGPU_U_SAVE), p3(WRFGPU_V_SAVE),
                          p3(WRFGPU_W_SAVE), p3(WRFGPU_PH_SAVE), p3(WRFGPU_T_SAVE), p2(WRFGPU_MU_TEND),
                          p2(WRFGPU_MUDF), rk_step, p1(WRFGPU_C1H), p1(WRFGPU_C2H), p3(WRFGPU_H_DIABATIC),
                          p2(WRFGPU_MUT), p2(WRFGPU_MSFTY), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
                          p2(WRFGPU_MSFVX_INV), td);
      return 0;
    case ORACLE_R_SIXTH_DIFF_SPECIES:
      // rk_scalar_tend's stage-1 diffusion of species `species` into the
      // H_DIABATIC buffer (module_em.F:1378-1435): explicit (diff_opt = 1,
      // its class's mix2_off off; iteration 1: qv against qv_base), then
      // sixth-order (diff_6th_opt != 0, its class's mix6_off off)
      if (cf.diff_opt == 1 && !(species < D.n_moist ? cf.moist_mix2_off : cf.scalar_mix2_off)) {
        const R prandtl = R(1.) / R(3.0);
        horizontal_diffusion(D.cf, 'm', D.q(species), p3(WRFGPU_H_DIABATIC), p2(WRFGPU_MUTS), p1(WRFGPU_C1H),
                             p1(WRFGPU_C2H), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
                             p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY),
                             (R)cf.khdif / prandtl, rdx, rdy, td);
        vertical_diffusion(D.cf, iteration == 1 ? 'p' : 'm', D.q(species), p3(WRFGPU_H_DIABATIC), p1(WRFGPU_QV_BASE),
                           (R*)nullptr, p1(WRFGPU_C1H), p1(WRFGPU_C2H), p3(WRFGPU_ALT), p2(WRFGPU_MUTS),
                           p1(WRFGPU_RDN), p1(WRFGPU_RDNW), (R)cf.kvdif / prandtl, td);
      }
      if (cf.diff_6th_opt != 0 && !(species < D.n_moist ? cf.moist_mix6_off : cf.scalar_mix6_off))
        sixth_order_diffusion('m', D.q(species), p3(WRFGPU_H_DIABATIC), p2(WRFGPU_MUTS), dt_rk, cf, p1(WRFGPU_C1H),
                              p1(WRFGPU_C2H), p3(WRFGPU_PHB), rdx, rdy, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY),
                              p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), td);
      return 0;
    case ORACLE_R_ADVECT_SCALAR:
      zero_tend(p3(WRFGPU_ADVECT_TEND), td);
      advect_scalar(D.q(species), D.q(species), p3(WRFGPU_ADVECT_TEND), p3(WRFGPU_RU_M), p3(WRFGPU_RV_M),
                    p3(WRFGPU_WW_M), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUTS), cf, p2(WRFGPU_MSFUX),
                    p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY),
                    p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW), td);
      return 0;
    case ORACLE_R_ADVECT_SCALAR_PD:
      zero_tend(p3(WRFGPU_ADVECT_TEND), td);
      advect_scalar_pd(D.q(species), D.qold(species), p3(WRFGPU_ADVECT_TEND), p3(WRFGPU_RU_M), p3(WRFGPU_RV_M),
                       p3(WRFGPU_WW_M), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUTS), p2(WRFGPU_MUB),
                       p2(WRFGPU_MU_1), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY),
                       p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW),
                       dt_rk, td);
      return 0;
    case ORACLE_R_UPDATE_SCALAR:
      rk_update_scalar(D.qold(species), D.q(species), p3(WRFGPU_ADVECT_TEND), p2(WRFGPU_MSFTY), p1(WRFGPU_C1H),
                       p1(WRFGPU_C2H), p2(WRFGPU_MU_1), p2(WRFGPU_MU_2), p2(WRFGPU_MUB), rk_step, dt_rk,
                       (R*)nullptr, td);
      return 0;
    case ORACLE_R_CALC_P_RHO_PHI:
      calc_p_rho_phi(D.q(0), D.n_moist, cf.hypsometric_opt, p3(WRFGPU_AL), p3(WRFGPU_ALB), p2(WRFGPU_MU_2),
                     p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C3H), p1(WRFGPU_C4H), p1(WRFGPU_C3F),
                     p1(WRFGPU_C4F), p3(WRFGPU_PH_2), p3(WRFGPU_PHB), p3(WRFGPU_P), p3(WRFGPU_PB), p3(WRFGPU_T_2), KR::p0,
                     KR::t0, p_top, p1(WRFGPU_ZNU), p1(WRFGPU_ZNW), p1(WRFGPU_DNW), p1(WRFGPU_RDNW), p1(WRFGPU_RDN),
                     cf.non_hydrostatic, cf.use_theta_m, td);
      return 0;
    case ORACLE_R_SET_W_SURFACE:
      set_w_surface(cf, p3(WRFGPU_W_2), p2(WRFGPU_HT), p3(WRFGPU_U_2), p3(WRFGPU_V_2), cf1, cf2, cf3, rdx, rdy,
                    p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), td);
      return 0;
    case ORACLE_R_RK_TENDENCY:
      for (int r : {ORACLE_R_ZERO_TEND, ORACLE_R_ADVECT_U, ORACLE_R_ADVECT_V, ORACLE_R_ADVECT_W, ORACLE_R_ADVECT_T,
                    ORACLE_R_RHS_PH, ORACLE_R_HPG, ORACLE_R_PG_BUOY_W, ORACLE_R_CORIOLIS, ORACLE_R_CURVATURE}) {
        int rc = run_routine(D, r, rk_step, iteration, species);
        if (rc) return rc;
      }
      return 0;
    default:
      return WRFGPU_E_ARG;
  }
}
}  // namespace

#define ORACLE_API(PFX, R)                                                                              \
  extern "C" int PFX##domain_create(const WrfGpuDomainDesc* desc, int nthreads, void** out) {           \
    try {                                                                                               \
      auto* D = new Domain<R>();                                                                        \
      D->init(*desc);                                                                                   \
      D->nthreads = nthreads > 0 ? nthreads : 1;                                                        \
      *out = D;                                                                                         \
      return 0;                                                                                         \
    } catch (const std::exception& e) {                                                                 \
      std::fprintf(stderr, "oracle: %s\n", e.what());                                                   \
      return WRFGPU_E_ARG;                                                                              \
    }                                                                                                   \
  }                                                                                                     \
  extern "C" int PFX##domain_destroy(void* h) { delete (Domain<R>*)h; return 0; }                      \
  extern "C" long PFX##field_size(void* h, int id) {                                                    \
    long n = 0; ((Domain<R>*)h)->field(id, &n); return n;                                               \
  }                                                                                                     \
  extern "C" int PFX##set_field(void* h, int id, const double* src, long n) {                          \
    long m = 0; R* p = ((Domain<R>*)h)->field(id, &m);                                                  \
    if (!p || m != n) return WRFGPU_E_ARG;                                                              \
    for (long i = 0; i < n; ++i) p[i] = (R)src[i];                                                      \
    return 0;                                                                                           \
  }                                                                                                     \
  extern "C" int PFX##set_field_f32(void* h, int id, const float* src, long n) {                       \
    long m = 0; R* p = ((Domain<R>*)h)->field(id, &m);                                                  \
    if (!p || m != n) return WRFGPU_E_ARG;                                                              \
    for (long i = 0; i < n; ++i) p[i] = (R)src[i];                                                      \
    return 0;                                                                                           \
  }                                                                                                     \
  extern "C" int PFX##get_field(void* h, int id, double* dst, long n) {                                \
    long m = 0; R* p = ((Domain<R>*)h)->field(id, &m);                                                  \
    if (!p || m != n) return WRFGPU_E_ARG;                                                              \
    for (long i = 0; i < n; ++i) dst[i] = (double)p[i];                                                 \
    return 0;                                                                                           \
  }                                                                                                     \
  extern "C" int PFX##step(void* h, int nsteps) {                                                       \
    try {                                                                                               \
      for (int s = 0; s < nsteps; ++s) ((Domain<R>*)h)->solve_em_step();                                \
      return 0;                                                                                         \
    } catch (const std::exception& e) {                                                                 \
      std::fprintf(stderr, "oracle: %s\n", e.what());                                                   \
      return WRFGPU_E_ARG;                                                                              \
    }                                                                                                   \
  }                                                                                                     \
  extern "C" int PFX##run_routine(void* h, int routine, int rk_step, int iteration, int species) {      \
    try {                                                                                               \
      return run_routine(*(Domain<R>*)h, routine, rk_step, iteration, species);                         \
    } catch (const std::exception& e) {                                                                 \
      std::fprintf(stderr, "oracle: %s\n", e.what());                                                   \
      return WRFGPU_E_ARG;                                                                              \
    }                                                                                                   \
  }                                                                                                     \
  extern "C" int PFX##fill_halo(void* h, int id, char var) {                                            \
    Domain<R>* D = (Domain<R>*)h;                                                                       \
    long n = 0; R* p = D->field(id, &n);                                                                \
    if (!p) return WRFGPU_E_ARG;                                                                        \
    if (n == D->n3) set_physical_bc3d(p, var, D->cf, D->d);                                             \
    else if (n == D->n2) set_physical_bc2d(p, var, D->cf, D->d);                                        \
    else return WRFGPU_E_ARG;                                                                           \
    return 0;                                                                                           \
  }                                                                                                     \
  extern "C" int PFX##num_sound_steps(void* h) { return ((Domain<R>*)h)->num_sound_steps(); }          \
  extern "C" int PFX##cfl(void* h, double* vert, double* horiz) {                                       \
    *vert = (double)((Domain<R>*)h)->max_vert_cfl; *horiz = (double)((Domain<R>*)h)->max_horiz_cfl;     \
    return 0;                                                                                           \
  }

ORACLE_API(oracle_f32_, float)
ORACLE_API(oracle_f64_, double)

// The reference's standalone advection fixture (module_advect_em.F:3-115,
// :10564-10871, "PROGRAM feeder"): a top-hat (1 for 35 < i < 55) on a
// 91 x 3 x 10 grid with ru = 90, rdx = 1/1000, dt = 5, advanced by RK3 loops
// with advect_scalar in the first two stages and advect_scalar (adv_opt 0)
// or advect_scalar_pd (adv_opt 1) in the third, and the feeder's own
// periodic copy (period 90) after every loop.  Writes the row field(:,1,2)
// every `every` loops into out[(loop/every) * 91 + i-1], starting with loop 0.
namespace {
template <typename R>
int feeder(int adv_opt, int nloops, int every, double* out) {
  Dims d{};
  d.ids = 1; d.ide = 91; d.jds = 1; d.jde = 3; d.kds = 1; d.kde = 10;
  d.ims = -5; d.ime = 96; d.jms = -5; d.jme = 8; d.kms = 1; d.kme = 10;
  d.its = 1; d.ite = 91; d.jts = 1; d.jte = 3; d.kts = 1; d.kte = 10;
  WrfDynConfig cf{};
  cf.h_sca_adv_order = 5; cf.v_sca_adv_order = 3; cf.periodic_x = 1; cf.periodic_y = 1;
  const long n3 = (long)(d.ime - d.ims + 1) * (d.kme - d.kms + 1) * (d.jme - d.jms + 1);
  const long n2 = (long)(d.ime - d.ims + 1) * (d.jme - d.jms + 1);
  std::vector<R> field(n3, 0), field_old(n3, 0), ru(n3, R(90)), rv(n3, 0), rom(n3, 0), tend(n3, 0);
  std::vector<R> mut(n2, 1), mub(n2, 1), mu_old(n2, 0), msf(n2, 1);
  std::vector<R> znw(10), rdzw(10), dnw(10), rdnw(10), dn(10), rdn(10), fzp(10), fzm(10), c1(10, 1), c2(10, 0);
  A3<R> F(field.data(), d), FO(field_old.data(), d);
  for (int j = d.jts; j <= d.jte; ++j)
    for (int k = d.kts; k <= d.kte; ++k)
      for (int i = d.its; i <= d.ite; ++i)
        if (i > 35 && i < 55) { F(i, k, j) = R(1.); FO(i, k, j) = R(1.); }
  for (int k = d.kts; k <= d.kte; ++k) znw[k - 1] = R(1) - (R(k) - R(d.kts)) / (R(d.kte) - R(d.kts));
  for (int k = d.kts; k <= d.kte - 1; ++k) rdzw[k - 1] = R(1.) / (znw[k - 1] - znw[k]);
  for (int k = 1; k <= d.kde - 1; ++k) { dnw[k - 1] = znw[k] - znw[k - 1]; rdnw[k - 1] = R(1.) / dnw[k - 1]; }
  for (int k = 2; k <= d.kde - 1; ++k) {
    dn[k - 1] = R(0.5) * (dnw[k - 1] + dnw[k - 2]); rdn[k - 1] = R(1.) / dn[k - 1];
    fzp[k - 1] = R(.5) * dnw[k - 1] / dn[k - 1]; fzm[k - 1] = R(.5) * dnw[k - 2] / dn[k - 1];
  }
  const R rdx = R(1) / R(1000.), rdy = R(1) / R(1000.), dt = R(5);
  auto save = [&](int loop) {
    int slot = loop / every;
    for (int i = d.its; i <= d.ite; ++i) out[(long)slot * 91 + (i - 1)] = (double)F(i, 1, 2);
  };
  save(0);
  auto adv = [&]() {
    std::fill(tend.begin(), tend.end(), R(0));
    advect_scalar(field.data(), field_old.data(), tend.data(), ru.data(), rv.data(), rom.data(), c1.data(), c2.data(),
                  mut.data(), cf, msf.data(), msf.data(), msf.data(), msf.data(), msf.data(), msf.data(), fzm.data(),
                  fzp.data(), rdx, rdy, rdzw.data(), d);
  };
  for (int loop = 1; loop <= nloops; ++loop) {
    adv();
    for (long q = 0; q < n3; ++q) field[q] = field_old[q] + dt * tend[q] / R(3.);
    adv();
    for (long q = 0; q < n3; ++q) field[q] = field_old[q] + dt * tend[q] / R(2.);
    std::fill(tend.begin(), tend.end(), R(0));
    if (adv_opt == 1)
      advect_scalar_pd(field.data(), field_old.data(), tend.data(), ru.data(), rv.data(), rom.data(), c1.data(),
                       c2.data(), mut.data(), mub.data(), mu_old.data(), cf, msf.data(), msf.data(), msf.data(),
                       msf.data(), msf.data(), msf.data(), fzm.data(), fzp.data(), rdx, rdy, rdzw.data(), dt, d);
    else
      advect_scalar(field.data(), field_old.data(), tend.data(), ru.data(), rv.data(), rom.data(), c1.data(),
                    c2.data(), mut.data(), cf, msf.data(), msf.data(), msf.data(), msf.data(), msf.data(), msf.data(),
                    fzm.data(), fzp.data(), rdx, rdy, rdzw.data(), d);
    for (long q = 0; q < n3; ++q) field[q] = field_old[q] + dt * (tend[q]);
    for (int j = d.jms; j <= d.jme; ++j)
      for (int k = 1; k <= d.kde; ++k)
        for (int i = d.ims; i <= d.ime; ++i) F(i, k, j) = F(i, 2, j);
    for (int k = d.kms; k <= d.kme; ++k)
      for (int i = d.ims; i <= d.ime; ++i) { F(i, k, 2) = F(i, k, 1); F(i, k, 3) = F(i, k, 1); }
    for (int q = 0; q <= 4; ++q)
      for (int j = d.jms; j <= d.jme; ++j)
        for (int k = d.kms; k <= d.kme; ++k) F(d.ite + q, k, j) = F(d.ids + q, k, j);
    for (int q = 0; q <= 4; ++q)
      for (int j = d.jms; j <= d.jme; ++j)
        for (int k = d.kms; k <= d.kme; ++k) F(d.ids - q, k, j) = F(d.ite - q, k, j);
    field_old = field;
    if (loop % every == 0) save(loop);
  }
  return 0;
}
}  // namespace

extern "C" int oracle_f32_tophat_feeder(int adv_opt, int nloops, int every, double* out) {
  return feeder<float>(adv_opt, nloops, every, out);
}
extern "C" int oracle_f64_tophat_feeder(int adv_opt, int nloops, int every, double* out) {
  return feeder<double>(adv_opt, nloops, every, out);
}
