/* ORACLE — test infrastructure only.  Routine ids for the oracle's routine
 * runner; the GPU library's wrfgpu_run_routine accepts the same ids
 * (WRFGPU_R_* in include/wrfgpu.h carry the same values). */
#ifndef ORACLE_ROUTINES_H
#define ORACLE_ROUTINES_H
enum {
  ORACLE_R_RK_STEP_PREP = 1,
  ORACLE_R_ZERO_TEND = 2,
  ORACLE_R_ADVECT_U = 3,
  ORACLE_R_ADVECT_V = 4,
  ORACLE_R_ADVECT_W = 5,
  ORACLE_R_ADVECT_T = 6,
  ORACLE_R_RHS_PH = 7,
  ORACLE_R_HPG = 8,
  ORACLE_R_PG_BUOY_W = 9,
  ORACLE_R_CORIOLIS = 10,
  ORACLE_R_CURVATURE = 11,
  ORACLE_R_SMALL_STEP_PREP = 12,
  ORACLE_R_CALC_P_RHO = 13,
  ORACLE_R_CALC_COEF_W = 14,
  ORACLE_R_ADVANCE_UV = 15,
  ORACLE_R_ADVANCE_MU_T = 16,
  ORACLE_R_ADVANCE_W = 17,
  ORACLE_R_SUMFLUX = 18,
  ORACLE_R_SMALL_STEP_FINISH = 19,
  ORACLE_R_UPDATE_SCALAR_PD = 20,
  ORACLE_R_ADVECT_SCALAR = 21,
  ORACLE_R_ADVECT_SCALAR_PD = 22,
  ORACLE_R_UPDATE_SCALAR = 23,
  ORACLE_R_CALC_P_RHO_PHI = 24,
  ORACLE_R_SET_W_SURFACE = 25,
  ORACLE_R_RK_TENDENCY = 26,
  /* the routine-level C entry points' forms: sc_tend (and rk_scalar_tend's
   * scalar_tends) carried in the H_DIABATIC field, mu_new in MU_2 */
  ORACLE_R_UPDATE_SCALAR_PD_ARGS = 30,
  ORACLE_R_UPDATE_SCALAR_ARGS = 31,
  ORACLE_R_SIXTH_DIFF_SPECIES = 32,
  /* rk_tendency's stage-1 forward terms added to the *_tendf fields
   * (WRFGPU_RU_TENDF ..), with the large step dt */
  ORACLE_R_FORWARD_TERMS = 33,
  /* rk_addtend_dry, every term: ph_tendf carried in ADVECT_TEND, mu_tendf in MUDF */
  ORACLE_R_ADDTEND_DRY_ARGS = 34
};
#endif
