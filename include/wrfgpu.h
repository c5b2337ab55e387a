/*
 * wrfgpu.h — C ABI of the GB300 WRF-ARW dynamical-core large step.
 *
 * Two layers of entry points replace the reference's model-layer calls:
 *
 *  1. Per-subroutine entry points, one per Fortran subroutine on the
 *     physics-off solve_em path, with the reference's argument order and
 *     meaning.  Arrays are host pointers to element (ims,kms,jms) of a
 *     Fortran (ims:ime, kms:kme, jms:jme) array (i fastest); 2-D arrays are
 *     (ims:ime, jms:jme), 1-D column arrays (kms:kme).  Scalars and index
 *     bounds are passed by pointer (Fortran pass-by-reference), logicals as
 *     int32.  config_flags becomes the flat POD WrfDynConfig.  These copy
 *     host<->device around one kernel launch (parity mode).
 *
 *  2. A coarse, device-resident domain API (create / set_field / step /
 *     get_field / destroy) and an ensemble API that advances many uneven
 *     domains per launch.  The large step runs entirely on the GPU; the
 *     host only enqueues the captured CUDA graph.
 *
 * Every entry point returns 0 on success or a negative WRFGPU_E* code; the
 * reference aborts through wrf_error_fatal (frame/module_wrf_error.F:316)
 * instead, which a Fortran shim reproduces by calling it on non-zero.
 * No entry point traps on the device.
 */
#ifndef WRFGPU_H
#define WRFGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Memory halo width of every array (the serial build's bdyzone = 4,
 * share/module_bc.F:33; frame/module_domain.F:331-517 sets ims = ids-4). */
#define WRFGPU_HALO 4

/* Error codes. */
#define WRFGPU_OK 0
#define WRFGPU_E_ARG -1         /* bad argument / unsupported option        */
#define WRFGPU_E_CUDA -2        /* CUDA runtime error                        */
#define WRFGPU_E_NONFINITE -3   /* non-finite value detected in the state    */
#define WRFGPU_E_CFL -4         /* vertical CFL above the configured limit   */
#define WRFGPU_E_TIMEOUT -5     /* bounded device wait gave up               */
#define WRFGPU_E_NOMEM -6       /* device allocation failed                  */
#define WRFGPU_E_SIZE -7        /* request larger than a fixed capacity      */

/* grid_config_rec_type subset read by the path (Registry/Registry.EM_COMMON:
 * 2840-2938, 2285).  Logicals are int32 0/1. */
typedef struct WrfDynConfig {
  int32_t periodic_x, periodic_y;
  int32_t symmetric_xs, symmetric_xe, symmetric_ys, symmetric_ye;
  int32_t open_xs, open_xe, open_ys, open_ye;
  int32_t specified, nested, polar;
  int32_t rk_ord;
  int32_t h_mom_adv_order, v_mom_adv_order, h_sca_adv_order, v_sca_adv_order;
  int32_t moist_adv_opt, scalar_adv_opt; /* 0 ORIGINAL, 1 POSITIVEDEF */
  int32_t non_hydrostatic, top_lid, use_theta_m, hypsometric_opt, phi_adv_z;
  int32_t w_damping, damp_opt, diff_opt, zadvect_implicit, map_proj;
  int32_t time_step_sound;
  float w_crit_cfl;       /* namelist w_crit_cfl (Registry default 1.0); enters the w_damping = 1 term */
  float dampcoef, zdamp;  /* namelist dampcoef, zdamp (Registry defaults 0.2, 5000 m): damp_opt = 3 */
  /* sixth-order numerical diffusion (Registry.EM_COMMON:2860-2863): diff_6th_opt
   * 0 off, 1 on, 2 on with up-gradient fluxes dropped; diff_6th_slopeopt 1 tapers
   * it over steep terrain (threshold diff_6th_thresh, Registry default 0.10);
   * diff_6th_factor (Registry default 0.12); moist_mix6_off / scalar_mix6_off 1
   * leave the moist / passive species undiffused. */
  int32_t diff_6th_opt, diff_6th_slopeopt;
  float diff_6th_factor, diff_6th_thresh;
  int32_t moist_mix6_off, scalar_mix6_off;
  /* explicit diffusion (diff_opt = 1) with constant coefficients (km_opt = 1):
   * khdif, kvdif in m2/s (Registry defaults 0); moist_mix2_off / scalar_mix2_off
   * 1 leave the moist / passive species undiffused. */
  int32_t km_opt, moist_mix2_off, scalar_mix2_off, pad_cfg;
  float khdif, kvdif;
} WrfDynConfig;

/* Domain scalars that solve_em reads from grid% (double on the ABI; each
 * build rounds them to its working precision). */
typedef struct WrfGpuScalars {
  double dt, dx, dy, rdx, rdy;
  double cf1, cf2, cf3, cfn, cfn1;
  double epssm, smdiv, emdiv;
  double p_top;
} WrfGpuScalars;

/* Domain description: ids=jds=kds=1; ide, jde are the staggered ends
 * (e_we, e_sn), kde = e_vert. */
typedef struct WrfGpuDomainDesc {
  int32_t ide, jde, kde;
  int32_t n_moist;  /* moist species carried (qv only on this path: 1) */
  int32_t n_scalar; /* passive scalars                                  */
  int32_t pad0;
  WrfDynConfig config;
  WrfGpuScalars scalars;
} WrfGpuDomainDesc;

/* Field table of the domain state (ids for set_field / get_field). */
enum WrfGpuFieldId {
  /* 3-D (ims:ime, kms:kme, jms:jme) */
  WRFGPU_U_1 = 0, WRFGPU_U_2, WRFGPU_V_1, WRFGPU_V_2, WRFGPU_W_1, WRFGPU_W_2,
  WRFGPU_T_1, WRFGPU_T_2, WRFGPU_PH_1, WRFGPU_PH_2,
  WRFGPU_PHB, WRFGPU_PB, WRFGPU_ALB, WRFGPU_P, WRFGPU_AL, WRFGPU_ALT, WRFGPU_PHP,
  WRFGPU_RU, WRFGPU_RV, WRFGPU_RW, WRFGPU_WW, WRFGPU_WW1,
  WRFGPU_CQU, WRFGPU_CQV, WRFGPU_CQW,
  WRFGPU_RU_TEND, WRFGPU_RV_TEND, WRFGPU_RW_TEND, WRFGPU_T_TEND, WRFGPU_PH_TEND,
  WRFGPU_U_SAVE, WRFGPU_V_SAVE, WRFGPU_W_SAVE, WRFGPU_T_SAVE, WRFGPU_PH_SAVE,
  WRFGPU_C2A, WRFGPU_PM1, WRFGPU_A, WRFGPU_ALPHA, WRFGPU_GAMMA, WRFGPU_T_2SAVE,
  WRFGPU_RU_M, WRFGPU_RV_M, WRFGPU_WW_M, WRFGPU_ADVECT_TEND, WRFGPU_H_DIABATIC,
  WRFGPU_T_INIT,  /* base-state theta perturbation (module_initialize_ideal.F:973): explicit diffusion of theta */
  WRFGPU_N3D,
  /* rk_tendency's stored forward tendencies ru_tendf, rv_tendf, rw_tendf,
   * t_tendf (3-D): present only in members that use diff_opt = 1,
   * diff_6th_opt != 0 or damp_opt = 2 */
  WRFGPU_TENDF_BASE = 90,
  WRFGPU_RU_TENDF = WRFGPU_TENDF_BASE, WRFGPU_RV_TENDF, WRFGPU_RW_TENDF, WRFGPU_T_TENDF,
  /* 2-D (ims:ime, jms:jme) */
  WRFGPU_F2D_BASE = 100,
  WRFGPU_MU_1 = WRFGPU_F2D_BASE, WRFGPU_MU_2, WRFGPU_MUB, WRFGPU_MUT, WRFGPU_MUU, WRFGPU_MUV,
  WRFGPU_MUTS, WRFGPU_MUUS, WRFGPU_MUVS, WRFGPU_MUDF, WRFGPU_MU_SAVE, WRFGPU_MUAVE, WRFGPU_MU_TEND,
  WRFGPU_MSFUX, WRFGPU_MSFUY, WRFGPU_MSFVX, WRFGPU_MSFVX_INV, WRFGPU_MSFVY, WRFGPU_MSFTX, WRFGPU_MSFTY,
  WRFGPU_HT, WRFGPU_F, WRFGPU_E, WRFGPU_SINA, WRFGPU_COSA,
  WRFGPU_F2D_END,
  /* 1-D (kms:kme) */
  WRFGPU_F1D_BASE = 200,
  WRFGPU_ZNW = WRFGPU_F1D_BASE, WRFGPU_ZNU, WRFGPU_DNW, WRFGPU_RDNW, WRFGPU_DN, WRFGPU_RDN,
  WRFGPU_FNM, WRFGPU_FNP, WRFGPU_C1H, WRFGPU_C2H, WRFGPU_C1F, WRFGPU_C2F,
  WRFGPU_C3H, WRFGPU_C4H, WRFGPU_C3F, WRFGPU_C4F,
  /* base-state profiles of the initial column (1,1) (module_initialize_ideal.F:1578-1586),
   * read by the Rayleigh damping toward them (damp_opt = 2) */
  WRFGPU_U_BASE, WRFGPU_V_BASE, WRFGPU_T_BASE, WRFGPU_Z_BASE,
  WRFGPU_QV_BASE,  /* qv of column (1,1): explicit vertical diffusion of qv */
  WRFGPU_F1D_END,
  /* species: WRFGPU_SPECIES_BASE + 2*s is species s (moist first, then
   * passive scalars), + 1 its "old" (_1) copy */
  WRFGPU_SPECIES_BASE = 300
};
#define WRFGPU_N2D (WRFGPU_F2D_END - WRFGPU_F2D_BASE)
#define WRFGPU_N1D (WRFGPU_F1D_END - WRFGPU_F1D_BASE)

/* ------------------------------------------------------------------------
 * Coarse device-resident API.  A domain is an ensemble of one member; all
 * calls take the ensemble handle and a member index where relevant.
 * ---------------------------------------------------------------------- */
typedef struct WrfGpuEnsemble WrfGpuEnsemble;

/* creation flags */
#define WRFGPU_FLAG_MIXED 1      /* FP64 column sums, omega recursion and tridiagonal solve */
#define WRFGPU_FLAG_NO_GRAPH 2   /* enqueue kernels directly instead of replaying a CUDA graph */
#define WRFGPU_FLAG_NO_CHECKS 4  /* skip the per-stage CFL / non-finite health check */

/* Create n members (uneven sizes allowed) advanced together.  Replaces the
 * reference's domain allocation for the dynamics state (frame/module_domain.F
 * alloc_and_configure_domain) on the device side.  Lateral boundaries, one
 * condition per side (share/module_bc.F:60-133): x periodic or open on both
 * sides, y periodic, symmetric or open on both sides; open sides at least 12
 * points apart.  Anything else (specified, nested, polar, symmetric x)
 * returns WRFGPU_E_ARG. */
int wrfgpu_ensemble_create(const WrfGpuDomainDesc* descs, int n, int flags, WrfGpuEnsemble** out);
int wrfgpu_ensemble_destroy(WrfGpuEnsemble* h);
/* Element count of a field of one member (memory dims, halo included). */
long long wrfgpu_field_size(WrfGpuEnsemble* h, int member, int id);
/* Host <-> device copies of one field (Fortran memory layout). */
int wrfgpu_set_field_f32(WrfGpuEnsemble* h, int member, int id, const float* src, long long n);
int wrfgpu_get_field_f32(WrfGpuEnsemble* h, int member, int id, float* dst, long long n);
int wrfgpu_set_field(WrfGpuEnsemble* h, int member, int id, const double* src, long long n);
int wrfgpu_get_field(WrfGpuEnsemble* h, int member, int id, double* dst, long long n);
/* Advance every member by nsteps large steps: the replacement of the RK3 loop
 * of dyn_em/solve_em.F:578-3459 plus its end-of-step fills (:4439-4750).
 * Asynchronous: returns once the work is enqueued. */
int wrfgpu_step(WrfGpuEnsemble* h, int nsteps);
int wrfgpu_sync(WrfGpuEnsemble* h);
/* Host state bound to the step (the coarse upload / step / download of a host
 * time loop): for field ids[f] of `member`, in[f] (n[f] values, Fortran memory
 * layout) is copied in before every step of wrfgpu_step_host and the field is
 * copied out to out[f] after it; in or out (or one entry of either) may be
 * null, and in[f] may equal out[f].  Buffers must be page-locked
 * (cudaHostAlloc / cudaHostRegister) and stay valid while bound; binding a
 * field again replaces its buffers.  WRFGPU_E_ARG for an unknown field, a
 * wrong count or pageable memory. */
int wrfgpu_bind_host_state(WrfGpuEnsemble* h, int member, int nfield, const int* ids, const float* const* in,
                           float* const* out, const long long* n);
int wrfgpu_unbind_host_state(WrfGpuEnsemble* h);
/* nsteps times: the bound inputs copied in, one large step, the bound outputs
 * copied out, each step's inputs read after the previous step's outputs are
 * written (so in[f] == out[f] runs a host time loop); returns when the last
 * copy is complete.  The copies overlap the kernels: the passive scalars'
 * uploads run during stage 1's dynamics, the dry state's downloads during
 * the last stage's scalar transport (followed there, within one call, by
 * the next step's dry uploads when no later download can change their host
 * arrays), and the passive scalars' downloads during the next step of the
 * same call.  The results equal those of
 * wrfgpu_set_field_f32 of every input, wrfgpu_step and wrfgpu_get_field_f32
 * of every output, step by step, bit for bit. */
int wrfgpu_step_host(WrfGpuEnsemble* h, int nsteps);
/* Advance nsteps and return the device time in milliseconds (CUDA events on
 * the ensemble's stream). */
int wrfgpu_time_steps(WrfGpuEnsemble* h, int nsteps, float* ms);
/* Routine ids of wrfgpu_run_routine: one per model-layer call of the
 * physics-off solve_em path (the file:line each follows is in the kernel
 * sources).  WRFGPU_R_RK_TENDENCY runs the whole of rk_tendency
 * (dyn_em/module_em.F:370-781) as the fused solver does. */
enum WrfGpuRoutine {
  WRFGPU_R_RK_STEP_PREP = 1, WRFGPU_R_ZERO_TEND, WRFGPU_R_ADVECT_U, WRFGPU_R_ADVECT_V, WRFGPU_R_ADVECT_W,
  WRFGPU_R_ADVECT_T, WRFGPU_R_RHS_PH, WRFGPU_R_HORIZONTAL_PRESSURE_GRADIENT, WRFGPU_R_PG_BUOY_W,
  WRFGPU_R_CORIOLIS, WRFGPU_R_CURVATURE, WRFGPU_R_SMALL_STEP_PREP, WRFGPU_R_CALC_P_RHO, WRFGPU_R_CALC_COEF_W,
  WRFGPU_R_ADVANCE_UV, WRFGPU_R_ADVANCE_MU_T, WRFGPU_R_ADVANCE_W, WRFGPU_R_SUMFLUX, WRFGPU_R_SMALL_STEP_FINISH,
  WRFGPU_R_RK_UPDATE_SCALAR_PD, WRFGPU_R_ADVECT_SCALAR, WRFGPU_R_ADVECT_SCALAR_PD, WRFGPU_R_RK_UPDATE_SCALAR,
  WRFGPU_R_CALC_P_RHO_PHI, WRFGPU_R_SET_W_SURFACE, WRFGPU_R_RK_TENDENCY
};
/* Run one model-layer routine on the resident state (kernel-level parity).
 * rk_step 1..3; iteration = acoustic step (1-based) for the acoustic
 * routines (0 = before the first, for calc_p_rho); species for the scalar
 * routines. */
int wrfgpu_run_routine(WrfGpuEnsemble* h, int routine, int rk_step, int iteration, int species);
/* set_physical_bc3d / set_physical_bc2d of one field of every member. */
int wrfgpu_fill_halo(WrfGpuEnsemble* h, int id, char var);
/* Health: error bits since the last clear, max vertical / horizontal CFL
 * (w_damp diagnostics, dyn_em/module_big_step_utilities_em.F:2503-2712).
 * Returns WRFGPU_E_NONFINITE / WRFGPU_E_CFL when the bits are set. */
int wrfgpu_status(WrfGpuEnsemble* h, int member, unsigned* err_bits, double* max_vert_cfl, double* max_horiz_cfl);
int wrfgpu_clear_status(WrfGpuEnsemble* h);
/* Self-test of the bounded device wait every TMA-ring kernel uses (no
 * counterpart in the reference, whose loops have no device waits): one
 * block waits on an mbarrier phase for at most `polls` polls (1 .. 2^22).
 * With arrive != 0 the phase is completed first and the call returns 0;
 * with arrive = 0 nothing completes it, the wait gives up, the block records
 * the timeout bit in *status_bits and the call returns WRFGPU_E_TIMEOUT —
 * the device context stays usable. */
int wrfgpu_selftest_bounded_wait(int polls, int arrive, unsigned* status_bits);
int wrfgpu_set_cfl_limit(WrfGpuEnsemble* h, double limit);
int wrfgpu_num_sound_steps(WrfGpuEnsemble* h, int member);
long long wrfgpu_device_bytes(WrfGpuEnsemble* h);
int wrfgpu_kernel_launches_per_step(WrfGpuEnsemble* h);
/* Per-phase device time of nsteps steps enqueued directly with CUDA events
 * between kernel launches (the reference's BENCH_START/BENCH_END timers,
 * inc/bench_solve_em_def.h).  Returns the number of phases filled. */
int wrfgpu_profile_phases(WrfGpuEnsemble* h, int nsteps, double* ms_out, int* launches_out, int nphase);

/* No counterpart in the reference (its tiling is fixed by the namelist).
 * Online autotuning of the launch configuration: runs rounds x 4 real large
 * steps (the model advances), trying for each of the 14 tuned kernel
 * families its launch variants — blocks per SM of the column and
 * scalar-transport kernels, level chunks of the split column kernels — and
 * keeps the fastest per family for the captured step.  Every variant
 * computes the same bits.  Family order: scalar_pd_update,
 * scalar_adv_update, advance_w, advance_uv, sumflux_calc_p_rho, step_prep,
 * small_step_finish, small_step_prep, cfl_check, rk_tend_w, rk_tend_u,
 * rk_tend_v, calc_p_rho_phi, advance_mu_t. */
#define WRFGPU_NTUNE 14
int wrfgpu_autotune(WrfGpuEnsemble* h, int rounds);
/* The chosen variant of each family, the parameter it stands for (blocks per
 * SM, level chunks, or 10 x blocks per SM + level chunks for advance_uv,
 * sumflux_calc_p_rho, rk_tend_u and rk_tend_v), and the measured ms per step of every variant
 * (ms[f * 4 + v], -1 when not timed).  Returns WRFGPU_NTUNE. */
int wrfgpu_tuning(WrfGpuEnsemble* h, int* variant, int* param, float* ms, int nfamily);
const char* wrfgpu_phase_name(int phase);
const char* wrfgpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* WRFGPU_H */
