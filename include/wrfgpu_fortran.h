/*
 * wrfgpu_fortran.h — per-subroutine drop-in entry points.
 *
 * One entry point per model-layer routine of the physics-off solve_em path,
 * with the reference's Fortran argument order and meaning, so that a Fortran
 * shim can bind each with an ISO_C_BINDING interface (an INTERFACE block of
 * BIND(C) declarations with the same dummy arguments) and call it in place
 * of the original:
 *
 *   - every argument is passed by reference (a pointer), as Fortran does
 *     without the VALUE attribute;
 *   - arrays point at element (ims,kms,jms) of a REAL (ims:ime, kms:kme,
 *     jms:jme) array (i fastest), (ims,jms) of a 2-D (ims:ime, jms:jme)
 *     array, or kms of a 1-D (kms:kme) array;
 *   - LOGICAL arguments are 32-bit integers (0 / non-zero);
 *   - TYPE(grid_config_rec_type) config_flags becomes the flat WrfDynConfig
 *     (wrfgpu.h), filled once by the shim;
 *   - scalar arguments the physics-off path does not use are accepted and
 *     ignored (documented per routine).
 *
 * Execution: "parity mode".  Each call copies the routine's input arrays to
 * a device-resident scratch domain of the same dimensions (cached between
 * calls), runs the routine's kernel(s) and copies its output arrays back.
 * It is meant for routine-by-routine verification inside an unmodified
 * solve_em; the fast path is the device-resident domain API of wrfgpu.h.
 *
 * Index conventions accepted: ids = jds = kds = 1 and one patch covering
 * the domain; memory dimensions with a halo of at least 4 in i and j
 * (ims <= ids-4, ime >= ide+4, same in j: the window ids-4 .. ide+4 is used
 * and a wider halo is left as it is) and kms = kds, kme = kde; any tile of
 * the patch (ids <= its <= ite <= ide, same in j, kts = kds, kte = kde: the
 * OpenMP tiles of solve_em's tile loops), for which the routine runs over the
 * patch and only the tile's points of the output arrays are written back
 * (a whole-patch tile writes back the whole window).  Anything else returns
 * WRFGPU_E_ARG; max_vert_cfl / max_horiz_cfl are the patch's maxima.  The
 * options accepted are those of wrfgpu_ensemble_create.  Return: 0 or a
 * negative WRFGPU_E_* code (the reference aborts through wrf_error_fatal
 * instead).
 */
#ifndef WRFGPU_FORTRAN_H
#define WRFGPU_FORTRAN_H
#include "wrfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define WRFGPU_DIMS_ARGS                                                                                   \
  const int *ids, const int *ide, const int *jds, const int *jde, const int *kds, const int *kde,         \
      const int *ims, const int *ime, const int *jms, const int *jme, const int *kms, const int *kme,     \
      const int *its, const int *ite, const int *jts, const int *jte, const int *kts, const int *kte

/* dyn_em/module_em.F:37 rk_step_prep.  moist: (ims:ime,kms:kme,jms:jme,n_moist), qv first. */
int wrfgpu_rk_step_prep(const WrfDynConfig *config_flags, const int *rk_step, const float *u, const float *v,
                        const float *w, const float *t, const float *ph, const float *mu, const float *c1h,
                        const float *c2h, const float *c1f, const float *c2f, const float *moist, float *ru,
                        float *rv, float *rw, float *ww, float *php, float *alt, float *muu, float *muv,
                        const float *mub, float *mut, const float *phb, const float *pb, const float *p,
                        const float *al, const float *alb, float *cqu, float *cqv, float *cqw, const float *msfux,
                        const float *msfuy, const float *msfvx, const float *msfvx_inv, const float *msfvy,
                        const float *msftx, const float *msfty, const float *fnm, const float *fnp, const float *dnw,
                        const float *rdx, const float *rdy, const int *n_moist, WRFGPU_DIMS_ARGS);

/* dyn_em/module_em.F:190 rk_tendency.  The large-step tendencies of the
 * physics-off path (RTHFTEN, h_diabatic, ph_tendf and the *_old arrays are
 * unused; wwE, wwI are ww, IEVA off).  At rk_step 1, when config_flags (or
 * the diff_6th_opt, damp_opt, khdif, kvdif, dampcoef, zdamp arguments, which
 * take precedence as in the reference's call) ask for the explicit diffusion
 * (diff_opt = 1 with km_opt = 1; xkmhd / xkhh, when given, must hold khdif /
 * khdif / prandtl), the sixth-order diffusion or the Rayleigh damping
 * (damp_opt = 2), the forward step (:801-944) adds their tendencies to
 * ru_tendf, rv_tendf, rw_tendf and t_tendf, which arrive holding the physics
 * tendencies (zeros with physics off); rk_addtend_dry is the caller's next
 * call, as in solve_em. */
int wrfgpu_rk_tendency(const WrfDynConfig *config_flags, const int *rk_step, float *ru_tend, float *rv_tend,
                       float *rw_tend, float *ph_tend, float *t_tend, float *ru_tendf, float *rv_tendf,
                       float *rw_tendf, const float *ph_tendf, float *t_tendf, float *mu_tend,
                       float *u_save, float *v_save, float *w_save, float *ph_save, float *t_save, float *mu_save,
                       const float *RTHFTEN, const float *ru, const float *rv, const float *rw, const float *ww,
                       const float *wwE, const float *wwI, const float *u, const float *v, const float *w,
                       const float *t, const float *ph, const float *u_old, const float *v_old, const float *w_old,
                       const float *t_old, const float *ph_old, const float *h_diabatic, const float *phb,
                       const float *t_init, const float *mu_old, const float *mu, const float *mut,
                       const float *muu, const float *muv, const float *mub, const float *c1h, const float *c2h,
                       const float *c1f, const float *c2f, const float *al, const float *ht, const float *alt,
                       const float *p, const float *pb, const float *php, const float *cqu, const float *cqv,
                       float *cqw, const float *u_base, const float *v_base, const float *t_base,
                       const float *qv_base, const float *z_base, const float *msfux, const float *msfuy,
                       const float *msfvx, const float *msfvx_inv, const float *msfvy, const float *msftx,
                       const float *msfty, const float *clat, const float *f, const float *e, const float *sina,
                       const float *cosa, const float *fnm, const float *fnp, const float *rdn, const float *rdnw,
                       const float *dt, const float *rdx, const float *rdy, const float *khdif,
                       const float *kvdif, const float *xkmhd, const float *xkhh, const int *diff_6th_opt,
                       const float *diff_6th_factor, const int *adv_opt, const float *dampcoef,
                       const float *zdamp, const int *damp_opt, const int *rad_nudge, const float *cf1,
                       const float *cf2, const float *cf3, const float *cfn, const float *cfn1, const int *n_moist,
                       const int *non_hydrostatic, const int *top_lid, const float *u_frame, const float *v_frame,
                       WRFGPU_DIMS_ARGS, float *max_vert_cfl, float *max_horiz_cfl);

/* dyn_em/module_advect_em.F:126, :1530, :4364 advect_u / advect_v / advect_w
 * (tendency += -div(flux)); time_step is only used for its sign (forward).
 * fld_old enters only the radiation terms of open boundaries, where the
 * reference's callers (rk_tendency, rk_scalar_tend) pass fld itself: with
 * open boundaries a different fld_old returns WRFGPU_E_ARG. */
#define WRFGPU_ADVECT_MOM_ARGS                                                                             \
  const float *fld, const float *fld_old, float *tendency, const float *ru, const float *rv, const float *rom, \
      const float *c1, const float *c2, const float *mut, const int *time_step, const WrfDynConfig *config_flags, \
      const float *msfux, const float *msfuy, const float *msfvx, const float *msfvy, const float *msftx,       \
      const float *msfty, const float *fzm, const float *fzp, const float *rdx, const float *rdy,               \
      const float *rdzw, WRFGPU_DIMS_ARGS
int wrfgpu_advect_u(WRFGPU_ADVECT_MOM_ARGS);
int wrfgpu_advect_v(WRFGPU_ADVECT_MOM_ARGS);
int wrfgpu_advect_w(WRFGPU_ADVECT_MOM_ARGS);
/* dyn_em/module_advect_em.F:3029 advect_scalar */
int wrfgpu_advect_scalar(WRFGPU_ADVECT_MOM_ARGS);

/* dyn_em/module_advect_em.F:6069 advect_scalar_pd (tenddec = .false.:
 * h_tendency and z_tendency are not written). */
int wrfgpu_advect_scalar_pd(const float *field, const float *field_old, float *tendency, float *h_tendency,
                            float *z_tendency, const float *ru, const float *rv, const float *rom, const float *c1,
                            const float *c2, const float *mut, const float *mub, const float *mu_old,
                            const int *time_step, const WrfDynConfig *config_flags, const int *tenddec,
                            const float *msfux, const float *msfuy, const float *msfvx, const float *msfvy,
                            const float *msftx, const float *msfty, const float *fzm, const float *fzp,
                            const float *rdx, const float *rdy, const float *rdzw, const float *dt,
                            WRFGPU_DIMS_ARGS);

/* No counterpart in the reference: advect_scalar_pd on DEVICE arrays (same
 * layout and meaning as above, unused arguments dropped; tendency
 * accumulates), enqueued on `stream` (a cudaStream_t, NULL = default stream)
 * without allocating device memory.  For callers whose state is already on
 * the GPU and that cannot allocate there.  The limiter-factor scratch is a
 * fixed static device array: the memory shape may hold at most 8 Mi points
 * (WRFGPU_E_SIZE otherwise).  Options a device domain does not accept
 * return WRFGPU_E_ARG.  The first call on a device (or after its context
 * was re-created) does a one-time setup and should come before any stream
 * capture; calls that overlap in time race on the shared scratch.  The
 * kernels have no device-side failure: the return code is the whole status. */
int wrfgpu_advect_scalar_pd_noalloc(const float *field, const float *field_old, float *tendency,
                                    const float *ru, const float *rv, const float *rom, const float *c1,
                                    const float *c2, const float *mut, const float *mub, const float *mu_old,
                                    const WrfDynConfig *config_flags, const float *msftx, const float *msfty,
                                    const float *fzm, const float *fzp, const float *rdx, const float *rdy,
                                    const float *rdzw, const float *dt, WRFGPU_DIMS_ARGS, void *stream);

/* dyn_em/module_small_step_em.F:16 small_step_prep */
int wrfgpu_small_step_prep(float *u_1, float *u_2, float *v_1, float *v_2, float *w_1, float *w_2, float *t_1,
                           float *t_2, float *ph_1, float *ph_2, const float *mub, float *mu_1, float *mu_2,
                           const float *muu, float *muus, const float *muv, float *muvs, const float *mut,
                           float *muts, float *mudf, const float *c1h, const float *c2h, const float *c1f,
                           const float *c2f, const float *c3h, const float *c4h, const float *c3f, const float *c4f,
                           float *u_save, float *v_save, float *w_save, float *t_save, float *ph_save,
                           float *mu_save, const float *ww, float *ww_save, float *c2a, const float *pb,
                           const float *p, const float *alt, const float *msfux, const float *msfuy,
                           const float *msfvx, const float *msfvx_inv, const float *msfvy, const float *msftx,
                           const float *msfty, const float *rdx, const float *rdy, const int *rk_step,
                           WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:438 calc_p_rho (step 0: before the first
 * acoustic step, else the iteration; divergence damping smdiv) */
int wrfgpu_calc_p_rho(float *al, float *p, const float *ph, const float *alt, const float *t_2, const float *t_1,
                      const float *c2a, float *pm1, const float *mu, const float *mut, const float *c1h,
                      const float *c2h, const float *c1f, const float *c2f, const float *c3h, const float *c4h,
                      const float *c3f, const float *c4f, const float *znu, const float *t0, const float *rdnw,
                      const float *dnw, const float *smdiv, const int *non_hydrostatic, const int *step,
                      WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:570 calc_coef_w */
int wrfgpu_calc_coef_w(float *a, float *alpha, float *gamma, const float *mut, const float *c1h, const float *c2h,
                       const float *c1f, const float *c2f, const float *c3h, const float *c4h, const float *c3f,
                       const float *c4f, const float *cqw, const float *rdn, const float *rdnw, const float *c2a,
                       const float *dts, const float *g, const float *epssm, const int *top_lid, WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:654 advance_uv (spec_zone unused: no
 * specified boundaries) */
int wrfgpu_advance_uv(float *u, const float *ru_tend, float *v, const float *rv_tend, const float *p,
                      const float *pb, const float *ph, const float *php, const float *alt, const float *al,
                      const float *mu, const float *muu, const float *cqu, const float *muv, const float *cqv,
                      const float *mudf, const float *c1h, const float *c2h, const float *c1f, const float *c2f,
                      const float *c3h, const float *c4h, const float *c3f, const float *c4f, const float *msfux,
                      const float *msfuy, const float *msfvx, const float *msfvx_inv, const float *msfvy,
                      const float *rdx, const float *rdy, const float *dts, const float *cf1, const float *cf2,
                      const float *cf3, const float *fnm, const float *fnp, const float *emdiv, const float *rdnw,
                      const WrfDynConfig *config_flags, const int *spec_zone, const int *non_hydrostatic,
                      const int *top_lid, WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:969 advance_mu_t (uam, vam, wwam unused) */
int wrfgpu_advance_mu_t(float *ww, float *ww_1, const float *u, const float *u_1, const float *v, const float *v_1,
                        float *mu, const float *mut, float *muave, float *muts, const float *muu, const float *muv,
                        float *mudf, const float *c1h, const float *c2h, const float *c1f, const float *c2f,
                        const float *c3h, const float *c4h, const float *c3f, const float *c4f, const float *uam,
                        const float *vam, const float *wwam, float *t, const float *t_1, float *t_ave,
                        const float *ft, const float *mu_tend, const float *rdx, const float *rdy, const float *dts,
                        const float *epssm, const float *dnw, const float *fnm, const float *fnp, const float *rdnw,
                        const float *msfux, const float *msfuy, const float *msfvx, const float *msfvx_inv,
                        const float *msfvy, const float *msftx, const float *msfty, const int *step,
                        const WrfDynConfig *config_flags, WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:1178 advance_w */
int wrfgpu_advance_w(float *w, const float *rw_tend, const float *ww, const float *w_save, const float *u,
                     const float *v, const float *mu1, const float *mut, const float *muave, const float *muts,
                     const float *c1h, const float *c2h, const float *c1f, const float *c2f, const float *c3h,
                     const float *c4h, const float *c3f, const float *c4f, float *t_2ave, const float *t_2,
                     const float *t_1, float *ph, const float *ph_1, const float *phb, const float *ph_tend,
                     const float *ht, const float *c2a, const float *cqw, const float *alt, const float *alb,
                     const float *a, const float *alpha, const float *gamma, const float *rdx, const float *rdy,
                     const float *dts, const float *t0, const float *epssm, const float *dnw, const float *fnm,
                     const float *fnp, const float *rdnw, const float *rdn, const float *cf1, const float *cf2,
                     const float *cf3, const float *msftx, const float *msfty, const WrfDynConfig *config_flags,
                     const int *top_lid, WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:1473 sumflux */
int wrfgpu_sumflux(const float *ru, const float *rv, const float *ww, const float *u_lin, const float *v_lin,
                   const float *ww_lin, const float *muu, const float *muv, const float *c1h, const float *c2h,
                   const float *c1f, const float *c2f, const float *c3h, const float *c4h, const float *c3f,
                   const float *c4f, float *ru_m, float *rv_m, float *ww_m, const float *epssm, const float *msfux,
                   const float *msfuy, const float *msfvx, const float *msfvx_inv, const float *msfvy,
                   const int *iteration, const int *number_of_small_timesteps, WRFGPU_DIMS_ARGS);

/* dyn_em/module_small_step_em.F:295 small_step_finish (h_diabatic unused);
 * muus and muvs are read as given (solve_em forms them with calc_mu_uv_1
 * just before, solve_em.F:1732). */
int wrfgpu_small_step_finish(float *u_2, const float *u_1, float *v_2, const float *v_1, float *w_2,
                             const float *w_1, float *t_2, const float *t_1, float *ph_2, const float *ph_1,
                             float *ww, const float *ww1, float *mu_2, const float *mu_1, const float *mut,
                             const float *muts, const float *muu, float *muus, const float *muv, float *muvs,
                             const float *c1h, const float *c2h, const float *c1f, const float *c2f,
                             const float *c3h, const float *c4h, const float *c3f, const float *c4f,
                             const float *u_save, const float *v_save, const float *w_save, const float *t_save,
                             const float *ph_save, const float *mu_save, const float *msfux, const float *msfuy,
                             const float *msfvx, const float *msfvy, const float *msftx, const float *msfty,
                             const float *h_diabatic, const int *number_of_small_timesteps, const float *dts,
                             const int *rk_step, const int *rk_order, WRFGPU_DIMS_ARGS);

/* dyn_em/module_em.F:1587 rk_update_scalar.  scalar_1, scalar_2, sc_tend:
 * (ims:ime,kms:kme,jms:jme,scs:sce) arrays (sc_tend may be NULL: zero);
 * advh_t, advz_t, h_tendency, z_tendency unused (tenddec = .false.) */
int wrfgpu_rk_update_scalar(const int *scs, const int *sce, float *scalar_1, float *scalar_2, const float *sc_tend,
                            const float *advh_t, const float *advz_t, const float *advect_tend,
                            const float *h_tendency, const float *z_tendency, const float *msftx,
                            const float *msfty, const float *c1, const float *c2, const float *mu_old,
                            const float *mu_new, const float *mu_base, const int *rk_step, const float *dt,
                            const int *spec_zone, const WrfDynConfig *config_flags, const int *tenddec,
                            WRFGPU_DIMS_ARGS);

/* dyn_em/module_em.F:1803 rk_update_scalar_pd: scalar (the old species,
 * updated in place) and sc_tend are (ims:ime,kms:kme,jms:jme,scs:sce);
 * sc_tend is added and then zeroed, as the reference does (spec_zone
 * unused: no specified boundaries). */
int wrfgpu_rk_update_scalar_pd(const int *scs, const int *sce, float *scalar, float *sc_tend, const float *c1,
                               const float *c2, const float *mu_old, const float *mu_new, const float *mu_base,
                               const int *rk_step, const float *dt, const int *spec_zone,
                               const WrfDynConfig *config_flags, WRFGPU_DIMS_ARGS);

/* Index of qv in the moist array (P_QV = PARAM_FIRST_SCALAR in the
 * Registry-generated indices): rk_scalar_tend diffuses species P_QV of a
 * moist step vertically against its base profile. */
#define WRFGPU_P_QV 2

/* dyn_em/module_em.F:959 rk_addtend_dry: at rk_step 1 the saved tendencies
 * join the forward ones (ru_tendf += u_save msfuy, rv_tendf += v_save msfvx,
 * rw_tendf += w_save msfty, ph_tendf += ph_save, t_tendf += t_save), then the
 * forward tendencies are added to the large-step ones (divided by the map
 * factors; theta with (c1 mut + c2) h_diabatic / msfty) and mu_tendf to
 * mu_tend.  The patch dims ips..kpe must be those of the single patch the
 * domain is (ips = ids, ..., kpe = kde); msftx, msfux, msfvy are unused as
 * in the reference. */
int wrfgpu_rk_addtend_dry(float *ru_tend, float *rv_tend, float *rw_tend, float *ph_tend, float *t_tend,
                          float *ru_tendf, float *rv_tendf, float *rw_tendf, float *ph_tendf, float *t_tendf,
                          const float *u_save, const float *v_save, const float *w_save, const float *ph_save,
                          const float *t_save, float *mu_tend, float *mu_tendf, const int *rk_step,
                          const float *c1, const float *c2, const float *h_diabatic, const float *mut,
                          const float *msftx, const float *msfty, const float *msfux, const float *msfuy,
                          const float *msfvx, const float *msfvx_inv, const float *msfvy, const int *ids,
                          const int *ide, const int *jds, const int *jde, const int *kds, const int *kde,
                          const int *ims, const int *ime, const int *jms, const int *jme, const int *kms,
                          const int *kme, const int *ips, const int *ipe, const int *jps, const int *jpe,
                          const int *kps, const int *kpe, const int *its, const int *ite, const int *jts,
                          const int *jte, const int *kts, const int *kte);

/* dyn_em/module_em.F:1096 rk_scalar_tend: for each species scs..sce
 * (scalar, scalar_old, scalar_tends: (ims:ime,kms:kme,jms:jme,scs:sce)),
 * advect_tend is zeroed over the tile and receives advect_scalar_pd at the
 * last stage when adv_opt = 1 (positive definite), else advect_scalar.  At
 * stage 1 scalar_tends receives the species' explicit diffusion
 * (config_flags->diff_opt = 1 with km_opt = 1 and mix2_off false:
 * horizontal_diffusion with khdif / prandtl, then vertical_diffusion with
 * kvdif / prandtl, vertical_diffusion_mp against `base` for species
 * WRFGPU_P_QV of a moist step; xkmhd, when given, must hold khdif / prandtl)
 * and then its sixth-order diffusion (diff_6th_opt != 0, mix6_off false).
 * adv_opt other than 0 / 1, tenddec and other diffusion options return
 * WRFGPU_E_ARG; ww, wwI, u_old, v_old, c1f, c2f, h_tendency, z_tendency,
 * RQVFTEN and ph are unused on this path (IEVA off, no cumulus tendency). */
int wrfgpu_rk_scalar_tend(const int *scs, const int *sce, const WrfDynConfig *config_flags, const int *tenddec,
                          const int *rk_step, const float *dt_step, const float *ru, const float *rv,
                          const float *ww, const float *wwE, const float *wwI, const float *u_old,
                          const float *v_old, const float *mut, const float *mub, const float *mu_old,
                          const float *c1h, const float *c2h, const float *c1f, const float *c2f,
                          const float *alt, const float *scalar_old, const float *scalar, float *scalar_tends,
                          float *advect_tend, float *h_tendency, float *z_tendency, const float *RQVFTEN,
                          const float *base, const int *moist_step, const float *fnm, const float *fnp,
                          const float *msfux, const float *msfuy, const float *msfvx, const float *msfvx_inv,
                          const float *msfvy, const float *msftx, const float *msfty, const float *rdx,
                          const float *rdy, const float *rdn, const float *rdnw, const float *khdif,
                          const float *kvdif, const float *xkmhd, const int *diff_6th_opt,
                          const float *diff_6th_factor, const int *adv_opt, const float *phb, const float *ph,
                          const int *mix2_off, const int *mix6_off, WRFGPU_DIMS_ARGS);

/* dyn_em/module_big_step_utilities_em.F:953 calc_p_rho_phi (non-hydrostatic,
 * hypsometric_opt 1 or 2; moist: (ims:ime,kms:kme,jms:jme,n_moist)) */
int wrfgpu_calc_p_rho_phi(const float *moist, const int *n_moist, const int *hypsometric_opt, float *al,
                          const float *alb, const float *mu, const float *muts, const float *c1, const float *c2,
                          const float *c3h, const float *c4h, const float *c3f, const float *c4f, const float *ph,
                          const float *phb, float *p, const float *pb, const float *t, const float *p0,
                          const float *t0, const float *ptop, const float *znu, const float *znw, const float *dnw,
                          const float *rdnw, const float *rdn, const int *non_hydrostatic, const int *use_theta_m,
                          WRFGPU_DIMS_ARGS);

/* Release the cached scratch domains of the routine-level entry points. */
int wrfgpu_fortran_release(void);

#ifdef __cplusplus
}
#endif
#endif /* WRFGPU_FORTRAN_H */
