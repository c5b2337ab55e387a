// Routine-level C ABI (include/wrfgpu_fortran.h): each entry point binds the
// caller's Fortran arrays to the fields of a device scratch domain, in the
// order and meaning of the reference subroutine it replaces, and runs that
// routine's kernel(s) once (parity mode, see fcall.h / driver.cu).
#include <cmath>
#include "fcall.h"
#include "../../include/wrfgpu_fortran.h"

using wrfgpu::FCall;

namespace {

void set_dims(FCall& c, const int* ids, const int* ide, const int* jds, const int* jde, const int* kds,
              const int* kde, const int* ims, const int* ime, const int* jms, const int* jme, const int* kms,
              const int* kme, const int* its, const int* ite, const int* jts, const int* jte, const int* kts,
              const int* kte) {
  const int* d[18] = {ids, ide, jds, jde, kds, kde, ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte};
  for (int q = 0; q < 18; ++q) c.dims[q] = d[q];
}
#define DIMS ids, ide, jds, jde, kds, kde, ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte
#define R(id, p) c.bind(id, p, true, false)
#define W(id, p) c.bind(id, p, false, true)
#define RW(id, p) c.bind(id, p, true, true)

void bind_coefs(FCall& c, const float* c1h, const float* c2h, const float* c1f, const float* c2f) {
  R(WRFGPU_C1H, c1h); R(WRFGPU_C2H, c2h); R(WRFGPU_C1F, c1f); R(WRFGPU_C2F, c2f);
}
void bind_coefs34(FCall& c, const float* c3h, const float* c4h, const float* c3f, const float* c4f) {
  R(WRFGPU_C3H, c3h); R(WRFGPU_C4H, c4h); R(WRFGPU_C3F, c3f); R(WRFGPU_C4F, c4f);
}
int cfg_ok(const WrfDynConfig* cf) { return cf ? 0 : WRFGPU_E_ARG; }

}  // namespace

extern "C" {

int wrfgpu_rk_step_prep(const WrfDynConfig* config_flags, const int* rk_step, const float* u, const float* v,
                        const float* w, const float* t, const float* ph, const float* mu, const float* c1h,
                        const float* c2h, const float* c1f, const float* c2f, const float* moist, float* ru,
                        float* rv, float* rw, float* ww, float* php, float* alt, float* muu, float* muv,
                        const float* mub, float* mut, const float* phb, const float* pb, const float* p,
                        const float* al, const float* alb, float* cqu, float* cqv, float* cqw, const float* msfux,
                        const float* msfuy, const float* msfvx, const float* msfvx_inv, const float* msfvy,
                        const float* msftx, const float* msfty, const float* fnm, const float* fnp, const float* dnw,
                        const float* rdx, const float* rdy, const int* n_moist, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !rk_step || !rdx || !rdy || !n_moist || *n_moist != 1) return WRFGPU_E_ARG;
  (void)t;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = WRFGPU_R_RK_STEP_PREP; c.rk_step = *rk_step;
  c.rdx = *rdx; c.rdy = *rdy;
  R(WRFGPU_U_2, u); R(WRFGPU_V_2, v); R(WRFGPU_W_2, w); R(WRFGPU_PH_2, ph); R(WRFGPU_MU_2, mu);
  bind_coefs(c, c1h, c2h, c1f, c2f);
  R(WRFGPU_SPECIES_BASE, moist);
  W(WRFGPU_RU, ru); W(WRFGPU_RV, rv); W(WRFGPU_RW, rw); W(WRFGPU_WW, ww); W(WRFGPU_PHP, php); W(WRFGPU_ALT, alt);
  W(WRFGPU_MUU, muu); W(WRFGPU_MUV, muv); R(WRFGPU_MUB, mub); W(WRFGPU_MUT, mut); R(WRFGPU_PHB, phb);
  R(WRFGPU_PB, pb); R(WRFGPU_P, p); R(WRFGPU_AL, al); R(WRFGPU_ALB, alb);
  W(WRFGPU_CQU, cqu); W(WRFGPU_CQV, cqv); W(WRFGPU_CQW, cqw);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  R(WRFGPU_MSFVY, msfvy); R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  R(WRFGPU_FNM, fnm); R(WRFGPU_FNP, fnp); R(WRFGPU_DNW, dnw);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_rk_tendency(const WrfDynConfig* config_flags, const int* rk_step, float* ru_tend, float* rv_tend,
                       float* rw_tend, float* ph_tend, float* t_tend, float* ru_tendf, float* rv_tendf,
                       float* rw_tendf, const float* ph_tendf, float* t_tendf, float* mu_tend,
                       float* u_save, float* v_save, float* w_save, float* ph_save, float* t_save, float* mu_save,
                       const float* RTHFTEN, const float* ru, const float* rv, const float* rw, const float* ww,
                       const float* wwE, const float* wwI, const float* u, const float* v, const float* w,
                       const float* t, const float* ph, const float* u_old, const float* v_old, const float* w_old,
                       const float* t_old, const float* ph_old, const float* h_diabatic, const float* phb,
                       const float* t_init, const float* mu_old, const float* mu, const float* mut,
                       const float* muu, const float* muv, const float* mub, const float* c1h, const float* c2h,
                       const float* c1f, const float* c2f, const float* al, const float* ht, const float* alt,
                       const float* p, const float* pb, const float* php, const float* cqu, const float* cqv,
                       float* cqw, const float* u_base, const float* v_base, const float* t_base,
                       const float* qv_base, const float* z_base, const float* msfux, const float* msfuy,
                       const float* msfvx, const float* msfvx_inv, const float* msfvy, const float* msftx,
                       const float* msfty, const float* clat, const float* f, const float* e, const float* sina,
                       const float* cosa, const float* fnm, const float* fnp, const float* rdn, const float* rdnw,
                       const float* dt, const float* rdx, const float* rdy, const float* khdif,
                       const float* kvdif, const float* xkmhd, const float* xkhh, const int* diff_6th_opt,
                       const float* diff_6th_factor, const int* adv_opt, const float* dampcoef,
                       const float* zdamp, const int* damp_opt, const int* rad_nudge, const float* cf1,
                       const float* cf2, const float* cf3, const float* cfn, const float* cfn1, const int* n_moist,
                       const int* non_hydrostatic, const int* top_lid, const float* u_frame, const float* v_frame,
                       WRFGPU_DIMS_ARGS, float* max_vert_cfl, float* max_horiz_cfl) {
  if (cfg_ok(config_flags) || !rk_step || !dt || !rdx || !rdy || !cf1 || !cf2 || !cf3 || !cfn || !cfn1)
    return WRFGPU_E_ARG;
  // physics and IEVA inputs of the reference's signature are zero / off on
  // this path; the diffusion and damping inputs feed the forward step below
  (void)ph_tendf; (void)RTHFTEN; (void)wwE; (void)wwI; (void)u_old; (void)v_old; (void)w_old; (void)t_old;
  (void)ph_old; (void)h_diabatic; (void)mu_old; (void)ht; (void)qv_base; (void)clat; (void)adv_opt;
  (void)rad_nudge; (void)n_moist; (void)non_hydrostatic; (void)top_lid; (void)u_frame; (void)v_frame;
  // the forward step's options (module_em.F:801-944): the arguments of the
  // reference's call where given, else the configuration's
  WrfDynConfig fcf = *config_flags;
  if (diff_6th_opt) fcf.diff_6th_opt = *diff_6th_opt;
  if (diff_6th_factor) fcf.diff_6th_factor = *diff_6th_factor;
  if (damp_opt) fcf.damp_opt = *damp_opt;
  if (dampcoef) fcf.dampcoef = *dampcoef;
  if (zdamp) fcf.zdamp = *zdamp;
  if (khdif) fcf.khdif = *khdif;
  if (kvdif) fcf.kvdif = *kvdif;
  const bool fwd = *rk_step == 1 && (fcf.diff_opt == 1 || fcf.diff_6th_opt != 0 || fcf.damp_opt == 2);
  if (fwd) {
    if (!ru_tendf || !rv_tendf || !rw_tendf || !t_tendf || !phb || !ph || !mut || !muu || !muv) return WRFGPU_E_ARG;
    if (fcf.diff_opt == 1) {
      if (!t_init || !alt || !rdn || !rdnw || !u_base || !v_base) return WRFGPU_E_ARG;
      // km_opt = 1 (isotropic_km): the coefficient arrays hold khdif and khdif / prandtl
      const size_t o0 = (size_t)(*its - *ims) +
                        (size_t)(*ime - *ims + 1) * ((size_t)(*kts - *kms) + (size_t)(*kme - *kms + 1) * (size_t)(*jts - *jms));
      if ((xkmhd && xkmhd[o0] != fcf.khdif) || (xkhh && xkhh[o0] != fcf.khdif / (1.f / 3.0f))) return WRFGPU_E_ARG;
    }
    if (fcf.damp_opt == 2 && (!u_base || !v_base || !t_base || !z_base)) return WRFGPU_E_ARG;
  }
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = WRFGPU_R_RK_TENDENCY; c.rk_step = *rk_step;
  c.dt = *dt; c.rdx = *rdx; c.rdy = *rdy;
  c.have_cf = true; c.cf1 = *cf1; c.cf2 = *cf2; c.cf3 = *cf3;
  c.have_cfn = true; c.cfn = *cfn; c.cfn1 = *cfn1;
  c.zero_saves = true;
  c.max_vert_cfl = max_vert_cfl; c.max_horiz_cfl = max_horiz_cfl;
  W(WRFGPU_RU_TEND, ru_tend); W(WRFGPU_RV_TEND, rv_tend); W(WRFGPU_RW_TEND, rw_tend); W(WRFGPU_PH_TEND, ph_tend);
  W(WRFGPU_T_TEND, t_tend); W(WRFGPU_MU_TEND, mu_tend);
  W(WRFGPU_U_SAVE, u_save); W(WRFGPU_V_SAVE, v_save); W(WRFGPU_W_SAVE, w_save); W(WRFGPU_PH_SAVE, ph_save);
  W(WRFGPU_T_SAVE, t_save); W(WRFGPU_MU_SAVE, mu_save);
  R(WRFGPU_RU, ru); R(WRFGPU_RV, rv); R(WRFGPU_RW, rw); R(WRFGPU_WW, ww);
  R(WRFGPU_U_2, u); R(WRFGPU_V_2, v); R(WRFGPU_W_2, w); R(WRFGPU_T_2, t); R(WRFGPU_PH_2, ph); R(WRFGPU_PHB, phb);
  R(WRFGPU_MU_2, mu); R(WRFGPU_MUT, mut); R(WRFGPU_MUU, muu); R(WRFGPU_MUV, muv); R(WRFGPU_MUB, mub);
  bind_coefs(c, c1h, c2h, c1f, c2f);
  R(WRFGPU_AL, al); R(WRFGPU_ALT, alt); R(WRFGPU_P, p); R(WRFGPU_PB, pb); R(WRFGPU_PHP, php);
  R(WRFGPU_CQU, cqu); R(WRFGPU_CQV, cqv); RW(WRFGPU_CQW, cqw);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  R(WRFGPU_MSFVY, msfvy); R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  R(WRFGPU_F, f); R(WRFGPU_E, e); R(WRFGPU_SINA, sina); R(WRFGPU_COSA, cosa);
  R(WRFGPU_FNM, fnm); R(WRFGPU_FNP, fnp); R(WRFGPU_RDN, rdn); R(WRFGPU_RDNW, rdnw);
  int rc = wrfgpu::fortran_call(c);
  if (rc || !fwd) return rc;
  // stage 1's forward terms added to ru_tendf .. t_tendf (rk_addtend_dry,
  // a separate call of solve_em, adds those to the large-step tendencies)
  FCall d;
  set_dims(d, DIMS);
  d.cfg = fcf; d.routine = 133; d.rk_step = 1;
  d.dt = *dt; d.rdx = *rdx; d.rdy = *rdy;
  {
    FCall& c = d;  // the binding macros name the call `c`
    RW(WRFGPU_RU_TENDF, ru_tendf); RW(WRFGPU_RV_TENDF, rv_tendf); RW(WRFGPU_RW_TENDF, rw_tendf);
    RW(WRFGPU_T_TENDF, t_tendf);
    R(WRFGPU_U_2, u); R(WRFGPU_V_2, v); R(WRFGPU_W_2, w); R(WRFGPU_T_2, t); R(WRFGPU_PH_2, ph);
    R(WRFGPU_PHB, phb); R(WRFGPU_T_INIT, t_init); R(WRFGPU_ALT, alt);
    R(WRFGPU_MUT, mut); R(WRFGPU_MUU, muu); R(WRFGPU_MUV, muv);
    bind_coefs(c, c1h, c2h, c1f, c2f);
    R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
    R(WRFGPU_MSFVY, msfvy); R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
    R(WRFGPU_RDN, rdn); R(WRFGPU_RDNW, rdnw);
    R(WRFGPU_U_BASE, u_base); R(WRFGPU_V_BASE, v_base); R(WRFGPU_T_BASE, t_base); R(WRFGPU_Z_BASE, z_base);
  }
  return wrfgpu::fortran_call(d);
}

// advect_u / advect_v / advect_w / advect_scalar: tendency += -div(flux)
static int advect_common(int routine, int fld_id, int tend_id, int rdz_id, const float* fld, float* tendency,
                         const float* ru, const float* rv, const float* rom, const float* c1, const float* c2,
                         const float* mut, const int* time_step, const WrfDynConfig* config_flags,
                         const float* msfux, const float* msfuy, const float* msfvx, const float* msfvy,
                         const float* msftx, const float* msfty, const float* fzm, const float* fzp,
                         const float* rdx, const float* rdy, const float* rdzw, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !rdx || !rdy || (time_step && *time_step < 0)) return WRFGPU_E_ARG;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = routine; c.rk_step = 2;
  c.rdx = *rdx; c.rdy = *rdy;
  R(fld_id, fld); RW(tend_id, tendency);
  const bool scalar = fld_id >= WRFGPU_SPECIES_BASE;
  R(scalar ? WRFGPU_RU_M : WRFGPU_RU, ru); R(scalar ? WRFGPU_RV_M : WRFGPU_RV, rv); R(scalar ? WRFGPU_WW_M : WRFGPU_WW, rom);
  R(WRFGPU_C1H, c1); R(WRFGPU_C2H, c2); R(scalar ? WRFGPU_MUTS : WRFGPU_MUT, mut);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVY, msfvy);
  R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  R(WRFGPU_FNM, fzm); R(WRFGPU_FNP, fzp); R(rdz_id, rdzw);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_advect_u(const float* u, const float* u_old, float* tendency, const float* ru, const float* rv,
                    const float* rom, const float* c1, const float* c2, const float* mut, const int* time_step,
                    const WrfDynConfig* config_flags, const float* msfux, const float* msfuy, const float* msfvx,
                    const float* msfvy, const float* msftx, const float* msfty, const float* fzm, const float* fzp,
                    const float* rdx, const float* rdy, const float* rdzw, WRFGPU_DIMS_ARGS) {
  // the old field enters only the radiation terms of open boundaries, and
  // the reference's calls (rk_tendency, rk_scalar_tend) pass the field itself
  if (u_old != u && config_flags && (config_flags->open_xs || config_flags->open_ys)) return WRFGPU_E_ARG;
  return advect_common(WRFGPU_R_ADVECT_U, WRFGPU_U_2, WRFGPU_RU_TEND, WRFGPU_RDNW, u, tendency, ru, rv, rom, c1, c2,
                       mut, time_step, config_flags, msfux, msfuy, msfvx, msfvy, msftx, msfty, fzm, fzp, rdx, rdy,
                       rdzw, DIMS);
}
int wrfgpu_advect_v(const float* v, const float* v_old, float* tendency, const float* ru, const float* rv,
                    const float* rom, const float* c1, const float* c2, const float* mut, const int* time_step,
                    const WrfDynConfig* config_flags, const float* msfux, const float* msfuy, const float* msfvx,
                    const float* msfvy, const float* msftx, const float* msfty, const float* fzm, const float* fzp,
                    const float* rdx, const float* rdy, const float* rdzw, WRFGPU_DIMS_ARGS) {
  // the old field enters only the radiation terms of open boundaries, and
  // the reference's calls (rk_tendency, rk_scalar_tend) pass the field itself
  if (v_old != v && config_flags && (config_flags->open_xs || config_flags->open_ys)) return WRFGPU_E_ARG;
  return advect_common(WRFGPU_R_ADVECT_V, WRFGPU_V_2, WRFGPU_RV_TEND, WRFGPU_RDNW, v, tendency, ru, rv, rom, c1, c2,
                       mut, time_step, config_flags, msfux, msfuy, msfvx, msfvy, msftx, msfty, fzm, fzp, rdx, rdy,
                       rdzw, DIMS);
}
int wrfgpu_advect_w(const float* w, const float* w_old, float* tendency, const float* ru, const float* rv,
                    const float* rom, const float* c1, const float* c2, const float* mut, const int* time_step,
                    const WrfDynConfig* config_flags, const float* msfux, const float* msfuy, const float* msfvx,
                    const float* msfvy, const float* msftx, const float* msfty, const float* fzm, const float* fzp,
                    const float* rdx, const float* rdy, const float* rdzu, WRFGPU_DIMS_ARGS) {
  // the old field enters only the radiation terms of open boundaries, and
  // the reference's calls (rk_tendency, rk_scalar_tend) pass the field itself
  if (w_old != w && config_flags && (config_flags->open_xs || config_flags->open_ys)) return WRFGPU_E_ARG;
  return advect_common(WRFGPU_R_ADVECT_W, WRFGPU_W_2, WRFGPU_RW_TEND, WRFGPU_RDN, w, tendency, ru, rv, rom, c1, c2,
                       mut, time_step, config_flags, msfux, msfuy, msfvx, msfvy, msftx, msfty, fzm, fzp, rdx, rdy,
                       rdzu, DIMS);
}
int wrfgpu_advect_scalar(const float* field, const float* field_old, float* tendency, const float* ru,
                         const float* rv, const float* rom, const float* c1, const float* c2, const float* mut,
                         const int* time_step, const WrfDynConfig* config_flags, const float* msfux,
                         const float* msfuy, const float* msfvx, const float* msfvy, const float* msftx,
                         const float* msfty, const float* fzm, const float* fzp, const float* rdx, const float* rdy,
                         const float* rdzw, WRFGPU_DIMS_ARGS) {
  // the old field enters only the radiation terms of open boundaries, and
  // the reference's calls (rk_tendency, rk_scalar_tend) pass the field itself
  if (field_old != field && config_flags && (config_flags->open_xs || config_flags->open_ys)) return WRFGPU_E_ARG;
  return advect_common(121, WRFGPU_SPECIES_BASE, WRFGPU_ADVECT_TEND, WRFGPU_RDNW, field, tendency, ru, rv, rom, c1,
                       c2, mut, time_step, config_flags, msfux, msfuy, msfvx, msfvy, msftx, msfty, fzm, fzp, rdx,
                       rdy, rdzw, DIMS);
}

int wrfgpu_advect_scalar_pd(const float* field, const float* field_old, float* tendency, float* h_tendency,
                            float* z_tendency, const float* ru, const float* rv, const float* rom, const float* c1,
                            const float* c2, const float* mut, const float* mub, const float* mu_old,
                            const int* time_step, const WrfDynConfig* config_flags, const int* tenddec,
                            const float* msfux, const float* msfuy, const float* msfvx, const float* msfvy,
                            const float* msftx, const float* msfty, const float* fzm, const float* fzp,
                            const float* rdx, const float* rdy, const float* rdzw, const float* dt,
                            WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !rdx || !rdy || !dt || (tenddec && *tenddec) || (time_step && *time_step < 0))
    return WRFGPU_E_ARG;
  (void)h_tendency; (void)z_tendency;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = 122; c.rk_step = 3;
  c.rdx = *rdx; c.rdy = *rdy; c.dtrk = *dt;
  R(WRFGPU_SPECIES_BASE, field); R(WRFGPU_SPECIES_BASE + 1, field_old); RW(WRFGPU_ADVECT_TEND, tendency);
  R(WRFGPU_RU_M, ru); R(WRFGPU_RV_M, rv); R(WRFGPU_WW_M, rom); R(WRFGPU_C1H, c1); R(WRFGPU_C2H, c2);
  R(WRFGPU_MUTS, mut); R(WRFGPU_MUB, mub); R(WRFGPU_MU_1, mu_old);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVY, msfvy);
  R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  R(WRFGPU_FNM, fzm); R(WRFGPU_FNP, fzp); R(WRFGPU_RDNW, rdzw);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_small_step_prep(float* u_1, float* u_2, float* v_1, float* v_2, float* w_1, float* w_2, float* t_1,
                           float* t_2, float* ph_1, float* ph_2, const float* mub, float* mu_1, float* mu_2,
                           const float* muu, float* muus, const float* muv, float* muvs, const float* mut,
                           float* muts, float* mudf, const float* c1h, const float* c2h, const float* c1f,
                           const float* c2f, const float* c3h, const float* c4h, const float* c3f, const float* c4f,
                           float* u_save, float* v_save, float* w_save, float* t_save, float* ph_save,
                           float* mu_save, const float* ww, float* ww_save, float* c2a, const float* pb,
                           const float* p, const float* alt, const float* msfux, const float* msfuy,
                           const float* msfvx, const float* msfvx_inv, const float* msfvy, const float* msftx,
                           const float* msfty, const float* rdx, const float* rdy, const int* rk_step,
                           WRFGPU_DIMS_ARGS) {
  if (!rk_step || !rdx || !rdy) return WRFGPU_E_ARG;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = [] { WrfDynConfig k{}; k.periodic_x = k.periodic_y = 1; k.rk_ord = 3; k.h_mom_adv_order = 5;
               k.h_sca_adv_order = 5; k.v_mom_adv_order = 3; k.v_sca_adv_order = 3; k.non_hydrostatic = 1;
               k.hypsometric_opt = 2; return k; }();
  c.routine = WRFGPU_R_SMALL_STEP_PREP; c.rk_step = *rk_step; c.rdx = *rdx; c.rdy = *rdy;
  RW(WRFGPU_U_1, u_1); RW(WRFGPU_U_2, u_2); RW(WRFGPU_V_1, v_1); RW(WRFGPU_V_2, v_2); RW(WRFGPU_W_1, w_1);
  RW(WRFGPU_W_2, w_2); RW(WRFGPU_T_1, t_1); RW(WRFGPU_T_2, t_2); RW(WRFGPU_PH_1, ph_1); RW(WRFGPU_PH_2, ph_2);
  R(WRFGPU_MUB, mub); RW(WRFGPU_MU_1, mu_1); RW(WRFGPU_MU_2, mu_2); R(WRFGPU_MUU, muu); RW(WRFGPU_MUUS, muus);
  R(WRFGPU_MUV, muv); RW(WRFGPU_MUVS, muvs); R(WRFGPU_MUT, mut); RW(WRFGPU_MUTS, muts); RW(WRFGPU_MUDF, mudf);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  RW(WRFGPU_U_SAVE, u_save); RW(WRFGPU_V_SAVE, v_save); RW(WRFGPU_W_SAVE, w_save); RW(WRFGPU_T_SAVE, t_save);
  RW(WRFGPU_PH_SAVE, ph_save); RW(WRFGPU_MU_SAVE, mu_save); R(WRFGPU_WW, ww); RW(WRFGPU_WW1, ww_save);
  RW(WRFGPU_C2A, c2a); R(WRFGPU_PB, pb); R(WRFGPU_P, p); R(WRFGPU_ALT, alt);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  R(WRFGPU_MSFVY, msfvy); R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  return wrfgpu::fortran_call(c);
}

// the physics-off configuration the acoustic routines run with when the
// reference does not pass config_flags
static WrfDynConfig default_cfg(int top_lid) {
  WrfDynConfig k{};
  k.periodic_x = k.periodic_y = 1; k.rk_ord = 3; k.h_mom_adv_order = 5; k.h_sca_adv_order = 5;
  k.v_mom_adv_order = 3; k.v_sca_adv_order = 3; k.non_hydrostatic = 1; k.hypsometric_opt = 2; k.top_lid = top_lid;
  k.moist_adv_opt = 1; k.scalar_adv_opt = 1; k.use_theta_m = 1; k.phi_adv_z = 1;
  return k;
}

int wrfgpu_calc_p_rho(float* al, float* p, const float* ph, const float* alt, const float* t_2, const float* t_1,
                      const float* c2a, float* pm1, const float* mu, const float* mut, const float* c1h,
                      const float* c2h, const float* c1f, const float* c2f, const float* c3h, const float* c4h,
                      const float* c3f, const float* c4f, const float* znu, const float* t0, const float* rdnw,
                      const float* dnw, const float* smdiv, const int* non_hydrostatic, const int* step,
                      WRFGPU_DIMS_ARGS) {
  if (!smdiv || !step || !non_hydrostatic || !*non_hydrostatic || (t0 && *t0 != 300.f)) return WRFGPU_E_ARG;
  (void)znu; (void)dnw;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = default_cfg(0); c.routine = WRFGPU_R_CALC_P_RHO; c.iteration = *step; c.smdiv = *smdiv;
  RW(WRFGPU_AL, al); RW(WRFGPU_P, p); R(WRFGPU_PH_2, ph); R(WRFGPU_ALT, alt); R(WRFGPU_T_2, t_2);
  R(WRFGPU_T_SAVE, t_1); R(WRFGPU_C2A, c2a); RW(WRFGPU_PM1, pm1); R(WRFGPU_MU_2, mu); R(WRFGPU_MUTS, mut);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  R(WRFGPU_RDNW, rdnw);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_calc_coef_w(float* a, float* alpha, float* gamma, const float* mut, const float* c1h, const float* c2h,
                       const float* c1f, const float* c2f, const float* c3h, const float* c4h, const float* c3f,
                       const float* c4f, const float* cqw, const float* rdn, const float* rdnw, const float* c2a,
                       const float* dts, const float* g, const float* epssm, const int* top_lid, WRFGPU_DIMS_ARGS) {
  if (!dts || !epssm || !top_lid || (g && *g != 9.81f)) return WRFGPU_E_ARG;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = default_cfg(*top_lid); c.routine = WRFGPU_R_CALC_COEF_W; c.rk_step = 2; c.dts = *dts; c.epssm = *epssm;
  W(WRFGPU_A, a); W(WRFGPU_ALPHA, alpha); W(WRFGPU_GAMMA, gamma); R(WRFGPU_MUT, mut);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  R(WRFGPU_CQW, cqw); R(WRFGPU_RDN, rdn); R(WRFGPU_RDNW, rdnw); R(WRFGPU_C2A, c2a);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_advance_uv(float* u, const float* ru_tend, float* v, const float* rv_tend, const float* p,
                      const float* pb, const float* ph, const float* php, const float* alt, const float* al,
                      const float* mu, const float* muu, const float* cqu, const float* muv, const float* cqv,
                      const float* mudf, const float* c1h, const float* c2h, const float* c1f, const float* c2f,
                      const float* c3h, const float* c4h, const float* c3f, const float* c4f, const float* msfux,
                      const float* msfuy, const float* msfvx, const float* msfvx_inv, const float* msfvy,
                      const float* rdx, const float* rdy, const float* dts, const float* cf1, const float* cf2,
                      const float* cf3, const float* fnm, const float* fnp, const float* emdiv, const float* rdnw,
                      const WrfDynConfig* config_flags, const int* spec_zone, const int* non_hydrostatic,
                      const int* top_lid, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !rdx || !rdy || !dts || !cf1 || !cf2 || !cf3 || !emdiv) return WRFGPU_E_ARG;
  (void)spec_zone; (void)non_hydrostatic; (void)top_lid;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = WRFGPU_R_ADVANCE_UV; c.rk_step = 2; c.iteration = 1;
  c.rdx = *rdx; c.rdy = *rdy; c.dts = *dts; c.emdiv = *emdiv;
  c.have_cf = true; c.cf1 = *cf1; c.cf2 = *cf2; c.cf3 = *cf3;
  RW(WRFGPU_U_2, u); R(WRFGPU_RU_TEND, ru_tend); RW(WRFGPU_V_2, v); R(WRFGPU_RV_TEND, rv_tend);
  R(WRFGPU_P, p); R(WRFGPU_PB, pb); R(WRFGPU_PH_2, ph); R(WRFGPU_PHP, php); R(WRFGPU_ALT, alt); R(WRFGPU_AL, al);
  R(WRFGPU_MU_2, mu); R(WRFGPU_MUU, muu); R(WRFGPU_CQU, cqu); R(WRFGPU_MUV, muv); R(WRFGPU_CQV, cqv);
  R(WRFGPU_MUDF, mudf);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  R(WRFGPU_MSFVY, msfvy); R(WRFGPU_FNM, fnm); R(WRFGPU_FNP, fnp); R(WRFGPU_RDNW, rdnw);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_advance_mu_t(float* ww, float* ww_1, const float* u, const float* u_1, const float* v, const float* v_1,
                        float* mu, const float* mut, float* muave, float* muts, const float* muu, const float* muv,
                        float* mudf, const float* c1h, const float* c2h, const float* c1f, const float* c2f,
                        const float* c3h, const float* c4h, const float* c3f, const float* c4f, const float* uam,
                        const float* vam, const float* wwam, float* t, const float* t_1, float* t_ave,
                        const float* ft, const float* mu_tend, const float* rdx, const float* rdy, const float* dts,
                        const float* epssm, const float* dnw, const float* fnm, const float* fnp, const float* rdnw,
                        const float* msfux, const float* msfuy, const float* msfvx, const float* msfvx_inv,
                        const float* msfvy, const float* msftx, const float* msfty, const int* step,
                        const WrfDynConfig* config_flags, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !rdx || !rdy || !dts || !epssm || !step) return WRFGPU_E_ARG;
  (void)uam; (void)vam; (void)wwam;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = WRFGPU_R_ADVANCE_MU_T; c.rk_step = 2; c.iteration = *step;
  c.rdx = *rdx; c.rdy = *rdy; c.dts = *dts; c.epssm = *epssm;
  RW(WRFGPU_WW, ww); RW(WRFGPU_WW1, ww_1); R(WRFGPU_U_2, u); R(WRFGPU_U_SAVE, u_1); R(WRFGPU_V_2, v);
  R(WRFGPU_V_SAVE, v_1); RW(WRFGPU_MU_2, mu); R(WRFGPU_MUT, mut); RW(WRFGPU_MUAVE, muave); RW(WRFGPU_MUTS, muts);
  R(WRFGPU_MUU, muu); R(WRFGPU_MUV, muv); RW(WRFGPU_MUDF, mudf);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  RW(WRFGPU_T_2, t); R(WRFGPU_T_SAVE, t_1); RW(WRFGPU_T_2SAVE, t_ave); R(WRFGPU_T_TEND, ft);
  R(WRFGPU_MU_TEND, mu_tend); R(WRFGPU_DNW, dnw); R(WRFGPU_FNM, fnm); R(WRFGPU_FNP, fnp); R(WRFGPU_RDNW, rdnw);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  R(WRFGPU_MSFVY, msfvy); R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_advance_w(float* w, const float* rw_tend, const float* ww, const float* w_save, const float* u,
                     const float* v, const float* mu1, const float* mut, const float* muave, const float* muts,
                     const float* c1h, const float* c2h, const float* c1f, const float* c2f, const float* c3h,
                     const float* c4h, const float* c3f, const float* c4f, float* t_2ave, const float* t_2,
                     const float* t_1, float* ph, const float* ph_1, const float* phb, const float* ph_tend,
                     const float* ht, const float* c2a, const float* cqw, const float* alt, const float* alb,
                     const float* a, const float* alpha, const float* gamma, const float* rdx, const float* rdy,
                     const float* dts, const float* t0, const float* epssm, const float* dnw, const float* fnm,
                     const float* fnp, const float* rdnw, const float* rdn, const float* cf1, const float* cf2,
                     const float* cf3, const float* msftx, const float* msfty, const WrfDynConfig* config_flags,
                     const int* top_lid, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !rdx || !rdy || !dts || !epssm || !cf1 || !cf2 || !cf3 || (t0 && *t0 != 300.f))
    return WRFGPU_E_ARG;
  (void)top_lid; (void)dnw; (void)alb;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = *config_flags; c.routine = WRFGPU_R_ADVANCE_W; c.rk_step = 2; c.iteration = 1;
  c.rdx = *rdx; c.rdy = *rdy; c.dts = *dts; c.epssm = *epssm;
  c.have_cf = true; c.cf1 = *cf1; c.cf2 = *cf2; c.cf3 = *cf3;
  RW(WRFGPU_W_2, w); R(WRFGPU_RW_TEND, rw_tend); R(WRFGPU_WW, ww); R(WRFGPU_W_SAVE, w_save); R(WRFGPU_U_2, u);
  R(WRFGPU_V_2, v); R(WRFGPU_MU_2, mu1); R(WRFGPU_MUT, mut); R(WRFGPU_MUAVE, muave); R(WRFGPU_MUTS, muts);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  RW(WRFGPU_T_2SAVE, t_2ave); R(WRFGPU_T_2, t_2); R(WRFGPU_T_SAVE, t_1); RW(WRFGPU_PH_2, ph);
  R(WRFGPU_PH_SAVE, ph_1); R(WRFGPU_PHB, phb); R(WRFGPU_PH_TEND, ph_tend); R(WRFGPU_HT, ht); R(WRFGPU_C2A, c2a);
  R(WRFGPU_CQW, cqw); R(WRFGPU_ALT, alt); R(WRFGPU_A, a); R(WRFGPU_ALPHA, alpha); R(WRFGPU_GAMMA, gamma);
  R(WRFGPU_FNM, fnm); R(WRFGPU_FNP, fnp); R(WRFGPU_RDNW, rdnw); R(WRFGPU_RDN, rdn);
  R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_sumflux(const float* ru, const float* rv, const float* ww, const float* u_lin, const float* v_lin,
                   const float* ww_lin, const float* muu, const float* muv, const float* c1h, const float* c2h,
                   const float* c1f, const float* c2f, const float* c3h, const float* c4h, const float* c3f,
                   const float* c4f, float* ru_m, float* rv_m, float* ww_m, const float* epssm, const float* msfux,
                   const float* msfuy, const float* msfvx, const float* msfvx_inv, const float* msfvy,
                   const int* iteration, const int* number_of_small_timesteps, WRFGPU_DIMS_ARGS) {
  if (!iteration || !number_of_small_timesteps || *number_of_small_timesteps < 1) return WRFGPU_E_ARG;
  (void)epssm;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = default_cfg(0); c.routine = WRFGPU_R_SUMFLUX; c.rk_step = 2; c.iteration = *iteration;
  c.nsmall = *number_of_small_timesteps;
  R(WRFGPU_U_2, ru); R(WRFGPU_V_2, rv); R(WRFGPU_WW, ww); R(WRFGPU_U_SAVE, u_lin); R(WRFGPU_V_SAVE, v_lin);
  R(WRFGPU_WW1, ww_lin); R(WRFGPU_MUU, muu); R(WRFGPU_MUV, muv);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  RW(WRFGPU_RU_M, ru_m); RW(WRFGPU_RV_M, rv_m); RW(WRFGPU_WW_M, ww_m);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  R(WRFGPU_MSFVY, msfvy);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_small_step_finish(float* u_2, const float* u_1, float* v_2, const float* v_1, float* w_2,
                             const float* w_1, float* t_2, const float* t_1, float* ph_2, const float* ph_1,
                             float* ww, const float* ww1, float* mu_2, const float* mu_1, const float* mut,
                             const float* muts, const float* muu, float* muus, const float* muv, float* muvs,
                             const float* c1h, const float* c2h, const float* c1f, const float* c2f,
                             const float* c3h, const float* c4h, const float* c3f, const float* c4f,
                             const float* u_save, const float* v_save, const float* w_save, const float* t_save,
                             const float* ph_save, const float* mu_save, const float* msfux, const float* msfuy,
                             const float* msfvx, const float* msfvy, const float* msftx, const float* msfty,
                             const float* h_diabatic, const int* number_of_small_timesteps, const float* dts,
                             const int* rk_step, const int* rk_order, WRFGPU_DIMS_ARGS) {
  if (!number_of_small_timesteps || !dts || !rk_step || !rk_order || *rk_order != 3) return WRFGPU_E_ARG;
  (void)h_diabatic;
  FCall c;
  set_dims(c, DIMS);
  // small_step_finish reads the muus, muvs its caller formed with calc_mu_uv_1
  c.cfg = default_cfg(0); c.routine = 119; c.rk_step = *rk_step;
  c.nsmall = *number_of_small_timesteps; c.dts = *dts;
  RW(WRFGPU_U_2, u_2); R(WRFGPU_U_1, u_1); RW(WRFGPU_V_2, v_2); R(WRFGPU_V_1, v_1); RW(WRFGPU_W_2, w_2);
  R(WRFGPU_W_1, w_1); RW(WRFGPU_T_2, t_2); R(WRFGPU_T_1, t_1); RW(WRFGPU_PH_2, ph_2); R(WRFGPU_PH_1, ph_1);
  RW(WRFGPU_WW, ww); R(WRFGPU_WW1, ww1); RW(WRFGPU_MU_2, mu_2); R(WRFGPU_MU_1, mu_1); R(WRFGPU_MUT, mut);
  R(WRFGPU_MUTS, muts); R(WRFGPU_MUU, muu); RW(WRFGPU_MUUS, muus); R(WRFGPU_MUV, muv); RW(WRFGPU_MUVS, muvs);
  bind_coefs(c, c1h, c2h, c1f, c2f); bind_coefs34(c, c3h, c4h, c3f, c4f);
  R(WRFGPU_U_SAVE, u_save); R(WRFGPU_V_SAVE, v_save); R(WRFGPU_W_SAVE, w_save); R(WRFGPU_T_SAVE, t_save);
  R(WRFGPU_PH_SAVE, ph_save); R(WRFGPU_MU_SAVE, mu_save);
  R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVY, msfvy);
  R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_rk_update_scalar(const int* scs, const int* sce, float* scalar_1, float* scalar_2, const float* sc_tend,
                            const float* advh_t, const float* advz_t, const float* advect_tend,
                            const float* h_tendency, const float* z_tendency, const float* msftx,
                            const float* msfty, const float* c1, const float* c2, const float* mu_old,
                            const float* mu_new, const float* mu_base, const int* rk_step, const float* dt,
                            const int* spec_zone, const WrfDynConfig* config_flags, const int* tenddec,
                            WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !scs || !sce || !rk_step || !dt || (tenddec && *tenddec) || *sce < *scs)
    return WRFGPU_E_ARG;
  (void)advh_t; (void)advz_t; (void)h_tendency; (void)z_tendency; (void)spec_zone;
  // scalar_1, scalar_2 and sc_tend are (ims:ime,kms:kme,jms:jme,scs:sce)
  const size_t n3 = (size_t)(*ime - *ims + 1) * (size_t)(*kme - *kms + 1) * (size_t)(*jme - *jms + 1);
  for (int im = *scs; im <= *sce; ++im) {
    const size_t off = (size_t)(im - *scs) * n3;
    FCall c;
    set_dims(c, DIMS);
    c.cfg = *config_flags; c.routine = 130; c.rk_step = *rk_step; c.dtrk = *dt;
    RW(WRFGPU_SPECIES_BASE + 1, scalar_1 + off); RW(WRFGPU_SPECIES_BASE, scalar_2 + off);
    R(WRFGPU_ADVECT_TEND, advect_tend);
    if (sc_tend) R(WRFGPU_H_DIABATIC, sc_tend + off);
    else c.zero_ids.push_back(WRFGPU_H_DIABATIC);
    R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty); R(WRFGPU_C1H, c1); R(WRFGPU_C2H, c2);
    R(WRFGPU_MU_1, mu_old); R(WRFGPU_MU_2, mu_new); R(WRFGPU_MUB, mu_base);
    int rc = wrfgpu::fortran_call(c);
    if (rc) return rc;
  }
  return WRFGPU_OK;
}

int wrfgpu_rk_update_scalar_pd(const int* scs, const int* sce, float* scalar, float* sc_tend, const float* c1,
                               const float* c2, const float* mu_old, const float* mu_new, const float* mu_base,
                               const int* rk_step, const float* dt, const int* spec_zone,
                               const WrfDynConfig* config_flags, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !scs || !sce || !rk_step || !dt || !scalar || !sc_tend || *sce < *scs)
    return WRFGPU_E_ARG;
  (void)spec_zone;
  const size_t n3 = (size_t)(*ime - *ims + 1) * (size_t)(*kme - *kms + 1) * (size_t)(*jme - *jms + 1);
  for (int im = *scs; im <= *sce; ++im) {
    const size_t off = (size_t)(im - *scs) * n3;
    FCall c;
    set_dims(c, DIMS);
    c.cfg = *config_flags; c.routine = 131; c.rk_step = *rk_step; c.dtrk = *dt;
    RW(WRFGPU_SPECIES_BASE + 1, scalar + off); RW(WRFGPU_H_DIABATIC, sc_tend + off);
    R(WRFGPU_C1H, c1); R(WRFGPU_C2H, c2);
    R(WRFGPU_MU_1, mu_old); R(WRFGPU_MU_2, mu_new); R(WRFGPU_MUB, mu_base);
    int rc = wrfgpu::fortran_call(c);
    if (rc) return rc;
  }
  return WRFGPU_OK;
}

int wrfgpu_rk_addtend_dry(float* ru_tend, float* rv_tend, float* rw_tend, float* ph_tend, float* t_tend,
                          float* ru_tendf, float* rv_tendf, float* rw_tendf, float* ph_tendf, float* t_tendf,
                          const float* u_save, const float* v_save, const float* w_save, const float* ph_save,
                          const float* t_save, float* mu_tend, float* mu_tendf, const int* rk_step,
                          const float* c1, const float* c2, const float* h_diabatic, const float* mut,
                          const float* msftx, const float* msfty, const float* msfux, const float* msfuy,
                          const float* msfvx, const float* msfvx_inv, const float* msfvy, const int* ids,
                          const int* ide, const int* jds, const int* jde, const int* kds, const int* kde,
                          const int* ims, const int* ime, const int* jms, const int* jme, const int* kms,
                          const int* kme, const int* ips, const int* ipe, const int* jps, const int* jpe,
                          const int* kps, const int* kpe, const int* its, const int* ite, const int* jts,
                          const int* jte, const int* kts, const int* kte) {
  if (!rk_step || !ips || !ipe || !jps || !jpe || !kps || !kpe || !ids || !ide || !jds || !jde || !kds || !kde)
    return WRFGPU_E_ARG;
  // one patch covering the domain
  if (*ips != *ids || *ipe != *ide || *jps != *jds || *jpe != *jde || *kps != *kds || *kpe != *kde)
    return WRFGPU_E_ARG;
  (void)msftx; (void)msfux; (void)msfvy;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = default_cfg(0); c.cfg.damp_opt = 2; c.cfg.zdamp = 1.f;  // a configuration that stores ru_tendf ..
  c.routine = 134; c.rk_step = *rk_step;
  RW(WRFGPU_RU_TEND, ru_tend); RW(WRFGPU_RV_TEND, rv_tend); RW(WRFGPU_RW_TEND, rw_tend);
  RW(WRFGPU_PH_TEND, ph_tend); RW(WRFGPU_T_TEND, t_tend);
  RW(WRFGPU_RU_TENDF, ru_tendf); RW(WRFGPU_RV_TENDF, rv_tendf); RW(WRFGPU_RW_TENDF, rw_tendf);
  RW(WRFGPU_ADVECT_TEND, ph_tendf); RW(WRFGPU_T_TENDF, t_tendf);
  R(WRFGPU_U_SAVE, u_save); R(WRFGPU_V_SAVE, v_save); R(WRFGPU_W_SAVE, w_save); R(WRFGPU_PH_SAVE, ph_save);
  R(WRFGPU_T_SAVE, t_save); RW(WRFGPU_MU_TEND, mu_tend); RW(WRFGPU_MUDF, mu_tendf);
  R(WRFGPU_C1H, c1); R(WRFGPU_C2H, c2); R(WRFGPU_H_DIABATIC, h_diabatic); R(WRFGPU_MUT, mut);
  R(WRFGPU_MSFTY, msfty); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
  if (!ru_tend || !rv_tend || !rw_tend || !ph_tend || !t_tend || !ru_tendf || !rv_tendf || !rw_tendf || !ph_tendf ||
      !t_tendf || !u_save || !v_save || !w_save || !ph_save || !t_save || !mu_tend || !mu_tendf || !c1 || !c2 ||
      !h_diabatic || !mut || !msfty || !msfuy || !msfvx || !msfvx_inv)
    return WRFGPU_E_ARG;
  return wrfgpu::fortran_call(c);
}

int wrfgpu_rk_scalar_tend(const int* scs, const int* sce, const WrfDynConfig* config_flags, const int* tenddec,
                          const int* rk_step, const float* dt_step, const float* ru, const float* rv,
                          const float* ww, const float* wwE, const float* wwI, const float* u_old,
                          const float* v_old, const float* mut, const float* mub, const float* mu_old,
                          const float* c1h, const float* c2h, const float* c1f, const float* c2f,
                          const float* alt, const float* scalar_old, const float* scalar, float* scalar_tends,
                          float* advect_tend, float* h_tendency, float* z_tendency, const float* RQVFTEN,
                          const float* base, const int* moist_step, const float* fnm, const float* fnp,
                          const float* msfux, const float* msfuy, const float* msfvx, const float* msfvx_inv,
                          const float* msfvy, const float* msftx, const float* msfty, const float* rdx,
                          const float* rdy, const float* rdn, const float* rdnw, const float* khdif,
                          const float* kvdif, const float* xkmhd, const int* diff_6th_opt,
                          const float* diff_6th_factor, const int* adv_opt, const float* phb, const float* ph,
                          const int* mix2_off, const int* mix6_off, WRFGPU_DIMS_ARGS) {
  if (cfg_ok(config_flags) || !scs || !sce || !rk_step || !dt_step || !rdx || !rdy || !adv_opt || !scalar ||
      !scalar_old || !advect_tend || (tenddec && *tenddec) || *sce < *scs)
    return WRFGPU_E_ARG;
  // the schemes of this path: 0 (5th/3rd order) and 1 (positive definite)
  if (*adv_opt != 0 && *adv_opt != 1) return WRFGPU_E_ARG;
  // IEVA off (wwI unused), no cumulus moisture tendency (RQVFTEN), tenddec
  // off (h_tendency, z_tendency); the explicit diffusion reads khdif, kvdif,
  // alt, rdn, rdnw and (qv) base
  (void)ww; (void)wwI; (void)u_old; (void)v_old; (void)c1f; (void)c2f; (void)h_tendency;
  (void)z_tendency; (void)RQVFTEN; (void)ph;
  const int one = 1;
  const size_t ni = (size_t)(*ime - *ims + 1), nk = (size_t)(*kme - *kms + 1);
  const size_t n3 = ni * nk * (size_t)(*jme - *jms + 1);
  for (int im = *scs; im <= *sce; ++im) {
    const size_t off = (size_t)(im - *scs) * n3;
    // zero_tend (module_big_step_utilities_em.F:4573): the tile, kts..kte
    for (int j = *jts; j <= *jte; ++j)
      for (int k = *kts; k <= *kte; ++k)
        for (int i = *its; i <= *ite; ++i)
          advect_tend[(size_t)(i - *ims) + ni * ((size_t)(k - *kms) + nk * (size_t)(j - *jms))] = 0.f;
    int rc;
    if (*rk_step == config_flags->rk_ord && *adv_opt == 1)
      rc = wrfgpu_advect_scalar_pd(scalar + off, scalar_old + off, advect_tend, nullptr, nullptr, ru, rv, wwE, c1h,
                                   c2h, mut, mub, mu_old, &one, config_flags, nullptr, msfux, msfuy, msfvx, msfvy,
                                   msftx, msfty, fnm, fnp, rdx, rdy, rdnw, dt_step, DIMS);
    else
      rc = wrfgpu_advect_scalar(scalar + off, scalar + off, advect_tend, ru, rv, wwE, c1h, c2h, mut, &one,
                                config_flags, msfux, msfuy, msfvx, msfvy, msftx, msfty, fnm, fnp, rdx, rdy, rdnw,
                                DIMS);
    if (rc) return rc;
    const int d6 = diff_6th_opt ? *diff_6th_opt : 0;
    const bool on6 = d6 != 0 && !(mix6_off && *mix6_off);
    const bool on2 = config_flags->diff_opt == 1 && !(mix2_off && *mix2_off);
    if (*rk_step == 1 && (on2 || on6)) {  // module_em.F:1378-1435
      if (!scalar_tends || !mut || !c1h || !c2h) return WRFGPU_E_ARG;
      if (on6 && (!phb || !diff_6th_factor)) return WRFGPU_E_ARG;
      const bool qv = moist_step && *moist_step && im == WRFGPU_P_QV;
      if (on2) {
        if (!khdif || !kvdif || !alt || !rdn || !rdnw || (qv && !base)) return WRFGPU_E_ARG;
        // km_opt = 1 (isotropic_km): the coefficient array holds khdif / prandtl
        if (xkmhd && xkmhd[(size_t)(*its - *ims) + ni * ((size_t)(*kts - *kms) + nk * (size_t)(*jts - *jms))] !=
                         *khdif / (1.f / 3.0f))
          return WRFGPU_E_ARG;
      }
      FCall c;
      set_dims(c, DIMS);
      c.cfg = *config_flags; c.cfg.diff_6th_opt = on6 ? d6 : 0;
      if (on6) c.cfg.diff_6th_factor = *diff_6th_factor;
      c.cfg.moist_mix2_off = c.cfg.scalar_mix2_off = on2 ? 0 : 1;
      c.cfg.moist_mix6_off = c.cfg.scalar_mix6_off = on6 ? 0 : 1;
      if (on2) { c.cfg.khdif = *khdif; c.cfg.kvdif = *kvdif; }
      c.routine = 132; c.rk_step = 1; c.iteration = qv ? 1 : 0;
      c.dtrk = *dt_step; c.rdx = *rdx; c.rdy = *rdy;
      R(WRFGPU_SPECIES_BASE, scalar + off); RW(WRFGPU_H_DIABATIC, scalar_tends + off);
      R(WRFGPU_MUTS, mut); R(WRFGPU_C1H, c1h); R(WRFGPU_C2H, c2h);
      R(WRFGPU_MSFUX, msfux); R(WRFGPU_MSFUY, msfuy); R(WRFGPU_MSFVX, msfvx); R(WRFGPU_MSFVX_INV, msfvx_inv);
      R(WRFGPU_MSFVY, msfvy); R(WRFGPU_MSFTX, msftx); R(WRFGPU_MSFTY, msfty);
      if (on6) R(WRFGPU_PHB, phb);
      if (on2) {
        R(WRFGPU_ALT, alt); R(WRFGPU_RDN, rdn); R(WRFGPU_RDNW, rdnw);
        if (qv) R(WRFGPU_QV_BASE, base);
      }
      rc = wrfgpu::fortran_call(c);
      if (rc) return rc;
    }
  }
  return WRFGPU_OK;
}

int wrfgpu_calc_p_rho_phi(const float* moist, const int* n_moist, const int* hypsometric_opt, float* al,
                          const float* alb, const float* mu, const float* muts, const float* c1, const float* c2,
                          const float* c3h, const float* c4h, const float* c3f, const float* c4f, const float* ph,
                          const float* phb, float* p, const float* pb, const float* t, const float* p0,
                          const float* t0, const float* ptop, const float* znu, const float* znw, const float* dnw,
                          const float* rdnw, const float* rdn, const int* non_hydrostatic, const int* use_theta_m,
                          WRFGPU_DIMS_ARGS) {
  if (!n_moist || *n_moist != 1 || !hypsometric_opt || !ptop || !non_hydrostatic || !*non_hydrostatic ||
      !use_theta_m || (p0 && *p0 != 100000.f) || (t0 && *t0 != 300.f))
    return WRFGPU_E_ARG;
  (void)znu; (void)znw; (void)dnw; (void)rdn;
  FCall c;
  set_dims(c, DIMS);
  c.cfg = default_cfg(0); c.cfg.hypsometric_opt = *hypsometric_opt; c.cfg.use_theta_m = *use_theta_m;
  c.routine = WRFGPU_R_CALC_P_RHO_PHI; c.p_top = *ptop;
  R(WRFGPU_SPECIES_BASE, moist); RW(WRFGPU_AL, al); R(WRFGPU_ALB, alb); R(WRFGPU_MU_2, mu); R(WRFGPU_MUTS, muts);
  R(WRFGPU_C1H, c1); R(WRFGPU_C2H, c2); bind_coefs34(c, c3h, c4h, c3f, c4f);
  R(WRFGPU_PH_2, ph); R(WRFGPU_PHB, phb); RW(WRFGPU_P, p); R(WRFGPU_PB, pb); R(WRFGPU_T_2, t);
  R(WRFGPU_RDNW, rdnw);
  return wrfgpu::fortran_call(c);
}

int wrfgpu_fortran_release(void) { return wrfgpu::fortran_release(); }

}  // extern "C"
