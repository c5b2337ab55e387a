// ORACLE — test infrastructure only (see wrf_oracle.hpp).
// Restatement of the physics-off large step of dyn_em/solve_em.F
// (:444-465 acoustic step count, :578-3459 RK3 loop, :4175-4205 final
// calc_p_rho_phi, :4439-4535 end-of-step boundary fills, :4735-4750
// set_w_surface), of rk_scalar_tend / rk_update_scalar / rk_update_scalar_pd
// (dyn_em/module_em.F:1096-1916) and of set_w_surface
// (dyn_em/module_bc_em.F:1196-1295).  OpenMP runs the reference's tile loops
// (set_tiles2 j-slabs); boundary fills run once per sync site, serially.
#pragma once
#include <map>
#include <string>
#include "wrf_oracle.hpp"
#include "oracle_bigstep.hpp"
#include "oracle_advect.hpp"
#include "oracle_small.hpp"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace wrforacle {

// module_em.F:1587-1799 rk_update_scalar.  sc_tend (:1700-1706) holds the
// stage-1 sixth-order diffusion of a diffused species; sc_tend_p is null for
// the others, whose sc_tend is zero (the "+ sc_tend" step then adds an exact
// zero and is left out).
template <typename R>
void rk_update_scalar(R* scalar_1_p, R* scalar_2_p, R* advect_tend_p, R* msfty_p, R* c1_p, R* c2_p, R* mu_old_p,
                      R* mu_new_p, R* mu_base_p, int rk_step, R dt, R* sc_tend_p, const Dims& d) {
  A3<R> scalar_1(scalar_1_p, d), scalar_2(scalar_2_p, d), advect_tend(advect_tend_p, d), sc_tend(sc_tend_p, d);
  A2<R> msfty(msfty_p, d), mu_old(mu_old_p, d), mu_new(mu_new_p, d), mu_base(mu_base_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const int i_end = std::min(d.ite, d.ide - 1), j_end = std::min(d.jte, d.jde - 1), k_end = std::min(d.kte, d.kde - 1);
  for (int j = d.jts; j <= j_end; ++j)
    for (int i = d.its; i <= i_end; ++i) {
      R muold = mu_old(i, j) + mu_base(i, j);
      R munew = mu_new(i, j) + mu_base(i, j);
      for (int k = d.kts; k <= k_end; ++k) {
        R tendency = advect_tend(i, k, j) * msfty(i, j);
        if (sc_tend_p) tendency = tendency + sc_tend(i, k, j);
        if (rk_step == 1) scalar_1(i, k, j) = scalar_2(i, k, j);
        scalar_2(i, k, j) = ((c1(k) * muold + c2(k)) * scalar_1(i, k, j) + dt * tendency) / (c1(k) * munew + c2(k));
      }
    }
}

// module_em.F:1803-1916 rk_update_scalar_pd: tendency = 0 + sc_tend (null:
// zero).  The reference then zeroes sc_tend (:1893); the caller passes null
// to the last stage's rk_update_scalar of these species instead.
template <typename R>
void rk_update_scalar_pd(R* scalar_p, R* c1_p, R* c2_p, R* mu_old_p, R* mu_new_p, R* mu_base_p, R dt, R* sc_tend_p,
                         const Dims& d) {
  A3<R> scalar(scalar_p, d), sc_tend(sc_tend_p, d);
  A2<R> mu_old(mu_old_p, d), mu_new(mu_new_p, d), mu_base(mu_base_p, d);
  A1<R> c1(c1_p, d), c2(c2_p, d);
  const int i_end = std::min(d.ite, d.ide - 1), j_end = std::min(d.jte, d.jde - 1), k_end = std::min(d.kte, d.kde - 1);
  for (int j = d.jts; j <= j_end; ++j)
    for (int i = d.its; i <= i_end; ++i) {
      R muold = mu_old(i, j) + mu_base(i, j);
      R munew = mu_new(i, j) + mu_base(i, j);
      for (int k = d.kts; k <= k_end; ++k) {
        R tendency = R(0.);
        if (sc_tend_p) tendency = tendency + sc_tend(i, k, j);
        scalar(i, k, j) = ((c1(k) * muold + c2(k)) * scalar(i, k, j) + dt * tendency) / (c1(k) * munew + c2(k));
      }
    }
}

// module_bc_em.F:1196-1295 set_w_surface (fill_w_flag = .false.).
template <typename R>
void set_w_surface(const WrfDynConfig& cf, R* w_p, R* ht_p, R* u_p, R* v_p, R cf1, R cf2, R cf3, R rdx, R rdy,
                   R* msftx_p, R* msfty_p, const Dims& d) {
  A3<R> w(w_p, d), u(u_p, d), v(v_p, d);
  A2<R> ht(ht_p, d), msftx(msftx_p, d), msfty(msfty_p, d);
  int jm1_limit = d.jds, jp1_limit = d.jde - 1, im1_limit = d.ids, ip1_limit = d.ide - 1;
  if (cf.periodic_x) { im1_limit = d.ids - 1; ip1_limit = d.ide; }
  if (cf.periodic_y) { jm1_limit = d.jds - 1; jp1_limit = d.jde; }
  for (int j = d.jts; j <= std::min(d.jte, d.jde - 1); ++j) {
    int jm1 = std::max(j - 1, jm1_limit), jp1 = std::min(j + 1, jp1_limit);
    for (int i = d.its; i <= std::min(d.ite, d.ide - 1); ++i) {
      int im1 = std::max(i - 1, im1_limit), ip1 = std::min(i + 1, ip1_limit);
      w(i, 1, j) = msfty(i, j) * R(.5) * rdy *
                       ((ht(i, jp1) - ht(i, j)) * (cf1 * v(i, 1, j + 1) + cf2 * v(i, 2, j + 1) + cf3 * v(i, 3, j + 1)) +
                        (ht(i, j) - ht(i, jm1)) * (cf1 * v(i, 1, j) + cf2 * v(i, 2, j) + cf3 * v(i, 3, j))) +
                   msftx(i, j) * R(.5) * rdx *
                       ((ht(ip1, j) - ht(i, j)) * (cf1 * u(i + 1, 1, j) + cf2 * u(i + 1, 2, j) + cf3 * u(i + 1, 3, j)) +
                        (ht(i, j) - ht(im1, j)) * (cf1 * u(i, 1, j) + cf2 * u(i, 2, j) + cf3 * u(i, 3, j)));
    }
  }
}

// Named fields of the domain state.  The order and names are those of the
// C-ABI field table (include/wrfgpu.h) shared by the GPU library.
template <typename R>
struct Domain {
  Dims d{};             // domain + memory dims; tile fields = whole patch
  WrfDynConfig cf{};
  WrfGpuScalars sc{};   // dt, dx, dy, rdx, rdy, cf1..cfn1, epssm, smdiv, emdiv, p_top
  int n_moist = 1, n_scalar = 0;
  std::vector<std::vector<R>> f3, f2, f1;   // indexed by WrfGpuFieldId ranges
  std::vector<std::vector<R>> qs;           // moist then passive: [2*s] current, [2*s+1] old
  std::vector<std::vector<R>> tendf;        // ru_tendf, rv_tendf, rw_tendf, t_tendf (diff_6th_opt != 0)
  std::vector<std::vector<R>> sctend;       // species' sc_tend (diff_6th_opt != 0)
  long n3 = 0, n2 = 0, n1 = 0;
  int nthreads = 1;
  R max_vert_cfl = 0, max_horiz_cfl = 0;

  void init(const WrfGpuDomainDesc& desc) {
    d.ids = 1; d.ide = desc.ide; d.jds = 1; d.jde = desc.jde; d.kds = 1; d.kde = desc.kde;
    d.ims = d.ids - WRFGPU_HALO; d.ime = d.ide + WRFGPU_HALO;
    d.jms = d.jds - WRFGPU_HALO; d.jme = d.jde + WRFGPU_HALO;
    d.kms = 1; d.kme = d.kde;
    d.its = d.ids; d.ite = d.ide; d.jts = d.jds; d.jte = d.jde; d.kts = d.kds; d.kte = d.kde;
    cf = desc.config; sc = desc.scalars;
    n_moist = desc.n_moist; n_scalar = desc.n_scalar;
    if (n_moist != 1) throw std::runtime_error("the physics-off path carries exactly one moist species (qv)");
    check_config(cf);
    n3 = (long)(d.ime - d.ims + 1) * (d.kme - d.kms + 1) * (d.jme - d.jms + 1);
    n2 = (long)(d.ime - d.ims + 1) * (d.jme - d.jms + 1);
    n1 = (long)(d.kme - d.kms + 1);
    f3.assign(WRFGPU_N3D, std::vector<R>(n3, R(0)));
    f2.assign(WRFGPU_N2D, std::vector<R>(n2, R(0)));
    f1.assign(WRFGPU_N1D, std::vector<R>(n1, R(0)));
    qs.assign(2 * (n_moist + n_scalar), std::vector<R>(n3, R(0)));
    const bool diff1 = cf.diff_opt == 1, diff6 = cf.diff_6th_opt != 0;
    tendf.assign(diff1 || diff6 || cf.damp_opt == 2 ? 4 : 0, std::vector<R>(n3, R(0)));
    sctend.assign(diff1 || diff6 ? n_moist + n_scalar : 0, std::vector<R>(n3, R(0)));
  }
  // species s's explicit (diff_opt = 1) and sixth-order diffusion switches
  bool mix2(int s) const { return cf.diff_opt == 1 && !(s < n_moist ? cf.moist_mix2_off : cf.scalar_mix2_off); }
  bool mix6(int s) const { return cf.diff_6th_opt != 0 && !(s < n_moist ? cf.moist_mix6_off : cf.scalar_mix6_off); }
  // species s's sc_tend, or null where it is not diffused
  R* sct_of(int s) { return mix2(s) || mix6(s) ? sctend[s].data() : nullptr; }
  R* p3(int id) { return f3[id].data(); }
  R* p2(int id) { return f2[id - WRFGPU_F2D_BASE].data(); }
  R* p1(int id) { return f1[id - WRFGPU_F1D_BASE].data(); }
  R* q(int s) { return qs[2 * s].data(); }
  R* qold(int s) { return qs[2 * s + 1].data(); }

  // Field access by C-ABI id (scalar species are WRFGPU_SPECIES_BASE + 2*s (+1 old)).
  R* field(int id, long* n) {
    if (id >= 0 && id < WRFGPU_N3D) { *n = n3; return p3(id); }
    if (id >= WRFGPU_F2D_BASE && id < WRFGPU_F2D_BASE + WRFGPU_N2D) { *n = n2; return p2(id); }
    if (id >= WRFGPU_F1D_BASE && id < WRFGPU_F1D_BASE + WRFGPU_N1D) { *n = n1; return p1(id); }
    if (id >= WRFGPU_SPECIES_BASE && id < WRFGPU_SPECIES_BASE + 2 * (n_moist + n_scalar)) {
      *n = n3; return qs[id - WRFGPU_SPECIES_BASE].data();
    }
    if (id >= WRFGPU_RU_TENDF && id <= WRFGPU_T_TENDF && !tendf.empty()) {
      *n = n3; return tendf[id - WRFGPU_RU_TENDF].data();
    }
    *n = 0; return nullptr;
  }

  // The reference's OpenMP tile loop: j-slab tiles of the single patch.
  template <typename F> void tiles(F fn) {
    int nt = std::max(1, std::min(nthreads, d.jde - d.jds));
    if (nt == 1) { fn(d); return; }
    int ny = d.jde - d.jds;  // mass rows jds..jde-1; the last tile also owns jde
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int t = 0; t < nt; ++t) {
      Dims td = d;
      td.jts = d.jds + (int)((long)ny * t / nt);
      td.jte = (t == nt - 1) ? d.jde : d.jds + (int)((long)ny * (t + 1) / nt) - 1;
      fn(td);
    }
  }
  void bc3(int id, char var) { set_physical_bc3d(p3(id), var, cf, d); }
  void bc3p(R* p, char var) { set_physical_bc3d(p, var, cf, d); }
  void bc2(int id, char var) { set_physical_bc2d(p2(id), var, cf, d); }

  int num_sound_steps() const {
    if (cf.time_step_sound != 0) return cf.time_step_sound;
    R spacing = std::min(R(sc.dx), R(sc.dy));
    return std::max(2 * ((int)(R(300.) * R(sc.dt) / spacing - R(0.01)) + 1), 4);
  }

  // rk_tendency's forward step at stage 1 (module_em.F:801-944): the explicit
  // diffusion (diff_opt = 1, km_opt = 1), the sixth-order diffusion and the
  // Rayleigh damping (damp_opt = 2) of the stage-1 state added to ru_tendf,
  // rv_tendf, rw_tendf and t_tendf (t0 .. t3) over tile td, dt the large step.
  void forward_terms(R* t0, R* t1, R* t2, R* t3, R dt, const Dims& td) {
    const bool diff1 = cf.diff_opt == 1, diff6 = cf.diff_6th_opt != 0, damp2 = cf.damp_opt == 2;
    const R rdx = R(sc.rdx), rdy = R(sc.rdy);
    if (diff1) {
      // module_em.F:801-877: explicit diffusion with the constant coefficients
      // of km_opt = 1 (xkmh = khdif, xkhh = khdif / prandtl; theta's vertical
      // coefficient 3 kvdif)
      const R khdif = (R)cf.khdif, kvdif = (R)cf.kvdif, prandtl = R(1.) / R(3.0);
      const R xkmh = khdif, xkhh = khdif / prandtl;
      horizontal_diffusion(cf, 'u', p3(WRFGPU_U_2), t0, p2(WRFGPU_MUT), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                           p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV),
                           p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), xkmh, rdx, rdy, td);
      horizontal_diffusion(cf, 'v', p3(WRFGPU_V_2), t1, p2(WRFGPU_MUT), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                           p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV),
                           p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), xkmh, rdx, rdy, td);
      horizontal_diffusion(cf, 'w', p3(WRFGPU_W_2), t2, p2(WRFGPU_MUT), p1(WRFGPU_C1F), p1(WRFGPU_C2F),
                           p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV),
                           p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), xkmh, rdx, rdy, td);
      horizontal_diffusion_3dmp(cf, p3(WRFGPU_T_2), t3, p2(WRFGPU_MUT), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                                p3(WRFGPU_T_INIT), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX_INV),
                                p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), xkhh, rdx, rdy, td);
      vertical_diffusion(cf, 'u', p3(WRFGPU_U_2), t0, p1(WRFGPU_U_BASE), (R*)nullptr, p1(WRFGPU_C1H),
                         p1(WRFGPU_C2H), p3(WRFGPU_ALT), p2(WRFGPU_MUU), p1(WRFGPU_RDN), p1(WRFGPU_RDNW), kvdif, td);
      vertical_diffusion(cf, 'v', p3(WRFGPU_V_2), t1, p1(WRFGPU_V_BASE), (R*)nullptr, p1(WRFGPU_C1H),
                         p1(WRFGPU_C2H), p3(WRFGPU_ALT), p2(WRFGPU_MUV), p1(WRFGPU_RDN), p1(WRFGPU_RDNW), kvdif, td);
      vertical_diffusion(cf, 'w', p3(WRFGPU_W_2), t2, (R*)nullptr, (R*)nullptr, p1(WRFGPU_C1F),
                         p1(WRFGPU_C2F), p3(WRFGPU_ALT), p2(WRFGPU_MUT), p1(WRFGPU_RDN), p1(WRFGPU_RDNW), kvdif, td);
      vertical_diffusion(cf, 't', p3(WRFGPU_T_2), t3, (R*)nullptr, p3(WRFGPU_T_INIT), p1(WRFGPU_C1H),
                         p1(WRFGPU_C2H), p3(WRFGPU_ALT), p2(WRFGPU_MUT), p1(WRFGPU_RDN), p1(WRFGPU_RDNW),
                         R(3.) * kvdif, td);
    }
    if (diff6) {
      // module_em.F:879-932, with the state of stage 1
      const int fld[4] = {WRFGPU_U_2, WRFGPU_V_2, WRFGPU_W_2, WRFGPU_T_2};
      const char nm[4] = {'u', 'v', 'w', 'm'};
      for (int q = 0; q < 4; ++q) {
        const bool wl = q == 2;  // w sits on full levels
        R* tt[4] = {t0, t1, t2, t3};
        sixth_order_diffusion(nm[q], p3(fld[q]), tt[q], p2(WRFGPU_MUT), dt, cf,
                              p1(wl ? WRFGPU_C1F : WRFGPU_C1H), p1(wl ? WRFGPU_C2F : WRFGPU_C2H), p3(WRFGPU_PHB),
                              rdx, rdy, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                              p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), td);
      }
    }
    if (damp2)  // module_em.F:933-944
      rk_rayleigh_damp(t0, t1, t2, t3, p3(WRFGPU_U_2),
                       p3(WRFGPU_V_2), p3(WRFGPU_W_2), p3(WRFGPU_T_2), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                       p1(WRFGPU_C1F), p1(WRFGPU_C2F), p2(WRFGPU_MUT), p2(WRFGPU_MUU), p2(WRFGPU_MUV),
                       p3(WRFGPU_PH_2), p3(WRFGPU_PHB), p1(WRFGPU_U_BASE), p1(WRFGPU_V_BASE), p1(WRFGPU_T_BASE),
                       p1(WRFGPU_Z_BASE), (R)cf.dampcoef, (R)cf.zdamp, td);
  }

  // One large step (solve_em.F:444-4750, physics off).
  void solve_em_step() {
    using KR = K<R>;
    const R dt = R(sc.dt), rdx = R(sc.rdx), rdy = R(sc.rdy);
    const R cf1 = R(sc.cf1), cf2 = R(sc.cf2), cf3 = R(sc.cf3), cfn = R(sc.cfn), cfn1 = R(sc.cfn1);
    const R epssm = R(sc.epssm), smdiv = R(sc.smdiv), emdiv = R(sc.emdiv), p_top = R(sc.p_top);
    const int rk_order = cf.rk_ord;
    const int ns_total = num_sound_steps();
    const R dts = dt / R(ns_total);
    R mvc = 0, mhc = 0;
    const int nsp = n_moist + n_scalar;

    // initialize_moist_old (solve_em.F:517-527) + its 'p' fill.
    tiles([&](const Dims& td) {
      A3<R> mo(qold(0), td), m(q(0), td);
      for (int j = td.jts; j <= std::min(td.jte, td.jde - 1); ++j)
        for (int k = td.kts; k <= td.kte - 1; ++k)
          for (int i = td.its; i <= std::min(td.ite, td.ide - 1); ++i) mo(i, k, j) = m(i, k, j);
    });
    bc3p(qold(0), 'p');

    for (int rk_step = 1; rk_step <= rk_order; ++rk_step) {
      R dt_rk, dts_rk; int nsmall;
      if (rk_step == 1) { dt_rk = dt / R(3.); dts_rk = dt_rk; nsmall = 1; }
      else if (rk_step == 2) { dt_rk = R(0.5) * dt; dts_rk = dts; nsmall = ns_total / 2; }
      else { dt_rk = dt; dts_rk = dts; nsmall = ns_total; }

      tiles([&](const Dims& td) {
        rk_step_prep(cf, rk_step, p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_W_2), p3(WRFGPU_T_2), p3(WRFGPU_PH_2),
                     p2(WRFGPU_MU_2), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F), p1(WRFGPU_C2F), q(0), n_moist,
                     p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_RW), p3(WRFGPU_WW), p3(WRFGPU_PHP), p3(WRFGPU_ALT),
                     p2(WRFGPU_MUU), p2(WRFGPU_MUV), p2(WRFGPU_MUB), p2(WRFGPU_MUT), p3(WRFGPU_PHB), p3(WRFGPU_PB),
                     p3(WRFGPU_P), p3(WRFGPU_AL), p3(WRFGPU_ALB), p3(WRFGPU_CQU), p3(WRFGPU_CQV), p3(WRFGPU_CQW),
                     p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY),
                     p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_DNW), rdx, rdy, td);
      });
      // rk_phys_bc_dry_1 (module_bc_em.F:960-1041) + al, ph_2 (solve_em.F:726-754)
      bc3(WRFGPU_RU, 'u'); bc3(WRFGPU_RV, 'v'); bc3(WRFGPU_RW, 'w'); bc3(WRFGPU_WW, 'w'); bc3(WRFGPU_PHP, 'w');
      bc3(WRFGPU_ALT, 't'); bc3(WRFGPU_P, 'p');
      bc2(WRFGPU_MUU, 'u'); bc2(WRFGPU_MUV, 'v'); bc2(WRFGPU_MUT, 't');
      bc3(WRFGPU_AL, 'p'); bc3(WRFGPU_PH_2, 'w');

      // rk_tendency (module_em.F:370-781); rk_addtend_dry then adds the
      // forward-in-time tendencies formed at stage 1 (the sixth-order
      // diffusion; zero physics tendencies otherwise).
      std::vector<R> tmv(64, R(0)), tmh(64, R(0));
      const bool diff6 = cf.diff_6th_opt != 0, damp2 = cf.damp_opt == 2, diff1 = cf.diff_opt == 1;
      if ((diff1 || diff6 || damp2) && rk_step == 1)
        for (auto& t : tendf) std::fill(t.begin(), t.end(), R(0));
      tiles([&](const Dims& td) {
        zero_tend(p3(WRFGPU_RU_TEND), td); zero_tend(p3(WRFGPU_RV_TEND), td); zero_tend(p3(WRFGPU_RW_TEND), td);
        zero_tend(p3(WRFGPU_T_TEND), td); zero_tend(p3(WRFGPU_PH_TEND), td);
        zero_tend(p3(WRFGPU_U_SAVE), td); zero_tend(p3(WRFGPU_V_SAVE), td); zero_tend(p3(WRFGPU_W_SAVE), td);
        zero_tend(p3(WRFGPU_PH_SAVE), td); zero_tend(p3(WRFGPU_T_SAVE), td);
        zero_tend2d(p2(WRFGPU_MU_TEND), td); zero_tend2d(p2(WRFGPU_MU_SAVE), td);
        advect_u(p3(WRFGPU_U_2), p3(WRFGPU_U_2), p3(WRFGPU_RU_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
                 p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                 p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM),
                 p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW), td);
        advect_v(p3(WRFGPU_V_2), p3(WRFGPU_V_2), p3(WRFGPU_RV_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
                 p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                 p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM),
                 p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW), td);
        advect_w(p3(WRFGPU_W_2), p3(WRFGPU_W_2), p3(WRFGPU_RW_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_WW),
                 p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                 p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM),
                 p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDN), td);
        advect_scalar(p3(WRFGPU_T_2), p3(WRFGPU_T_2), p3(WRFGPU_T_TEND), p3(WRFGPU_RU), p3(WRFGPU_RV),
                      p3(WRFGPU_WW), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUT), cf, p2(WRFGPU_MSFUX),
                      p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY),
                      p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW), td);
        rhs_ph(p3(WRFGPU_PH_TEND), p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_WW), p3(WRFGPU_PH_2), p3(WRFGPU_PH_2),
               p3(WRFGPU_PHB), p3(WRFGPU_W_2), p2(WRFGPU_MUT), p2(WRFGPU_MUU), p2(WRFGPU_MUV), p1(WRFGPU_C1F),
               p1(WRFGPU_C2F), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW), cfn, cfn1, rdx, rdy,
               p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY),
               p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), cf.non_hydrostatic, cf, td);
        horizontal_pressure_gradient(p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_PH_2), p3(WRFGPU_ALT),
                                     p3(WRFGPU_P), p3(WRFGPU_PB), p3(WRFGPU_AL), p3(WRFGPU_PHP), p3(WRFGPU_CQU),
                                     p3(WRFGPU_CQV), p2(WRFGPU_MUU), p2(WRFGPU_MUV), p2(WRFGPU_MU_2),
                                     p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW),
                                     cf1, cf2, cf3, cfn, cfn1, rdx, rdy, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                                     p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), cf,
                                     cf.non_hydrostatic, cf.top_lid, td);
        pg_buoy_w(p3(WRFGPU_RW_TEND), p3(WRFGPU_P), p3(WRFGPU_CQW), p2(WRFGPU_MU_2), p2(WRFGPU_MUB), p1(WRFGPU_C1F),
                  p1(WRFGPU_C2F), p1(WRFGPU_RDNW), p1(WRFGPU_RDN), KR::g, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), td);
        R a = 0, b = 0;
        w_damp_cfl(p3(WRFGPU_RW_TEND), p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_WW), p3(WRFGPU_W_2), p2(WRFGPU_MUT),
                   p1(WRFGPU_C1F), p1(WRFGPU_C2F), p1(WRFGPU_RDNW), rdx, rdy, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFVY), dt, cf,
                   &a, &b, td);
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        if (tid < 64) { tmv[tid] = std::max(tmv[tid], a); tmh[tid] = std::max(tmh[tid], b); }
        coriolis(p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_RW), p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND),
                 p3(WRFGPU_RW_TEND), cf, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                 p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_F), p2(WRFGPU_E), p2(WRFGPU_SINA), p2(WRFGPU_COSA),
                 p1(WRFGPU_FNM), p1(WRFGPU_FNP), td);
        curvature(p3(WRFGPU_RU), p3(WRFGPU_RV), p3(WRFGPU_RW), p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_W_2),
                  p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_RW_TEND), cf, p2(WRFGPU_MSFUX),
                  p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY),
                  (R*)nullptr, p1(WRFGPU_FNM), p1(WRFGPU_FNP), rdx, rdy, td);
        if (rk_step == 1 && (diff1 || diff6 || damp2))
          forward_terms(tendf[0].data(), tendf[1].data(), tendf[2].data(), tendf[3].data(), dt, td);
      });
      for (int t = 0; t < 64; ++t) { mvc = std::max(mvc, tmv[t]); mhc = std::max(mhc, tmh[t]); }
      if (diff1 || diff6 || damp2)
        tiles([&](const Dims& td) {
          rk_addtend_dry(p3(WRFGPU_RU_TEND), p3(WRFGPU_RV_TEND), p3(WRFGPU_RW_TEND), p3(WRFGPU_T_TEND),
                         tendf[0].data(), tendf[1].data(), tendf[2].data(), tendf[3].data(), p1(WRFGPU_C1H),
                         p1(WRFGPU_C2H), p2(WRFGPU_MUT), p2(WRFGPU_MSFTY), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX_INV), td);
        });

      tiles([&](const Dims& td) {
        small_step_prep(p3(WRFGPU_U_1), p3(WRFGPU_U_2), p3(WRFGPU_V_1), p3(WRFGPU_V_2), p3(WRFGPU_W_1),
                        p3(WRFGPU_W_2), p3(WRFGPU_T_1), p3(WRFGPU_T_2), p3(WRFGPU_PH_1), p3(WRFGPU_PH_2),
                        p2(WRFGPU_MUB), p2(WRFGPU_MU_1), p2(WRFGPU_MU_2), p2(WRFGPU_MUU), p2(WRFGPU_MUUS),
                        p2(WRFGPU_MUV), p2(WRFGPU_MUVS), p2(WRFGPU_MUT), p2(WRFGPU_MUTS), p2(WRFGPU_MUDF),
                        p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F), p1(WRFGPU_C2F), p3(WRFGPU_U_SAVE),
                        p3(WRFGPU_V_SAVE), p3(WRFGPU_W_SAVE), p3(WRFGPU_T_SAVE), p3(WRFGPU_PH_SAVE), p2(WRFGPU_MU_SAVE),
                        p3(WRFGPU_WW), p3(WRFGPU_WW1), p3(WRFGPU_C2A), p3(WRFGPU_PB), p3(WRFGPU_P), p3(WRFGPU_ALT),
                        p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFTY), rk_step, td);
        calc_p_rho(p3(WRFGPU_AL), p3(WRFGPU_P), p3(WRFGPU_PH_2), p3(WRFGPU_ALT), p3(WRFGPU_T_2), p3(WRFGPU_T_SAVE),
                   p3(WRFGPU_C2A), p3(WRFGPU_PM1), p2(WRFGPU_MU_2), p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                   KR::t0, p1(WRFGPU_RDNW), smdiv, cf.non_hydrostatic, 0, td);
        calc_coef_w(p3(WRFGPU_A), p3(WRFGPU_ALPHA), p3(WRFGPU_GAMMA), p2(WRFGPU_MUT), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                    p1(WRFGPU_C1F), p1(WRFGPU_C2F), p3(WRFGPU_CQW), p1(WRFGPU_RDN), p1(WRFGPU_RDNW), p3(WRFGPU_C2A),
                    dts_rk, KR::g, epssm, cf.top_lid, td);
      });
      // solve_em.F:1176-1264
      bc3(WRFGPU_RU_TEND, 'u'); bc3(WRFGPU_RV_TEND, 'v'); bc3(WRFGPU_PH_2, 'w'); bc3(WRFGPU_AL, 'p');
      bc3(WRFGPU_P, 'p'); bc3(WRFGPU_T_1, 'p'); bc3(WRFGPU_T_SAVE, 't');
      bc2(WRFGPU_MU_1, 't'); bc2(WRFGPU_MU_2, 't'); bc2(WRFGPU_MUDF, 't');

      for (int iteration = 1; iteration <= nsmall; ++iteration) {
        tiles([&](const Dims& td) {
          advance_uv(p3(WRFGPU_U_2), p3(WRFGPU_RU_TEND), p3(WRFGPU_V_2), p3(WRFGPU_RV_TEND), p3(WRFGPU_P),
                     p3(WRFGPU_PB), p3(WRFGPU_PH_2), p3(WRFGPU_PHP), p3(WRFGPU_ALT), p3(WRFGPU_AL), p2(WRFGPU_MU_2),
                     p2(WRFGPU_MUU), p3(WRFGPU_CQU), p2(WRFGPU_MUV), p3(WRFGPU_CQV), p2(WRFGPU_MUDF), p1(WRFGPU_C1H),
                     p1(WRFGPU_C2H), p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV),
                     p2(WRFGPU_MSFVY), rdx, rdy, dts_rk, cf1, cf2, cf3, p1(WRFGPU_FNM), p1(WRFGPU_FNP), emdiv,
                     p1(WRFGPU_RDNW), cf, cf.non_hydrostatic, cf.top_lid, td);
        });
        tiles([&](const Dims& td) {
          advance_mu_t(p3(WRFGPU_WW), p3(WRFGPU_WW1), p3(WRFGPU_U_2), p3(WRFGPU_U_SAVE), p3(WRFGPU_V_2),
                       p3(WRFGPU_V_SAVE), p2(WRFGPU_MU_2), p2(WRFGPU_MUT), p2(WRFGPU_MUAVE), p2(WRFGPU_MUTS),
                       p2(WRFGPU_MUU), p2(WRFGPU_MUV), p2(WRFGPU_MUDF), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p3(WRFGPU_T_2),
                       p3(WRFGPU_T_SAVE), p3(WRFGPU_T_2SAVE), p3(WRFGPU_T_TEND), p2(WRFGPU_MU_TEND), rdx, rdy, dts_rk,
                       epssm, p1(WRFGPU_DNW), p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW), p2(WRFGPU_MSFUX),
                       p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX),
                       p2(WRFGPU_MSFTY), cf, td);
        });
        tiles([&](const Dims& td) {
          advance_w(p3(WRFGPU_W_2), p3(WRFGPU_RW_TEND), p3(WRFGPU_WW), p3(WRFGPU_W_SAVE), p3(WRFGPU_U_2),
                    p3(WRFGPU_V_2), p2(WRFGPU_MU_2), p2(WRFGPU_MUT), p2(WRFGPU_MUAVE), p2(WRFGPU_MUTS),
                    p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F), p1(WRFGPU_C2F), p3(WRFGPU_T_2SAVE), p3(WRFGPU_T_2),
                    p3(WRFGPU_T_SAVE), p3(WRFGPU_PH_2), p3(WRFGPU_PH_SAVE), p3(WRFGPU_PHB), p3(WRFGPU_PH_TEND),
                    p2(WRFGPU_HT), p3(WRFGPU_C2A), p3(WRFGPU_CQW), p3(WRFGPU_ALT), p3(WRFGPU_ALB), p3(WRFGPU_A),
                    p3(WRFGPU_ALPHA), p3(WRFGPU_GAMMA), rdx, rdy, dts_rk, KR::t0, epssm, p1(WRFGPU_DNW),
                    p1(WRFGPU_FNM), p1(WRFGPU_FNP), p1(WRFGPU_RDNW), p1(WRFGPU_RDN), cf1, cf2, cf3, p2(WRFGPU_MSFTX),
                    p2(WRFGPU_MSFTY), cf, cf.top_lid, td);
        });
        tiles([&](const Dims& td) {
          sumflux(p3(WRFGPU_U_2), p3(WRFGPU_V_2), p3(WRFGPU_WW), p3(WRFGPU_U_SAVE), p3(WRFGPU_V_SAVE), p3(WRFGPU_WW1),
                  p2(WRFGPU_MUU), p2(WRFGPU_MUV), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p3(WRFGPU_RU_M), p3(WRFGPU_RV_M),
                  p3(WRFGPU_WW_M), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX_INV), iteration, nsmall, td);
          calc_p_rho(p3(WRFGPU_AL), p3(WRFGPU_P), p3(WRFGPU_PH_2), p3(WRFGPU_ALT), p3(WRFGPU_T_2),
                     p3(WRFGPU_T_SAVE), p3(WRFGPU_C2A), p3(WRFGPU_PM1), p2(WRFGPU_MU_2), p2(WRFGPU_MUTS),
                     p1(WRFGPU_C1H), p1(WRFGPU_C2H), KR::t0, p1(WRFGPU_RDNW), smdiv, cf.non_hydrostatic, iteration, td);
        });
        // solve_em.F:1659-1716
        bc3(WRFGPU_PH_2, 'w'); bc3(WRFGPU_AL, 'p'); bc3(WRFGPU_P, 'p');
        bc2(WRFGPU_MUTS, 't'); bc2(WRFGPU_MU_2, 't'); bc2(WRFGPU_MUDF, 't');
      }

      tiles([&](const Dims& td) {
        calc_mu_uv_1(cf, p2(WRFGPU_MUTS), p2(WRFGPU_MUUS), p2(WRFGPU_MUVS), td);
        small_step_finish(p3(WRFGPU_U_2), p3(WRFGPU_U_1), p3(WRFGPU_V_2), p3(WRFGPU_V_1), p3(WRFGPU_W_2),
                          p3(WRFGPU_W_1), p3(WRFGPU_T_2), p3(WRFGPU_T_1), p3(WRFGPU_PH_2), p3(WRFGPU_PH_1),
                          p3(WRFGPU_WW), p3(WRFGPU_WW1), p2(WRFGPU_MU_2), p2(WRFGPU_MU_1), p2(WRFGPU_MUT),
                          p2(WRFGPU_MUTS), p2(WRFGPU_MUU), p2(WRFGPU_MUUS), p2(WRFGPU_MUV), p2(WRFGPU_MUVS),
                          p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C1F), p1(WRFGPU_C2F), p3(WRFGPU_U_SAVE),
                          p3(WRFGPU_V_SAVE), p3(WRFGPU_W_SAVE), p3(WRFGPU_T_SAVE), p3(WRFGPU_PH_SAVE),
                          p2(WRFGPU_MU_SAVE), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFTY),
                          p3(WRFGPU_H_DIABATIC), nsmall, dts_rk, rk_step, rk_order, td);
      });
      if (rk_step == rk_order) {
        bc3(WRFGPU_RU_M, 'u'); bc3(WRFGPU_RV_M, 'v'); bc3(WRFGPU_WW_M, 'w');
        bc2(WRFGPU_MUT, 't'); bc2(WRFGPU_MUTS, 't');
      }
      // solve_em.F:1850-1960: physics tendencies (zero) into the old PD scalars.
      if (rk_step == rk_order) {
        for (int s = 0; s < nsp; ++s) {
          int adv = s < n_moist ? cf.moist_adv_opt : cf.scalar_adv_opt;
          if (adv != 1) continue;
          tiles([&](const Dims& td) {
            rk_update_scalar_pd(qold(s), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MU_1), p2(WRFGPU_MU_1),
                                p2(WRFGPU_MUB), dt_rk, sct_of(s), td);
          });
          bc3p(qold(s), 'p');
        }
      }
      // moist_variable_loop / scalar_variable_loop (solve_em.F:2198-2364, :2772-2955).
      for (int s = 0; s < nsp; ++s) {
        int adv = s < n_moist ? cf.moist_adv_opt : cf.scalar_adv_opt;
        R* sct = sct_of(s);
        if (sct && rk_step == 1) std::fill(sctend[s].begin(), sctend[s].end(), R(0));
        tiles([&](const Dims& td) {
          zero_tend(p3(WRFGPU_ADVECT_TEND), td);
          // rk_scalar_tend's stage-1 explicit diffusion (module_em.F:1378-1419; qv
          // against its base profile, coefficients khdif / prandtl and kvdif /
          // prandtl) and sixth-order diffusion (:1421-1435): muts and the stage's dt
          if (rk_step == 1 && mix2(s)) {
            const R prandtl = R(1.) / R(3.0);
            const R khdq = (R)cf.khdif / prandtl, kvdq = (R)cf.kvdif / prandtl;
            horizontal_diffusion(cf, 'm', q(s), sct, p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MSFUX),
                                 p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVX_INV), p2(WRFGPU_MSFVY),
                                 p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), khdq, rdx, rdy, td);
            vertical_diffusion(cf, s == 0 ? 'p' : 'm', q(s), sct, p1(WRFGPU_QV_BASE), (R*)nullptr, p1(WRFGPU_C1H),
                               p1(WRFGPU_C2H), p3(WRFGPU_ALT), p2(WRFGPU_MUTS), p1(WRFGPU_RDN), p1(WRFGPU_RDNW), kvdq,
                               td);
          }
          if (rk_step == 1 && mix6(s))
            sixth_order_diffusion('m', q(s), sct, p2(WRFGPU_MUTS), dt_rk, cf, p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                                  p3(WRFGPU_PHB), rdx, rdy, p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p2(WRFGPU_MSFUX),
                                  p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), td);
          if (rk_step == rk_order && adv == 1)
            advect_scalar_pd(q(s), qold(s), p3(WRFGPU_ADVECT_TEND), p3(WRFGPU_RU_M), p3(WRFGPU_RV_M),
                             p3(WRFGPU_WW_M), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUTS), p2(WRFGPU_MUB),
                             p2(WRFGPU_MU_1), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY), p2(WRFGPU_MSFVX),
                             p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM), p1(WRFGPU_FNP),
                             rdx, rdy, p1(WRFGPU_RDNW), dt_rk, td);
          else
            advect_scalar(q(s), q(s), p3(WRFGPU_ADVECT_TEND), p3(WRFGPU_RU_M), p3(WRFGPU_RV_M), p3(WRFGPU_WW_M),
                          p1(WRFGPU_C1H), p1(WRFGPU_C2H), p2(WRFGPU_MUTS), cf, p2(WRFGPU_MSFUX), p2(WRFGPU_MSFUY),
                          p2(WRFGPU_MSFVX), p2(WRFGPU_MSFVY), p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), p1(WRFGPU_FNM),
                          p1(WRFGPU_FNP), rdx, rdy, p1(WRFGPU_RDNW), td);
        });
        tiles([&](const Dims& td) {
          rk_update_scalar(qold(s), q(s), p3(WRFGPU_ADVECT_TEND), p2(WRFGPU_MSFTY), p1(WRFGPU_C1H), p1(WRFGPU_C2H),
                           p2(WRFGPU_MU_1), p2(WRFGPU_MU_2), p2(WRFGPU_MUB), rk_step, dt_rk,
                           (rk_step == rk_order && adv == 1) ? nullptr : sct, td);
        });
      }
      tiles([&](const Dims& td) {
        calc_p_rho_phi(q(0), n_moist, cf.hypsometric_opt, p3(WRFGPU_AL), p3(WRFGPU_ALB), p2(WRFGPU_MU_2),
                       p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C3H), p1(WRFGPU_C4H), p1(WRFGPU_C3F),
                       p1(WRFGPU_C4F), p3(WRFGPU_PH_2), p3(WRFGPU_PHB), p3(WRFGPU_P), p3(WRFGPU_PB), p3(WRFGPU_T_2),
                       KR::p0, KR::t0, p_top, p1(WRFGPU_ZNU), p1(WRFGPU_ZNW), p1(WRFGPU_DNW), p1(WRFGPU_RDNW),
                       p1(WRFGPU_RDN), cf.non_hydrostatic, cf.use_theta_m, td);
      });
      if (rk_step < rk_order) {
        // rk_phys_bc_dry_2 (module_bc_em.F:1045-1104) + species (solve_em.F:3258-3330)
        bc3(WRFGPU_U_2, 'U'); bc3(WRFGPU_V_2, 'V'); bc3(WRFGPU_W_2, 'w'); bc3(WRFGPU_T_2, 'p');
        bc3(WRFGPU_PH_2, 'w'); bc2(WRFGPU_MU_2, 't');
        for (int s = 0; s < nsp; ++s) bc3p(q(s), 'p');
      }
    }
    // solve_em.F:4180-4203 (repeats the stage-3 diagnosis; identical values)
    tiles([&](const Dims& td) {
      calc_p_rho_phi(q(0), n_moist, cf.hypsometric_opt, p3(WRFGPU_AL), p3(WRFGPU_ALB), p2(WRFGPU_MU_2),
                     p2(WRFGPU_MUTS), p1(WRFGPU_C1H), p1(WRFGPU_C2H), p1(WRFGPU_C3H), p1(WRFGPU_C4H), p1(WRFGPU_C3F),
                     p1(WRFGPU_C4F), p3(WRFGPU_PH_2), p3(WRFGPU_PHB), p3(WRFGPU_P), p3(WRFGPU_PB), p3(WRFGPU_T_2),
                     KR::p0, KR::t0, p_top, p1(WRFGPU_ZNU), p1(WRFGPU_ZNW), p1(WRFGPU_DNW), p1(WRFGPU_RDNW),
                     p1(WRFGPU_RDN), cf.non_hydrostatic, cf.use_theta_m, td);
    });
    // set_phys_bc_dry_2 (module_bc_em.F:808-908) + species (solve_em.F:4456-4530)
    bc3(WRFGPU_U_1, 'U'); bc3(WRFGPU_U_2, 'U'); bc3(WRFGPU_V_1, 'V'); bc3(WRFGPU_V_2, 'V');
    bc3(WRFGPU_W_1, 'w'); bc3(WRFGPU_W_2, 'w'); bc3(WRFGPU_T_1, 'p'); bc3(WRFGPU_T_2, 'p');
    bc3(WRFGPU_PH_1, 'w'); bc3(WRFGPU_PH_2, 'w'); bc2(WRFGPU_MU_1, 't'); bc2(WRFGPU_MU_2, 't');
    for (int s = 0; s < nsp; ++s) bc3p(q(s), 'p');
    tiles([&](const Dims& td) {
      set_w_surface(cf, p3(WRFGPU_W_2), p2(WRFGPU_HT), p3(WRFGPU_U_2), p3(WRFGPU_V_2), cf1, cf2, cf3, rdx, rdy,
                    p2(WRFGPU_MSFTX), p2(WRFGPU_MSFTY), td);
    });
    max_vert_cfl = mvc; max_horiz_cfl = mhc;
  }
};

}  // namespace wrforacle
