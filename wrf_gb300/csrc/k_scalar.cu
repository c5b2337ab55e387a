// Scalar transport and diagnosis kernels:
//   rk_update_scalar_pd  dyn_em/module_em.F:1803-1916 (physics tendency 0)
//   advect_scalar        dyn_em/module_advect_em.F:3394-3650, :4306-4333
//   advect_scalar_pd     dyn_em/module_advect_em.F:6505-6779, :7595-7645, limiter :7681-7781,
//                        divergence :7783-7883 — two passes: (1) per-cell limiter scale of
//                        every cell of the tile and its 1-cell halo into a scratch array,
//                        (2) per-cell divergence of the face fluxes, each face scaled by its
//                        upwind cell's factor (a face is only ever modified by its upwind
//                        cell, so the result does not depend on the reference's loop order)
//   rk_update_scalar     dyn_em/module_em.F:1587-1799
//   calc_p_rho_phi       dyn_em/module_big_step_utilities_em.F:953-1226 (non-hydrostatic)
//   set_w_surface        dyn_em/module_bc_em.F:1196-1295
// Roofline: HBM-bound; the limiter pass reads the 5 transport arrays twice
// (scale pass and divergence pass) plus the scale scratch.
#include "common.cuh"
#include "kernels.h"
#include "ffmath.h"
#include "open_adv.cuh"

namespace wrfgpu {

__device__ __forceinline__ bool mass_pt(const Mem& m, int i, int j) {
  return i >= m.its && i <= min(m.ite, m.ide - 1) && j >= m.jts && j <= min(m.jte, m.jde - 1);
}

// ------------------------------------------------------------ rk_update_scalar_pd
__global__ void __launch_bounds__(BX* BY) k_update_scalar_pd(Launch L, int rk_step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (!mass_pt(m, i, j) || k < m.kts || k > min(m.kte, m.kde - 1)) return;
  const Stage st = stage_of(m, rk_step);
  F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
  F2 mu1 = f2(m, WRFGPU_MU_1), mub = f2(m, WRFGPU_MUB);
  const float muold = mu1(i, j) + mub(i, j);
  const float munew = mu1(i, j) + mub(i, j);
  const float tendency = 0.f;
  for (int s = 0; s < m.nsp; ++s) {
    int adv = s < m.n_moist ? m.cf.moist_adv_opt : m.cf.scalar_adv_opt;
    if (adv != 1) continue;
    F3 q = f3p(m, m.qo[s]);
    q(i, k, j) = ((c1(k) * muold + c2(k)) * q(i, k, j) + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
  }
}

// Column form over mass tiles x level chunks (gridDim.y), species outermost,
// eight levels of loads in flight.
template <bool SCT>
__global__ void __launch_bounds__(TX* TY) k_update_scalar_pd_col(TileLaunch L, int rk_step) {
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  if (!mass_pt(m, i, j)) return;
  const int kts = m.kts, ktf = min(m.kte, m.kde - 1);
  const int per = (ktf - kts + 1 + (int)gridDim.y - 1) / (int)gridDim.y;
  const int k0 = kts + (int)blockIdx.y * per, k1 = min(ktf, k0 + per - 1);
  const Stage st = stage_of(m, rk_step);
  F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
  const float muold = f2(m, WRFGPU_MU_1)(i, j) + f2(m, WRFGPU_MUB)(i, j);
  const float munew = f2(m, WRFGPU_MU_1)(i, j) + f2(m, WRFGPU_MUB)(i, j);
  for (int s = 0; s < m.nsp; ++s) {
    int adv = s < m.n_moist ? m.cf.moist_adv_opt : m.cf.scalar_adv_opt;
    if (adv != 1) continue;
    F3 q = f3p(m, m.qo[s]);
    // tendency = 0 + sc_tend (the stage-1 sixth-order diffusion, if any);
    // the reference zeroes sc_tend here (:1893), so no later stage adds it
    float* sc = SCT ? sc_tend_of(m, s) : nullptr;
    if (sc == nullptr) {
      const float tendency = 0.f;
      chunked_levels<8, float>(
          k0, k1, [&](int k, float& v) { v = q(i, k, j); },
          [&](int k, const float& v) {
            q(i, k, j) = ((c1(k) * muold + c2(k)) * v + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
          });
    } else {
      F3 sct = f3p(m, sc);
      for (int k = k0; k <= k1; ++k) {
        float tendency = 0.f;
        tendency = tendency + sct(i, k, j);
        q(i, k, j) = ((c1(k) * muold + c2(k)) * q(i, k, j) + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
      }
    }
  }
}

// ------------------------------------------------------------ advect_scalar (+ zero_tend)
__device__ __forceinline__ bool pd_applies(const Mem& m, int species, int rk_step) {
  int adv = species < m.n_moist ? m.cf.moist_adv_opt : m.cf.scalar_adv_opt;
  return rk_step == m.cf.rk_ord && adv == 1;
}

// mode 0: always; mode 1: skip members whose species is advected by the
// positive-definite scheme at this stage (module_em.F:1265-1280).
__global__ void __launch_bounds__(BX* BY) k_advect_scalar(Launch L, int species, int rk_step, int mode) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (species >= m.nsp) return;
  const bool accum = (mode & 4) != 0;  // tendency += (routine-level callers)
  if ((mode & 3) == 1 && pd_applies(m, species, rk_step)) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  F3 tend = f3(m, WRFGPU_ADVECT_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte && k >= m.kts && k <= m.kte;
  const int ktf = min(m.kte, m.kde - 1);
  if (!(mass_pt(m, i, j) && k >= m.kts && k <= ktf)) {
    if (in_zero && !accum) tend(i, k, j) = 0.f;
    return;
  }
  const F3 fld = f3p(m, m.q[species]);
  const ScalarAdv a{fld, fld, f3(m, WRFGPU_RU_M), f3(m, WRFGPU_RV_M), f3(m, WRFGPU_WW_M), f2(m, WRFGPU_MSFTX),
                    f1(m, WRFGPU_FNM), f1(m, WRFGPU_FNP), f1(m, WRFGPU_RDNW)};
  tend(i, k, j) = adv_scalar_point(m, a, accum ? tend(i, k, j) : 0.f, i, j, k);
}

// ------------------------------------------------------------ advect_scalar_pd (open_adv.cuh)
// Pass 1: limiter scale of each cell of the tile + 1-cell halo (-1: not limited).
// mode 0: only members whose species uses the positive-definite scheme; mode 2: always.
__global__ void __launch_bounds__(BX* BY) k_pd_scale(Launch L, int species, int rk_step, int mode, float* const* scratch) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (species >= m.nsp) return;
  if ((mode & 3) == 0 && !pd_applies(m, species, rk_step)) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(m.kte, m.kde - 1);
  if (i < m.its - 1 || i > itf + 1 || j < m.jts - 1 || j > jtf + 1 || k < m.kts || k > ktf) return;
  const Stage st = stage_of(m, rk_step);
  const PDCtx c = pd_ctx(m, species, st.dt_rk);
  f3p(m, scratch[bp.m])(i, k, j) = pd_scale_cell(m, c, i, k, j);
}

// Pass 2: divergence of the limited fluxes (z, then x, then y) into advect_tend.
__global__ void __launch_bounds__(BX* BY) k_pd_tend(Launch L, int species, int rk_step, int mode, float* const* scratch) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (species >= m.nsp) return;
  const bool accum = (mode & 4) != 0;  // tendency += (routine-level callers)
  if ((mode & 3) == 0 && !pd_applies(m, species, rk_step)) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  F3 tend = f3(m, WRFGPU_ADVECT_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte && k >= m.kts && k <= m.kte;
  const int ktf = min(m.kte, m.kde - 1);
  if (!(mass_pt(m, i, j) && k >= m.kts && k <= ktf)) {
    if (in_zero && !accum) tend(i, k, j) = 0.f;
    return;
  }
  const Stage st = stage_of(m, rk_step);
  const PDCtx c = pd_ctx(m, species, st.dt_rk);
  const F3 sc = f3p(m, scratch[bp.m]);
  tend(i, k, j) = pd_tend_cell(m, c, i, k, j, accum ? tend(i, k, j) : 0.f,
                               [&](int ci, int ck, int cj) { return sc(ci, ck, cj); });
}

// ------------------------------------------------------------ edge strips
// The large step's scalar transport at the points next to an open boundary
// (open_adv.cuh), recomputed after the tile kernels from the same inputs
// (the arithmetic of k_scalar_adv_update / k_scalar_pd_update, so the
// points the open branches leave alone get the same bits twice), then
// rk_update_scalar into the spare buffer.
__device__ __forceinline__ void strip_update(const Mem& m, int s, int rk_step, int i, int j, int k, float tendency) {
  const Stage st = stage_of(m, rk_step);
  const F2 mu_old = f2(m, WRFGPU_MU_1), mu_new = f2(m, WRFGPU_MU_2), mub = f2(m, WRFGPU_MUB);
  const F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
  const float muold = mu_old(i, j) + mub(i, j), munew = mu_new(i, j) + mub(i, j);
  const F3 q = f3p(m, m.q[s]), qo = f3p(m, m.qo[s]), qa = f3p(m, m.qa[s]);
  float q1;
  if (rk_step == 1) { q1 = q(i, k, j); qo(i, k, j) = q1; }
  else q1 = qo(i, k, j);
  qa(i, k, j) = ((c1(k) * muold + c2(k)) * q1 + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
}
// advect_scalar species (every species at stages 1 and 2, the others at the
// last): the tendency plus the stored sc_tend of the species' diffusion
__global__ void __launch_bounds__(STRIP_THREADS) k_strip_scalar(StripLaunch L, int rk_step) {
  const StripPos sp = strip_pos(L);
  const Mem& m = block_member(L.mem, sp.m);
  if (!sp.valid) return;
  const int i = sp.i, j = sp.j, k = sp.k;
  if (!mass_pt(m, i, j) || k < m.kts || k > min(m.kte, m.kde - 1)) return;
  const F2 msfty = f2(m, WRFGPU_MSFTY);
  for (int s = 0; s < m.nsp; ++s) {
    if (pd_applies(m, s, rk_step)) continue;
    const F3 fld = f3p(m, m.q[s]);
    const ScalarAdv a{fld, fld, f3(m, WRFGPU_RU_M), f3(m, WRFGPU_RV_M), f3(m, WRFGPU_WW_M), f2(m, WRFGPU_MSFTX),
                      f1(m, WRFGPU_FNM), f1(m, WRFGPU_FNP), f1(m, WRFGPU_RDNW)};
    float tendency = msfty(i, j) * adv_scalar_point(m, a, 0.f, i, j, k);
    const F3 sct = f3p(m, sc_tend_of(m, s));
    if (sct.p) tendency = tendency + sct(i, k, j);
    strip_update(m, s, rk_step, i, j, k, tendency);
  }
}
// advect_scalar_pd species s at the last stage, in two passes: the limiter
// factors of the strip cells and their neighbours (the strip one wider, halo
// row / column included) into the member's PD scratch, then the limited
// divergence and the update at the strip cells
__global__ void __launch_bounds__(STRIP_THREADS) k_strip_pd_scale(StripLaunch L, int rk_step, int s,
                                                                 float* const* scratch) {
  const StripPos sp = strip_pos(L);
  const Mem& m = block_member(L.mem, sp.m);
  if (!sp.valid || s >= m.nsp || !pd_applies(m, s, rk_step)) return;
  const int i = sp.i, j = sp.j, k = sp.k;
  if (k < m.kts || k > min(m.kte, m.kde - 1)) return;
  const Stage st = stage_of(m, rk_step);
  const PDCtx c = pd_ctx(m, s, st.dt_rk, true);
  f3p(m, scratch[sp.m])(i, k, j) = pd_scale_cell(m, c, i, k, j);
}
__global__ void __launch_bounds__(STRIP_THREADS) k_strip_pd_tend(StripLaunch L, int rk_step, int s,
                                                                float* const* scratch) {
  const StripPos sp = strip_pos(L);
  const Mem& m = block_member(L.mem, sp.m);
  if (!sp.valid || s >= m.nsp || !pd_applies(m, s, rk_step)) return;
  const int i = sp.i, j = sp.j, k = sp.k;
  if (!mass_pt(m, i, j) || k < m.kts || k > min(m.kte, m.kde - 1)) return;
  const Stage st = stage_of(m, rk_step);
  const PDCtx c = pd_ctx(m, s, st.dt_rk, true);
  const F3 sc = f3p(m, scratch[sp.m]);
  const float t = pd_tend_cell(m, c, i, k, j, 0.f, [&](int ci, int ck, int cj) { return sc(ci, ck, cj); });
  strip_update(m, s, rk_step, i, j, k, f2(m, WRFGPU_MSFTY)(i, j) * t);
}
void launch_strip_scalar(const StripLaunch& L, int nb, int rk_step, cudaStream_t s) {
  if (nb > 0) k_strip_scalar<<<nb, STRIP_THREADS, 0, s>>>(L, rk_step);
}
void launch_strip_pd(const StripLaunch& wide, int nb_wide, const StripLaunch& L, int nb, int rk_step, int nsp_max,
                     float* const* d_scratch, cudaStream_t s) {
  if (nb <= 0) return;
  for (int sp = 0; sp < nsp_max; ++sp) {
    k_strip_pd_scale<<<nb_wide, STRIP_THREADS, 0, s>>>(wide, rk_step, sp, d_scratch);
    k_strip_pd_tend<<<nb, STRIP_THREADS, 0, s>>>(L, rk_step, sp, d_scratch);
  }
}

// ------------------------------------------------------------ rk_update_scalar
__global__ void __launch_bounds__(BX* BY) k_update_scalar(Launch L, int species, int rk_step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (species >= m.nsp) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (!mass_pt(m, i, j) || k < m.kts || k > min(m.kte, m.kde - 1)) return;
  const Stage st = stage_of(m, rk_step);
  F3 s1 = f3p(m, m.qo[species]), s2 = f3p(m, m.q[species]), at = f3(m, WRFGPU_ADVECT_TEND);
  F2 msfty = f2(m, WRFGPU_MSFTY), mu_old = f2(m, WRFGPU_MU_1), mu_new = f2(m, WRFGPU_MU_2), mub = f2(m, WRFGPU_MUB);
  F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
  const float muold = mu_old(i, j) + mub(i, j), munew = mu_new(i, j) + mub(i, j);
  const float tendency = at(i, k, j) * msfty(i, j);
  float q1;
  if (rk_step == 1) { q1 = s2(i, k, j); s1(i, k, j) = q1; }
  else q1 = s1(i, k, j);
  s2(i, k, j) = ((c1(k) * muold + c2(k)) * q1 + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
}

// ------------------------------------------------------------ routine-level scalar updates
// The routine-level C entry points' form of rk_update_scalar
// (module_em.F:1587-1799, pd = 0) and rk_update_scalar_pd (:1803-1916, pd =
// 1) for species 0 of a scratch domain, with the caller's sc_tend carried in
// the H_DIABATIC buffer: tendency = advect_tend msfty (rk_update_scalar only)
// + sc_tend, in the reference's order; rk_update_scalar_pd zeroes sc_tend
// after use and updates the old scalar with mu_old (MU_1) and mu_new (MU_2).
// The loop limits are the periodic / symmetric ones (the spec_zone limits of
// specified boundaries do not apply).
__global__ void __launch_bounds__(BX* BY) k_update_scalar_routine(Launch L, int rk_step, int pd) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (!mass_pt(m, i, j) || k < m.kts || k > min(m.kte, m.kde - 1)) return;
  const Stage st = stage_of(m, rk_step);
  F3 s1 = f3p(m, m.qo[0]), s2 = f3p(m, m.q[0]), at = f3(m, WRFGPU_ADVECT_TEND), sct = f3(m, WRFGPU_H_DIABATIC);
  F2 msfty = f2(m, WRFGPU_MSFTY), mu_old = f2(m, WRFGPU_MU_1), mu_new = f2(m, WRFGPU_MU_2), mub = f2(m, WRFGPU_MUB);
  F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
  const float muold = mu_old(i, j) + mub(i, j), munew = mu_new(i, j) + mub(i, j);
  if (pd) {
    float tendency = 0.f;
    tendency = tendency + sct(i, k, j);
    sct(i, k, j) = 0.f;
    s1(i, k, j) = ((c1(k) * muold + c2(k)) * s1(i, k, j) + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
    return;
  }
  float tendency = at(i, k, j) * msfty(i, j);
  tendency = tendency + sct(i, k, j);
  float q1;
  if (rk_step == 1) { q1 = s2(i, k, j); s1(i, k, j) = q1; }
  else q1 = s1(i, k, j);
  s2(i, k, j) = ((c1(k) * muold + c2(k)) * q1 + st.dt_rk * tendency) / (c1(k) * munew + c2(k));
}

// ------------------------------------------------------------ calc_p_rho_phi
__global__ void __launch_bounds__(BX* BY) k_calc_p_rho_phi(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (!mass_pt(m, i, j) || k < m.kts || k > min(m.kte, m.kde - 1)) return;
  F3 al = f3(m, WRFGPU_AL), alb = f3(m, WRFGPU_ALB), ph = f3(m, WRFGPU_PH_2), phb = f3(m, WRFGPU_PHB),
     p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB), t = f3(m, WRFGPU_T_2);
  F2 mu = f2(m, WRFGPU_MU_2), muts = f2(m, WRFGPU_MUTS);
  F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H), c3h = f1(m, WRFGPU_C3H), c4h = f1(m, WRFGPU_C4H),
     c3f = f1(m, WRFGPU_C3F), c4f = f1(m, WRFGPU_C4F), rdnw = f1(m, WRFGPU_RDNW);
  const float ptop = m.p_top;
  float alv;
  if (m.cf.hypsometric_opt == 1) {
    alv = -1.f / (c1(k) * muts(i, j) + c2(k)) * (alb(i, k, j) * (c1(k) * mu(i, j)) + rdnw(k) * (ph(i, k + 1, j) - ph(i, k, j)));
  } else {
    float pfu = c3f(k + 1) * muts(i, j) + c4f(k + 1) + ptop;
    float pfd = c3f(k) * muts(i, j) + c4f(k) + ptop;
    float phm = c3h(k) * muts(i, j) + c4h(k) + ptop;
    alv = (ph(i, k + 1, j) - ph(i, k, j) + phb(i, k + 1, j) - phb(i, k, j)) / phm / wrfgpu_ff::logf_cr(pfd / pfu) - alb(i, k, j);
  }
  al(i, k, j) = alv;
  float temp;
  if (m.cf.use_theta_m == 1) {
    temp = (R_D * (T0 + t(i, k, j))) / (P0 * (alv + alb(i, k, j)));
  } else {
    float qvf = 1.f + (461.6f / 287.f) * f3p(m, m.q[0])(i, k, j);
    temp = (R_D * (T0 + t(i, k, j)) * qvf) / (P0 * (alv + alb(i, k, j)));
  }
  float pv = wrfgpu_ff::powf_cr(temp, CPOVCV);
  p(i, k, j) = pv * P0 - pb(i, k, j);
}

// Column form over mass tiles x level chunks (gridDim.y chunks of
// kts..ktf): ph and phb of level k+1 carry down as level k of the next level,
// and so does the full-level pressure above (pfu(k) is pfd(k+1), the same
// expression), so each level reads ph and phb once.
__global__ void __launch_bounds__(TX* TY) k_calc_p_rho_phi_col(TileLaunch L) {
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  if (!mass_pt(m, i, j)) return;
  const int kts = m.kts, ktf = min(m.kte, m.kde - 1), kme = m.kme;
  const int per = (ktf - kts + 1 + (int)gridDim.y - 1) / (int)gridDim.y;
  const int k0 = kts + (int)blockIdx.y * per, k1 = min(ktf, k0 + per - 1);
  if (k0 > k1) return;
  const F3 al = f3(m, WRFGPU_AL), alb = f3(m, WRFGPU_ALB), ph = f3(m, WRFGPU_PH_2), phb = f3(m, WRFGPU_PHB),
           p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB), t = f3(m, WRFGPU_T_2), qv = f3p(m, m.q[0]);
  const F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H), c3h = f1(m, WRFGPU_C3H), c4h = f1(m, WRFGPU_C4H),
           c3f = f1(m, WRFGPU_C3F), c4f = f1(m, WRFGPU_C4F), rdnw = f1(m, WRFGPU_RDNW);
  const float ptop = m.p_top;
  const float muts_c = f2(m, WRFGPU_MUTS)(i, j), mu_c = f2(m, WRFGPU_MU_2)(i, j);
  const bool hyps1 = m.cf.hypsometric_opt == 1, theta_m = m.cf.use_theta_m == 1;
  float ph_lo = ph(i, k0, j), phb_lo = hyps1 ? 0.f : phb(i, k0, j);
  float pfd = hyps1 ? 0.f : c3f(k0) * muts_c + c4f(k0) + ptop;
  for (int k = k0; k <= k1; ++k) {
    if (k + 3 <= kme) {
      prefetch_l2(&ph(i, k + 3, j)); prefetch_l2(&phb(i, k + 3, j)); prefetch_l2(&alb(i, k + 2, j));
      prefetch_l2(&t(i, k + 2, j)); prefetch_l2(&pb(i, k + 2, j));
      if (!theta_m) prefetch_l2(&qv(i, k + 2, j));
    }
    const float ph_hi = ph(i, k + 1, j);
    const float albk = alb(i, k, j);
    float alv;
    if (hyps1) {
      alv = -1.f / (c1(k) * muts_c + c2(k)) * (albk * (c1(k) * mu_c) + rdnw(k) * (ph_hi - ph_lo));
    } else {
      const float phb_hi = phb(i, k + 1, j);
      const float pfu = c3f(k + 1) * muts_c + c4f(k + 1) + ptop;
      const float phm = c3h(k) * muts_c + c4h(k) + ptop;
      alv = (ph_hi - ph_lo + phb_hi - phb_lo) / phm / wrfgpu_ff::logf_cr(pfd / pfu) - albk;
      pfd = pfu;
      phb_lo = phb_hi;
    }
    al(i, k, j) = alv;
    float temp;
    if (theta_m) {
      temp = (R_D * (T0 + t(i, k, j))) / (P0 * (alv + albk));
    } else {
      float qvf = 1.f + (461.6f / 287.f) * qv(i, k, j);
      temp = (R_D * (T0 + t(i, k, j)) * qvf) / (P0 * (alv + albk));
    }
    const float pv = wrfgpu_ff::powf_cr(temp, CPOVCV);
    p(i, k, j) = pv * P0 - pb(i, k, j);
    ph_lo = ph_hi;
  }
}

// ------------------------------------------------------------ set_w_surface
__global__ void __launch_bounds__(BX* BY) k_set_w_surface(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j;
  if (!mass_pt(m, i, j)) return;
  const bool px = m.cf.periodic_x, py = m.cf.periodic_y;
  int jm1_limit = px || py ? m.jds : m.jds, jp1_limit = m.jde - 1, im1_limit = m.ids, ip1_limit = m.ide - 1;
  if (px) { im1_limit = m.ids - 1; ip1_limit = m.ide; }
  if (py) { jm1_limit = m.jds - 1; jp1_limit = m.jde; }
  const int jm1 = max(j - 1, jm1_limit), jp1 = min(j + 1, jp1_limit), im1 = max(i - 1, im1_limit), ip1 = min(i + 1, ip1_limit);
  F3 w = f3(m, WRFGPU_W_2), u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2);
  F2 ht = f2(m, WRFGPU_HT), msftx = f2(m, WRFGPU_MSFTX), msfty = f2(m, WRFGPU_MSFTY);
  const float cf1 = m.cf1, cf2 = m.cf2, cf3 = m.cf3;
  w(i, 1, j) = msfty(i, j) * .5f * m.rdy *
                   ((ht(i, jp1) - ht(i, j)) * (cf1 * v(i, 1, j + 1) + cf2 * v(i, 2, j + 1) + cf3 * v(i, 3, j + 1)) +
                    (ht(i, j) - ht(i, jm1)) * (cf1 * v(i, 1, j) + cf2 * v(i, 2, j) + cf3 * v(i, 3, j))) +
               msftx(i, j) * .5f * m.rdx *
                   ((ht(ip1, j) - ht(i, j)) * (cf1 * u(i + 1, 1, j) + cf2 * u(i + 1, 2, j) + cf3 * u(i + 1, 3, j)) +
                    (ht(i, j) - ht(im1, j)) * (cf1 * u(i, 1, j) + cf2 * u(i, 2, j) + cf3 * u(i, 3, j)));
}

// ------------------------------------------------------------ w_damp CFL diagnostics + health
// module_big_step_utilities_em.F:2503-2712 (the diagnostics; the w_damping = 1
// term of rw_tend is applied by the w-tendency kernels, in rk_tendency's order).
// One thread per mass column of a 32x8 tile and one block per (tile, chunk
// of levels 2..kde-1: gridDim.y chunks), the maxima kept in registers and
// reduced once per block (warp shuffles, then shared memory).  A maximum does
// not depend on the order it is taken in, so the result equals the
// reference's loop order's.  Also the health check: any non-finite u, v, w,
// theta or Courant number raises ERR_NONFINITE.
__global__ void __launch_bounds__(TX* TY, 4) k_cfl_check_col(TileLaunch L) {
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  const int per = (m.kde - 2 + gridDim.y - 1) / gridDim.y;
  const int k0 = 2 + blockIdx.y * per, k1 = min(m.kde - 1, k0 + per - 1);
  float vmax = 0.f, hmax = 0.f;
  bool bad = false;
  if (mass_pt(m, i, j) && k0 <= k1) {
    F3 ww = f3(m, WRFGPU_WW), u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2), w = f3(m, WRFGPU_W_2), t = f3(m, WRFGPU_T_2);
    F1 c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F), rdnw = f1(m, WRFGPU_RDNW);
    const float mutc = f2(m, WRFGPU_MUT)(i, j), mux = f2(m, WRFGPU_MSFUX)(i, j), mvy = f2(m, WRFGPU_MSFVY)(i, j);
    const float dt = m.dt, rdx = m.rdx, rdy = m.rdy;
#pragma unroll 4
    for (int k = k0; k <= k1; ++k) {
      const float vc = fabsf(ww.ro(i, k, j) / (c1f(k) * mutc + c2f(k)) * rdnw(k) * dt);
      const float hc = fmaxf_f(fabsf(u.ro(i, k, j) * rdx * mux * dt), fabsf(v.ro(i, k, j) * rdy * mvy * dt));
      // every load unconditional: a short-circuit || would hold the w and t
      // loads back until the other checks are known
      const float wv = w.ro(i, k, j), tv = t.ro(i, k, j);
      bad = bad | !isfinite(vc) | !isfinite(hc) | !isfinite(wv) | !isfinite(tv);
      vmax = fmaxf_f(vmax, isfinite(vc) ? vc : 0.f);
      hmax = fmaxf_f(hmax, isfinite(hc) ? hc : 0.f);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    vmax = fmaxf_f(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    hmax = fmaxf_f(hmax, __shfl_xor_sync(0xffffffffu, hmax, o));
  }
  const bool wbad = __any_sync(0xffffffffu, bad);
  __shared__ float sv[TY], sh[TY];
  __shared__ int sb[TY];
  if (threadIdx.x == 0) { sv[threadIdx.y] = vmax; sh[threadIdx.y] = hmax; sb[threadIdx.y] = wbad ? 1 : 0; }
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    float bv = 0.f, bh = 0.f;
    int bb = 0;
    for (int q = 0; q < TY; ++q) { bv = fmaxf_f(bv, sv[q]); bh = fmaxf_f(bh, sh[q]); bb |= sb[q]; }
    if (m.cfl_out) {
      atomicMax((unsigned*)&m.cfl_out[0], __float_as_uint(bv));
      atomicMax((unsigned*)&m.cfl_out[1], __float_as_uint(bh));
    }
    unsigned bits = 0;
    if (bb) bits |= ERR_NONFINITE;
    if (m.cfl_limit > 0.f && bv > m.cfl_limit) bits |= ERR_CFL;
    if (bits) raise_err(m, bits);
  }
}

// ------------------------------------------------------------ launchers
void launch_cfl_check_col(const TileLaunch& L, int nb, cudaStream_t s, int var) {
  k_cfl_check_col<<<dim3(nb, TUNE_PARAM[TU_CFL][var]), dim3(TX, TY), 0, s>>>(L);
}
void launch_update_scalar_pd(const Launch& L, int nb, StepArgs a, cudaStream_t s) {
  k_update_scalar_pd<<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step);
}
void launch_update_scalar_pd_col(const TileLaunch& L, int nb, StepArgs a, cudaStream_t s, bool sct) {
  if (sct) k_update_scalar_pd_col<true><<<dim3(nb, 4), dim3(TX, TY), 0, s>>>(L, a.rk_step);
  else k_update_scalar_pd_col<false><<<dim3(nb, 4), dim3(TX, TY), 0, s>>>(L, a.rk_step);
}
void launch_advect_scalar(const Launch& L, int nb, StepArgs a, cudaStream_t s) {
  k_advect_scalar<<<nb, dim3(BX, BY), 0, s>>>(L, a.species, a.rk_step, a.flags);
}
void launch_advect_scalar_pd2(const Launch& L, int nb, StepArgs a, float* const* d_scratch, cudaStream_t s) {
  k_pd_scale<<<nb, dim3(BX, BY), 0, s>>>(L, a.species, a.rk_step, a.flags, d_scratch);
  k_pd_tend<<<nb, dim3(BX, BY), 0, s>>>(L, a.species, a.rk_step, a.flags, d_scratch);
}
void launch_update_scalar_routine(const Launch& L, int nb, int rk_step, int pd, cudaStream_t s) {
  k_update_scalar_routine<<<nb, dim3(BX, BY), 0, s>>>(L, rk_step, pd);
}
void launch_update_scalar(const Launch& L, int nb, StepArgs a, cudaStream_t s) {
  k_update_scalar<<<nb, dim3(BX, BY), 0, s>>>(L, a.species, a.rk_step);
}
void launch_calc_p_rho_phi(const Launch& L, int nb, cudaStream_t s) { k_calc_p_rho_phi<<<nb, dim3(BX, BY), 0, s>>>(L); }
void launch_calc_p_rho_phi_col(const TileLaunch& L, int nb, cudaStream_t s, int var) {
  k_calc_p_rho_phi_col<<<dim3(nb, TUNE_PARAM[TU_CPRP][var]), dim3(TX, TY), 0, s>>>(L);
}
void launch_set_w_surface(const Launch& L, int nb, cudaStream_t s) { k_set_w_surface<<<nb, dim3(BX, BY), 0, s>>>(L); }

}  // namespace wrfgpu
