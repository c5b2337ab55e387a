// Sixth-order numerical diffusion of the dry state at the first RK stage
// and the Rayleigh damping toward the base state (damp_opt = 2)
// (sixth_order_diffusion, dyn_em/module_big_step_utilities_em.F:6220-6636,
// called from rk_tendency's forward step, dyn_em/module_em.F:879-932) and
// the addition of those forward-in-time tendencies to the large-step
// tendencies at every stage (rk_addtend_dry, dyn_em/module_em.F:959-1092).
//
// Both are point kernels over (i, j) x level blocks.  The diffusion runs once
// per large step on inputs that L2 holds for its 7-point stencils; the
// addition is one read of the stored tendency per point and stage.
#include "common.cuh"
#include "kernels.h"
#include "ffmath.h"

namespace wrfgpu {

namespace {

enum { DV_U = 0, DV_V = 1, DV_W = 2, DV_M = 3 };

// Xue's sixth-order flux through the face between f(-1) and f(0)
// (:6455-6461): 10 (f0 - f-1) - 5 (f+1 - f-2) + (f+2 - f-3).
__device__ __forceinline__ float flux6(float fm3, float fm2, float fm1, float f0, float fp1, float fp2) {
  return 10.0f * (f0 - fm1) - 5.0f * (fp1 - fm2) + (fp2 - fm3);
}

// max(1 - dzmax / dzthresh, 0): the terrain-slope taper (:6481-6497).
__device__ __forceinline__ float taper(float dzmax, float thresh) { return fmaxf(1.f - (dzmax / thresh), 0.f); }

// One point of sixth_order_diffusion for variable kind V at (i, k, j), with
// the column constants c1, c2 of level k: returns t0 + tendency_x +
// tendency_y in the reference's order (t0: the tendency's value before the
// call, zero where the tendency starts at zero).
template <int V>
__device__ float diff6_point(const Mem& m, const F3& f, const F2& mut, int i, int k, int j, float c1, float c2,
                             float coef, float t0 = 0.f) {
  const F3 phb = f3(m, WRFGPU_PHB);
  const int opt = m.cf.diff_6th_opt;
  const bool slope = m.cf.diff_6th_slopeopt >= 1;
  auto mass = [&](int ii, int jj) { return c1 * mut.ro(ii, jj) + c2; };
  const float q0 = f.ro(i, k, j);

  // ---- x (:6452-6538)
  const float xm3 = f.ro(i - 3, k, j), xm2 = f.ro(i - 2, k, j), xm1 = f.ro(i - 1, k, j);
  const float xp1 = f.ro(i + 1, k, j), xp2 = f.ro(i + 2, k, j), xp3 = f.ro(i + 3, k, j);
  float d0 = flux6(xm3, xm2, xm1, q0, xp1, xp2), d1 = flux6(xm2, xm1, q0, xp1, xp2, xp3);
  if (opt == 2) {
    if (d0 * (q0 - xm1) <= 0.f) d0 = 0.f;
    if (d1 * (xp1 - q0) <= 0.f) d1 = 0.f;
  }
  float s0 = 1.f, s1 = 1.f;
  if (slope) {
    const F2 msfux = f2(m, WRFGPU_MSFUX);
    const float dx = 1.f / m.rdx;
    const float thresh = m.cf.diff_6th_thresh * 9.81f * dx;
    float z0, z1;
    if (V == DV_U) {
      z0 = fmaxf(fabsf(phb.ro(i, k, j) - phb.ro(i - 1, k, j)) * msfux.ro(i, j),
                 fabsf(phb.ro(i - 1, k, j) - phb.ro(i - 2, k, j)) * msfux.ro(i - 1, j));
      z1 = fmaxf(fabsf(phb.ro(i + 1, k, j) - phb.ro(i, k, j)) * msfux.ro(i + 1, j),
                 fabsf(phb.ro(i, k, j) - phb.ro(i - 1, k, j)) * msfux.ro(i, j));
    } else if (V == DV_V) {
      z0 = fmaxf(fabsf(phb.ro(i, k, j) - phb.ro(i - 1, k, j)) * msfux.ro(i, j),
                 fabsf(phb.ro(i, k, j - 1) - phb.ro(i - 1, k, j - 1)) * msfux.ro(i, j - 1));
      z1 = fmaxf(fabsf(phb.ro(i + 1, k, j) - phb.ro(i, k, j)) * msfux.ro(i + 1, j),
                 fabsf(phb.ro(i + 1, k, j - 1) - phb.ro(i, k, j - 1)) * msfux.ro(i + 1, j - 1));
    } else {
      z0 = fabsf(phb.ro(i, k, j) - phb.ro(i - 1, k, j)) * msfux.ro(i, j);
      z1 = fabsf(phb.ro(i + 1, k, j) - phb.ro(i, k, j)) * msfux.ro(i + 1, j);
    }
    s0 = taper(z0, thresh);
    s1 = taper(z1, thresh);
  }
  float m0, m1, msf;
  if (V == DV_U) {
    m0 = mass(i - 1, j); m1 = mass(i, j); msf = f2(m, WRFGPU_MSFUX).ro(i, j);
  } else if (V == DV_V) {
    m0 = 0.25f * (mass(i - 1, j - 1) + mass(i, j - 1) + mass(i - 1, j) + mass(i, j));
    m1 = 0.25f * (mass(i, j - 1) + mass(i + 1, j - 1) + mass(i, j) + mass(i + 1, j));
    msf = f2(m, WRFGPU_MSFVX).ro(i, j);
  } else {
    m0 = 0.5f * (mass(i - 1, j) + mass(i, j));
    m1 = 0.5f * (mass(i, j) + mass(i + 1, j));
    msf = f2(m, WRFGPU_MSFTX).ro(i, j);
  }
  const float tx = coef * msf * ((s1 * m1 * d1) - (s0 * m0 * d0));

  // ---- y (:6543-6628)
  const float ym3 = f.ro(i, k, j - 3), ym2 = f.ro(i, k, j - 2), ym1 = f.ro(i, k, j - 1);
  const float yp1 = f.ro(i, k, j + 1), yp2 = f.ro(i, k, j + 2), yp3 = f.ro(i, k, j + 3);
  d0 = flux6(ym3, ym2, ym1, q0, yp1, yp2);
  d1 = flux6(ym2, ym1, q0, yp1, yp2, yp3);
  if (opt == 2) {
    if (d0 * (q0 - ym1) <= 0.f) d0 = 0.f;
    if (d1 * (yp1 - q0) <= 0.f) d1 = 0.f;
  }
  s0 = 1.f; s1 = 1.f;
  if (slope) {
    const F2 msfvy = f2(m, WRFGPU_MSFVY);
    const float dy = 1.f / m.rdy;
    const float thresh = m.cf.diff_6th_thresh * 9.81f * dy;
    float z0, z1;
    if (V == DV_U) {
      z0 = fmaxf(fabsf(phb.ro(i, k, j) - phb.ro(i, k, j - 1)) * msfvy.ro(i, j),
                 fabsf(phb.ro(i - 1, k, j) - phb.ro(i - 1, k, j - 1)) * msfvy.ro(i - 1, j));
      z1 = fmaxf(fabsf(phb.ro(i, k, j + 1) - phb.ro(i, k, j)) * msfvy.ro(i, j + 1),
                 fabsf(phb.ro(i - 1, k, j + 1) - phb.ro(i - 1, k, j)) * msfvy.ro(i - 1, j + 1));
    } else if (V == DV_V) {
      z0 = fmaxf(fabsf(phb.ro(i, k, j) - phb.ro(i, k, j - 1)) * msfvy.ro(i, j),
                 fabsf(phb.ro(i, k, j - 1) - phb.ro(i, k, j - 2)) * msfvy.ro(i, j - 1));
      z1 = fmaxf(fabsf(phb.ro(i, k, j + 1) - phb.ro(i, k, j)) * msfvy.ro(i, j + 1),
                 fabsf(phb.ro(i, k, j) - phb.ro(i, k, j - 1)) * msfvy.ro(i, j));
    } else {
      z0 = fabsf(phb.ro(i, k, j) - phb.ro(i, k, j - 1)) * msfvy.ro(i, j);
      z1 = fabsf(phb.ro(i, k, j + 1) - phb.ro(i, k, j)) * msfvy.ro(i, j + 1);
    }
    s0 = taper(z0, thresh);
    s1 = taper(z1, thresh);
  }
  if (V == DV_U) {
    m0 = 0.25f * (mass(i - 1, j - 1) + mass(i, j - 1) + mass(i - 1, j) + mass(i, j));
    m1 = 0.25f * (mass(i - 1, j) + mass(i, j) + mass(i - 1, j + 1) + mass(i, j + 1));
    msf = f2(m, WRFGPU_MSFUY).ro(i, j);
  } else if (V == DV_V) {
    m0 = mass(i, j - 1); m1 = mass(i, j); msf = f2(m, WRFGPU_MSFVY).ro(i, j);
  } else {
    m0 = 0.5f * (mass(i, j - 1) + mass(i, j));
    m1 = 0.5f * (mass(i, j) + mass(i, j + 1));
    msf = f2(m, WRFGPU_MSFTY).ro(i, j);
  }
  const float ty = coef * msf * ((s1 * m1 * d1) - (s0 * m0 * d0));
  float t = t0;
  t = t + tx;
  t = t + ty;
  return t;
}

// Stage 1, mode 0 (rk_tendency): the forward-in-time tendencies ru_tendf,
// rv_tendf, rw_tendf and t_tendf of the sixth-order diffusion of u_2, v_2,
// w_2 and t_2 with mut and the large step dt.  Mode 1 (rk_scalar_tend,
// module_em.F:1421-1435, after the acoustic steps): each diffused species'
// sc_tend, with muts and the stage's dt (dt / 3).  Loop limits of periodic /
// symmetric boundaries (:6330-6443); points outside them keep the zero the
// buffers were created with.
__global__ void __launch_bounds__(BX* BY) k_sixth_diff(Launch L, int mode) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid || m.tendf[0] == nullptr || m.cf.diff_6th_opt == 0) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  const int ktf = min(m.kte, m.kde - 1);
  if (i < m.its || j < m.jts || k < m.kts || k > ktf) return;
  const int i_end = min(m.ide - 1, m.ite), j_end = min(m.jde - 1, m.jte);
  const F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H);
  const float c1 = c1h(k), c2 = c2h(k);
  if (mode == 1) {
    if (i > i_end || j > j_end) return;
    const float coef = m.cf.diff_6th_factor * 0.015625f / (2.0f * stage_of(m, 1).dt_rk);
    const F2 muts = f2(m, WRFGPU_MUTS);
    for (int s = 0; s < m.nsp; ++s) {
      float* sc = sc_tend_of(m, s);
      if (sc) f3p(m, sc)(i, k, j) = diff6_point<DV_M>(m, f3p(m, m.q[s]), muts, i, k, j, c1, c2, coef);
    }
    return;
  }
  const float coef = m.cf.diff_6th_factor * 0.015625f / (2.0f * m.dt);
  const F2 mut = f2(m, WRFGPU_MUT);
  if (i <= m.ite && j <= j_end)
    f3p(m, m.tendf[0])(i, k, j) = diff6_point<DV_U>(m, f3(m, WRFGPU_U_2), mut, i, k, j, c1, c2, coef);
  if (i <= i_end && j <= m.jte)
    f3p(m, m.tendf[1])(i, k, j) = diff6_point<DV_V>(m, f3(m, WRFGPU_V_2), mut, i, k, j, c1, c2, coef);
  if (i <= i_end && j <= j_end) {
    if (k >= m.kts + 1) {
      const F1 c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F);
      f3p(m, m.tendf[2])(i, k, j) = diff6_point<DV_W>(m, f3(m, WRFGPU_W_2), mut, i, k, j, c1f(k), c2f(k), coef);
    }
    f3p(m, m.tendf[3])(i, k, j) = diff6_point<DV_M>(m, f3(m, WRFGPU_T_2), mut, i, k, j, c1, c2, coef);
  }
}

// The routine-level form of rk_scalar_tend's sixth-order diffusion
// (module_em.F:1421-1435): species 0 of a scratch domain accumulated into
// the caller's scalar_tends, carried in the H_DIABATIC buffer, with mut
// (MUTS) and the caller's dt_step.
__global__ void __launch_bounds__(BX* BY) k_sixth_diff_species_routine(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  const int ktf = min(m.kte, m.kde - 1);
  if (i < m.its || j < m.jts || k < m.kts || k > ktf) return;
  if (i > min(m.ide - 1, m.ite) || j > min(m.jde - 1, m.jte)) return;
  const F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H);
  const float coef = m.cf.diff_6th_factor * 0.015625f / (2.0f * stage_of(m, 1).dt_rk);
  F3 out = f3(m, WRFGPU_H_DIABATIC);
  out(i, k, j) = diff6_point<DV_M>(m, f3p(m, m.q[0]), f2(m, WRFGPU_MUTS), i, k, j, c1h(k), c2h(k), coef, out(i, k, j));
}

// Stage 1, damp_opt = 2: rk_rayleigh_damp (module_big_step_utilities_em.F:
// 5836-6110), relaxation of u, v, w and theta toward the base-state
// profiles in the top zdamp metres, into ru_tendf .. t_tendf.  One thread per
// column (i, j) of the memory extent, handling u, v, w and theta of that
// column; the top layer's level heights are formed again where they are
// used (the same expressions, so the same bits) instead of being stored.
// A member that also stores the sixth-order diffusion accumulates onto it
// (written earlier in the same stage); otherwise every level of the loop
// range is written, the damped ones as 0 - term and the others as 0, which is
// the reference's zeroed tendency plus its additions.  The level searches
// stop at kts.
__device__ __forceinline__ float rayleigh_weight(float ztop, float z, float zdamp) {
  const float dcoef = 1.0f - fminf_f(1.0f, (ztop - z) / zdamp);
  const float s = wrfgpu_ff::sinf_cr(0.5f * PI_F * dcoef);
  return s * s;
}
template <typename HF>
__device__ int rayleigh_top_level(float ztop, float zdamp, int kts, int ktf, HF height) {
  int k1 = ktf;
  float z = ztop;
  while (z >= ztop - zdamp && k1 >= kts) {
    z = height(k1);
    k1 = k1 - 1;
  }
  return k1 + 2;
}
__device__ __forceinline__ float rayleigh_profile(const F1& prof, const F1& zb, float z, int kts, int ktf) {
  int k2 = ktf;
  while (zb(k2) > z && k2 > kts) k2 = k2 - 1;
  if (k2 + 1 > ktf) return prof(k2) + (prof(k2) - prof(k2 - 1)) * (z - zb(k2)) / (zb(k2) - zb(k2 - 1));
  return prof(k2) + (prof(k2 + 1) - prof(k2)) * (z - zb(k2)) / (zb(k2 + 1) - zb(k2));
}
__global__ void __launch_bounds__(BX* BY) k_rayleigh_damp(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid || m.cf.damp_opt != 2 || m.tendf[0] == nullptr) return;
  const int i = bp.i, j = bp.j;
  if (i < m.its || j < m.jts) return;
  const int kts = m.kts, ktf = min(m.kte, m.kde - 1), kde = m.kde;
  const bool acc = m.cf.diff_6th_opt != 0;
  const float dampcoef = m.cf.dampcoef, zdamp = m.cf.zdamp;
  const F3 ph = f3(m, WRFGPU_PH_2), phb = f3(m, WRFGPU_PHB);
  const F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F);
  const F1 zb = f1(m, WRFGPU_Z_BASE);
  // u (:5897-5945)
  if (i <= min(m.ite, m.ide) && j <= min(m.jte, m.jde - 1)) {
    const F3 u = f3(m, WRFGPU_U_2), tend = f3p(m, m.tendf[0]);
    const F1 prof = f1(m, WRFGPU_U_BASE);
    const float mu = f2(m, WRFGPU_MUU)(i, j);
    const float ztop = 0.5f * (phb(i, kde, j) + phb(i - 1, kde, j) + ph(i, kde, j) + ph(i - 1, kde, j)) / G;
    auto height = [&](int k) {
      return 0.25f * (phb(i, k, j) + phb(i, k + 1, j) + phb(i - 1, k, j) + phb(i - 1, k + 1, j) + ph(i, k, j) +
                      ph(i, k + 1, j) + ph(i - 1, k, j) + ph(i - 1, k + 1, j)) / G;
    };
    const int k1 = rayleigh_top_level(ztop, zdamp, kts, ktf, height);
    for (int k = kts; k <= ktf; ++k) {
      float t = acc ? tend(i, k, j) : 0.f;
      if (k >= k1) {
        const float z = height(k);
        t = t - (c1h(k) * mu + c2h(k)) * (rayleigh_weight(ztop, z, zdamp) * dampcoef) *
                    (u(i, k, j) - rayleigh_profile(prof, zb, z, kts, ktf));
      }
      tend(i, k, j) = t;
    }
  }
  // v (:5947-5995)
  if (i <= min(m.ite, m.ide - 1) && j <= min(m.jte, m.jde)) {
    const F3 v = f3(m, WRFGPU_V_2), tend = f3p(m, m.tendf[1]);
    const F1 prof = f1(m, WRFGPU_V_BASE);
    const float mv = f2(m, WRFGPU_MUV)(i, j);
    const float ztop = 0.5f * (phb(i, kde, j) + phb(i, kde, j - 1) + ph(i, kde, j) + ph(i, kde, j - 1)) / G;
    auto height = [&](int k) {
      return 0.25f * (phb(i, k, j) + phb(i, k + 1, j) + phb(i, k, j - 1) + phb(i, k + 1, j - 1) + ph(i, k, j) +
                      ph(i, k + 1, j) + ph(i, k, j - 1) + ph(i, k + 1, j - 1)) / G;
    };
    const int k1 = rayleigh_top_level(ztop, zdamp, kts, ktf, height);
    for (int k = kts; k <= ktf; ++k) {
      float t = acc ? tend(i, k, j) : 0.f;
      if (k >= k1) {
        const float z = height(k);
        t = t - (c1h(k) * mv + c2h(k)) * (rayleigh_weight(ztop, z, zdamp) * dampcoef) *
                    (v(i, k, j) - rayleigh_profile(prof, zb, z, kts, ktf));
      }
      tend(i, k, j) = t;
    }
  }
  // w (:5997-6013) and theta (:6015-6062)
  if (i <= min(m.ite, m.ide - 1) && j <= min(m.jte, m.jde - 1)) {
    const F3 w = f3(m, WRFGPU_W_2), t3 = f3(m, WRFGPU_T_2);
    const F3 tw = f3p(m, m.tendf[2]), tt = f3p(m, m.tendf[3]);
    const F1 prof = f1(m, WRFGPU_T_BASE);
    const float mt = f2(m, WRFGPU_MUT)(i, j);
    const float ztop = (phb(i, kde, j) + ph(i, kde, j)) / G;
    for (int k = kts; k <= min(m.kte, kde); ++k) {
      float t = acc ? tw(i, k, j) : 0.f;
      const float z = (phb(i, k, j) + ph(i, k, j)) / G;
      if (z >= ztop - zdamp)
        t = t - (c1f(k) * mt + c2f(k)) * (rayleigh_weight(ztop, z, zdamp) * dampcoef) * w(i, k, j);
      tw(i, k, j) = t;
    }
    auto height = [&](int k) { return 0.5f * (phb(i, k, j) + phb(i, k + 1, j) + ph(i, k, j) + ph(i, k + 1, j)) / G; };
    const int k1 = rayleigh_top_level(ztop, zdamp, kts, ktf, height);
    for (int k = kts; k <= ktf; ++k) {
      float t = acc ? tt(i, k, j) : 0.f;
      if (k >= k1) {
        const float z = height(k);
        t = t - (c1h(k) * mt + c2h(k)) * (rayleigh_weight(ztop, z, zdamp) * dampcoef) *
                    (t3(i, k, j) - rayleigh_profile(prof, zb, z, kts, ktf));
      }
      tt(i, k, j) = t;
    }
  }
}

// Every stage: rk_addtend_dry for the stored tendencies.  With physics off
// the saved tendencies, h_diabatic, ph_tendf and mu_tendf are zero: the
// stage-1 "tendf + save * msf" steps add +0 to a tendency that is never -0
// and the ph / mu additions are left out; theta keeps its h_diabatic term,
// which can turn a -0 sum into +0.
__global__ void __launch_bounds__(BX* BY) k_addtend_dry(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid || m.tendf[0] == nullptr) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (i < m.its || j < m.jts || k < m.kts || k > m.kte) return;
  const int i_end = min(m.ite, m.ide - 1), j_end = min(m.jte, m.jde - 1);
  if (k <= m.kte - 1) {
    if (i <= m.ite && j <= j_end) {
      F3 t = f3(m, WRFGPU_RU_TEND);
      t(i, k, j) = t(i, k, j) + f3p(m, m.tendf[0]).ro(i, k, j) / f2(m, WRFGPU_MSFUY).ro(i, j);
    }
    if (i <= i_end && j <= m.jte) {
      F3 t = f3(m, WRFGPU_RV_TEND);
      t(i, k, j) = t(i, k, j) + f3p(m, m.tendf[1]).ro(i, k, j) * f2(m, WRFGPU_MSFVX_INV).ro(i, j);
    }
    if (i <= i_end && j <= j_end) {
      F3 t = f3(m, WRFGPU_T_TEND);
      const float msfty = f2(m, WRFGPU_MSFTY).ro(i, j);
      const float mass = f1(m, WRFGPU_C1H)(k) * f2(m, WRFGPU_MUT).ro(i, j) + f1(m, WRFGPU_C2H)(k);
      t(i, k, j) = t(i, k, j) + f3p(m, m.tendf[3]).ro(i, k, j) / msfty + mass * 0.f / msfty;
    }
  }
  if (i <= i_end && j <= j_end) {
    F3 t = f3(m, WRFGPU_RW_TEND);
    t(i, k, j) = t(i, k, j) + f3p(m, m.tendf[2]).ro(i, k, j) / f2(m, WRFGPU_MSFTY).ro(i, j);
  }
}

}  // namespace

void launch_sixth_diff(const Launch& L, int nblocks, int mode, cudaStream_t s) {
  k_sixth_diff<<<nblocks, dim3(BX, BY), 0, s>>>(L, mode);
}

void launch_sixth_diff_species_routine(const Launch& L, int nblocks, cudaStream_t s) {
  k_sixth_diff_species_routine<<<nblocks, dim3(BX, BY), 0, s>>>(L);
}

void launch_rayleigh_damp(const Launch& L2, int nblocks, cudaStream_t s) {
  k_rayleigh_damp<<<nblocks, dim3(BX, BY), 0, s>>>(L2);
}

void launch_addtend_dry(const Launch& L, int nblocks, cudaStream_t s) {
  k_addtend_dry<<<nblocks, dim3(BX, BY), 0, s>>>(L);
}

}  // namespace wrfgpu
