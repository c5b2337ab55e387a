// rk_tendency (dyn_em/module_em.F:370-781, physics off) as five fused
// kernels, one per tendency field.  Each output point applies, in the
// reference's order, zero_tend, the advection flux divergence (y, then x,
// then z), the pressure-gradient / buoyancy term, Coriolis and curvature;
// neighbouring fluxes are recomputed per point instead of being staged, so
// every value is the reference's expression evaluated on the same inputs.
//   ru_tend: advect_u (module_advect_em.F:486-745, :1470-1497),
//            horizontal_pressure_gradient (module_big_step_utilities_em.F:2346-2414),
//            coriolis (:3699-3711), curvature (:4289-4330)
//   rv_tend: advect_v (:1904-2171, :2961-2995), HPG (:2247-2300), coriolis (:3724-3736), curvature (:4385-4420)
//   rw_tend: advect_w (:4784-5096, :5996-6031), pg_buoy_w (:2419-2502), coriolis (:3738-3749), curvature (:4447-4466)
//   t_tend : advect_scalar on theta (:3394-3650, :4306-4333)
//   ph_tend: rhs_ph (:1365-1530, :1768-2075)
// Roofline: HBM-bound stencils (~0.5-1 flop/B); the horizontal 6-point
// neighbours are served from L1/L2, so DRAM traffic stays near one read per
// input array and one write per tendency.
#include "common.cuh"
#include "kernels.h"
#include "open_adv.cuh"

namespace wrfgpu {

// ---------------------------------------------------------------- ru_tend
template <int FL>
__device__ __forceinline__ void tend_u_point(const Mem& m, const int i, const int j, const int k) {
  F3 tend = f3(m, WRFGPU_RU_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte && k >= m.kts && k <= m.kte;
  const int ktf = min(m.kte, m.kde - 1);
  const bool in_acc = i >= m.its && i <= m.ite && j >= m.jts && j <= min(m.jte, m.jde - 1) && k >= m.kts && k <= ktf;
  if (!in_acc) {
    if ((FL & TF_ZERO) && in_zero) tend(i, k, j) = 0.f;
    return;
  }
  float t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
  F3 u = f3(m, WRFGPU_U_2), ru = f3(m, WRFGPU_RU), rv = f3(m, WRFGPU_RV), rw = f3(m, WRFGPU_RW);
  F2 msfux = f2(m, WRFGPU_MSFUX), msfuy = f2(m, WRFGPU_MSFUY);
  const float rdx = m.rdx, rdy = m.rdy;
  // open lateral boundaries: the columns next to them take lower-order
  // fluxes and radiation terms, and some terms leave the boundary u out
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const bool px = m.cf.periodic_x;
  const int ids = m.ids, ide = m.ide, jds = m.jds, jde = m.jde;
  // i range of the y advection, the radiation rows, the pressure gradient,
  // Coriolis and curvature (module_advect_em.F:521-525, :1280-1289;
  // module_big_step_utilities_em.F:2346-2351, :3710-3717, :4292-4298)
  const bool inner_x = px || ((!oxs || i >= ids + 1) && (!oxe || i <= ide - 1));
  if (FL & TF_ADV) {
    F3 rom = f3(m, WRFGPU_WW);
    F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzw = f1(m, WRFGPU_RDNW);
    // y flux divergence (module_advect_em.F:519-628)
    auto fy = [&](int jj) {
      const int o = open_order_mass(jj, oys, oye, jds, jde);
      if (o == 2) return 0.25f * (rv(i, k, jj) + rv(i - 1, k, jj)) * (u(i, k, jj) + u(i, k, jj - 1));
      float vel = 0.5f * (rv(i, k, jj) + rv(i - 1, k, jj));
      if (o == 3) return vel * flux3(u(i, k, jj - 2), u(i, k, jj - 1), u(i, k, jj), u(i, k, jj + 1), vel);
      return vel * flux5(u(i, k, jj - 3), u(i, k, jj - 2), u(i, k, jj - 1), u(i, k, jj), u(i, k, jj + 1), u(i, k, jj + 2), vel);
    };
    if (inner_x && (!oys || j >= jds + 1) && (!oye || j <= jde - 2)) {
      float mrdy = msfux(i, j) * rdy;
      t = t - mrdy * (fy(j + 1) - fy(j));
    }
    // x flux divergence (:632-743): second-order faces next to the boundary
    // take the boundary u itself (ub)
    auto fx = [&](int ii) {
      const int o = open_order_stag(ii, oxs, oxe, ids, ide);
      if (o == 2) {
        if (ii == ids + 1) return 0.25f * (ru(ii, k, j) + ru(ii - 1, k, j)) * (u(ii, k, j) + u(ii - 1, k, j));
        return 0.25f * (ru(ii, k, j) + ru(ii - 1, k, j)) * (u(ii - 1, k, j) + u(ii, k, j));
      }
      float vel = 0.5f * (ru(ii, k, j) + ru(ii - 1, k, j));
      if (o == 3) return vel * flux3(u(ii - 2, k, j), u(ii - 1, k, j), u(ii, k, j), u(ii + 1, k, j), vel);
      return vel * flux5(u(ii - 3, k, j), u(ii - 2, k, j), u(ii - 1, k, j), u(ii, k, j), u(ii + 1, k, j), u(ii + 2, k, j), vel);
    };
    if ((!oxs || i >= ids + 1) && (!oxe || i <= ide - 1)) {
      float mrdx = msfux(i, j) * rdx;
      t = t - mrdx * (fx(i + 1) - fx(i));
    }
    // radiation conditions (:1241-1335; u_old is u in rk_tendency)
    if ((oxs && i == ids) || (oxe && i == ide)) {
      F2 mut = f2(m, WRFGPU_MUT);
      F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
      if (i == ids) {
        const float ub = fminf_f(ru(i, k, j) - CB * (c1(k) * mut(i, j) + c2(k)), 0.f);
        t = t - rdx * ub * (u(i + 1, k, j) - u(i, k, j));
      } else {
        const float ub = fmaxf_f(ru(i, k, j) + CB * (c1(k) * mut(i - 1, j) + c2(k)), 0.f);
        t = t - rdx * ub * (u(i, k, j) - u(i - 1, k, j));
      }
    }
    if (((oys && j == jds) || (oye && j == jde - 1)) && (!oxs || i >= ids + 1) && (!oxe || i <= ide - 1)) {
      const float mrdy = msfux(i, j) * rdy;
      const int ip = min(ide - 1, i), im = max(ids, i - 1);
      if (j == jds) {
        const float vw = 0.5f * (rv(ip, k, j) + rv(im, k, j));
        const float vb = fminf_f(vw, 0.f);
        const float dvm = rv(ip, k, j + 1) - rv(ip, k, j);
        const float dvp = rv(im, k, j + 1) - rv(im, k, j);
        t = t - mrdy * (vb * (u(i, k, j + 1) - u(i, k, j)) + 0.5f * u(i, k, j) * (dvm + dvp));
      } else {
        const float vw = 0.5f * (rv(ip, k, j + 1) + rv(im, k, j + 1));
        const float vb = fmaxf_f(vw, 0.f);
        const float dvm = rv(ip, k, j + 1) - rv(ip, k, j);
        const float dvp = rv(im, k, j + 1) - rv(im, k, j);
        t = t - mrdy * (vb * (u(i, k, j) - u(i, k, j - 1)) + 0.5f * u(i, k, j) * (dvm + dvp));
      }
    }
    // vertical (:1338-1356: the reference narrows the i range on open_ys /
    // open_ye here, not on open_xs / open_xe)
    auto vf = [&](int kk) -> float {
      if (kk == m.kts || kk == m.kte) return 0.f;
      if (kk == m.kts + 1 || kk == ktf)
        return 0.5f * (rom(i, kk, j) + rom(i - 1, kk, j)) * (fzm(kk) * u(i, kk, j) + fzp(kk) * u(i, kk - 1, j));
      float vel = 0.5f * (rom(i - 1, kk, j) + rom(i, kk, j));
      return vel * flux3(u(i, kk - 2, j), u(i, kk - 1, j), u(i, kk, j), u(i, kk + 1, j), -vel);
    };
    if (px || ((!oys || i >= ids + 1) && (!oye || i <= ide - 1))) t = t - rdzw(k) * (vf(k + 1) - vf(k));
  }
  if (FL & TF_PG) {
    F3 ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT), p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB),
       al = f3(m, WRFGPU_AL), php = f3(m, WRFGPU_PHP), cqu = f3(m, WRFGPU_CQU);
    F2 muu = f2(m, WRFGPU_MUU), mu = f2(m, WRFGPU_MU_2);
    F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP),
       rdnw = f1(m, WRFGPU_RDNW);
    const int kde = m.kde;
    auto dpn = [&](int kk) -> float {
      if (kk == kde) {
        if (m.cf.top_lid)
          return .5f * (m.cfn * (p(i - 1, kde - 1, j) + p(i, kde - 1, j)) + m.cfn1 * (p(i - 1, kde - 2, j) + p(i, kde - 2, j)));
        return 0.f;
      }
      if (kk == 1)
        return .5f * (m.cf1 * (p(i - 1, 1, j) + p(i, 1, j)) + m.cf2 * (p(i - 1, 2, j) + p(i, 2, j)) +
                      m.cf3 * (p(i - 1, 3, j) + p(i, 3, j)));
      return .5f * (fnm(kk) * (p(i - 1, kk, j) + p(i, kk, j)) + fnp(kk) * (p(i - 1, kk - 1, j) + p(i, kk - 1, j)));
    };
    float dpx = (msfux(i, j) / msfuy(i, j)) * .5f * rdx * (c1h(k) * muu(i, j) + c2h(k)) *
                ((ph(i, k + 1, j) - ph(i - 1, k + 1, j) + ph(i, k, j) - ph(i - 1, k, j)) +
                 (alt(i, k, j) + alt(i - 1, k, j)) * (p(i, k, j) - p(i - 1, k, j)) +
                 (al(i, k, j) + al(i - 1, k, j)) * (pb(i, k, j) - pb(i - 1, k, j)));
    dpx = dpx + (msfux(i, j) / msfuy(i, j)) * rdx * (php(i, k, j) - php(i - 1, k, j)) *
                    (rdnw(k) * (dpn(k + 1) - dpn(k)) - .5f * ((c1h(k) * mu(i - 1, j)) + (c1h(k) * mu(i, j))));
    if (inner_x) t = t - cqu(i, k, j) * dpx;
  }
  if ((FL & TF_COR) && inner_x) {
    F2 f = f2(m, WRFGPU_F), e = f2(m, WRFGPU_E), cosa = f2(m, WRFGPU_COSA);
    t = t + (msfux(i, j) / msfuy(i, j)) * 0.5f * (f(i, j) + f(i - 1, j)) * 0.25f *
                (rv(i - 1, k, j + 1) + rv(i, k, j + 1) + rv(i - 1, k, j) + rv(i, k, j)) -
        0.5f * (e(i, j) + e(i - 1, j)) * 0.5f * (cosa(i, j) + cosa(i - 1, j)) * 0.25f *
            (rw(i - 1, k + 1, j) + rw(i - 1, k, j) + rw(i, k + 1, j) + rw(i, k, j));
  }
  if ((FL & TF_CURV) && inner_x) {
    F3 v = f3(m, WRFGPU_V_2);
    F2 msfvx = f2(m, WRFGPU_MSFVX);
    auto vxgm = [&](int ii) {
      return 0.5f * (u(ii, k, j) + u(ii + 1, k, j)) * (msfvx(ii, j + 1) - msfvx(ii, j)) * rdy -
             0.5f * (v(ii, k, j) + v(ii, k, j + 1)) * (msfuy(ii + 1, j) - msfuy(ii, j)) * rdx;
    };
    t = t + 0.5f * (vxgm(i) + vxgm(i - 1)) * 0.25f * (rv(i - 1, k, j + 1) + rv(i, k, j + 1) + rv(i - 1, k, j) + rv(i, k, j)) -
        u(i, k, j) * RERADIUS * 0.25f * (rw(i - 1, k + 1, j) + rw(i - 1, k, j) + rw(i, k + 1, j) + rw(i, k, j));
  }
  tend(i, k, j) = t;
}

template <int FL>
__global__ void __launch_bounds__(BX* BY) k_tend_u(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  tend_u_point<FL>(m, bp.i, bp.j, bp.k);
}


// ---------------------------------------------------------------- rv_tend
template <int FL>
__device__ __forceinline__ void tend_v_point(const Mem& m, const int i, const int j, const int k) {
  F3 tend = f3(m, WRFGPU_RV_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte && k >= m.kts && k <= m.kte;
  const int ktf = min(m.kte, m.kde - 1);
  const bool in_acc = i >= m.its && i <= min(m.ite, m.ide - 1) && j >= m.jts && j <= m.jte && k >= m.kts && k <= ktf;
  if (!in_acc) {
    if ((FL & TF_ZERO) && in_zero) tend(i, k, j) = 0.f;
    return;
  }
  float t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
  F3 v = f3(m, WRFGPU_V_2), ru = f3(m, WRFGPU_RU), rv = f3(m, WRFGPU_RV), rw = f3(m, WRFGPU_RW);
  F2 msfvx = f2(m, WRFGPU_MSFVX), msfvy = f2(m, WRFGPU_MSFVY);
  const float rdx = m.rdx, rdy = m.rdy;
  // open lateral boundaries (see tend_u_point)
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const int ids = m.ids, ide = m.ide, jds = m.jds, jde = m.jde;
  // j range of the x advection, the pressure gradient, Coriolis and
  // curvature (module_advect_em.F:2076-2077; module_big_step_utilities_em.F:
  // :2273-2276, :3765-3768, :4352-4356)
  const bool inner_y = (!oys || j >= jds + 1) && (!oye || j <= jde - 1);
  if (FL & TF_ADV) {
    F3 rom = f3(m, WRFGPU_WW);
    F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzw = f1(m, WRFGPU_RDNW);
    // y flux divergence (module_advect_em.F:1936-2062): second-order faces
    // next to the boundary take the boundary v itself (vb)
    auto fy = [&](int jj) {
      const int o = open_order_stag(jj, oys, oye, jds, jde);
      if (o == 2) {
        if (jj == jds + 1) return 0.25f * (rv(i, k, jj) + rv(i, k, jj - 1)) * (v(i, k, jj) + v(i, k, jj - 1));
        return 0.25f * (rv(i, k, jj) + rv(i, k, jj - 1)) * (v(i, k, jj) + v(i, k, jj - 1));
      }
      float vel = 0.5f * (rv(i, k, jj) + rv(i, k, jj - 1));
      if (o == 3) return vel * flux3(v(i, k, jj - 2), v(i, k, jj - 1), v(i, k, jj), v(i, k, jj + 1), vel);
      return vel * flux5(v(i, k, jj - 3), v(i, k, jj - 2), v(i, k, jj - 1), v(i, k, jj), v(i, k, jj + 1), v(i, k, jj + 2), vel);
    };
    if (inner_y) {
      float mrdy = msfvy(i, j) * rdy;
      t = t - mrdy * (fy(j + 1) - fy(j));
    }
    // x flux divergence (:2066-2171)
    auto fx = [&](int ii) {
      const int o = open_order_mass(ii, oxs, oxe, ids, ide);
      if (o == 2) return 0.25f * (ru(ii, k, j) + ru(ii, k, j - 1)) * (v(ii, k, j) + v(ii - 1, k, j));
      float vel = 0.5f * (ru(ii, k, j) + ru(ii, k, j - 1));
      if (o == 3) return vel * flux3(v(ii - 2, k, j), v(ii - 1, k, j), v(ii, k, j), v(ii + 1, k, j), vel);
      return vel * flux5(v(ii - 3, k, j), v(ii - 2, k, j), v(ii - 1, k, j), v(ii, k, j), v(ii + 1, k, j), v(ii + 2, k, j), vel);
    };
    if (inner_y && (!oxs || i >= ids + 1) && (!oxe || i <= ide - 2)) {
      float mrdx = msfvy(i, j) * rdx;
      t = t - mrdx * (fx(i + 1) - fx(i));
    }
    // radiation conditions (:2711-2808; v_old is v in rk_tendency)
    if ((oys && j == jds) || (oye && j == jde)) {
      F2 mut = f2(m, WRFGPU_MUT);
      F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
      if (j == jds) {
        const float vb = fminf_f(rv(i, k, j) - CB * (c1(k) * mut(i, j) + c2(k)), 0.f);
        t = t - rdy * vb * (v(i, k, j + 1) - v(i, k, j));
      } else {
        const float vb = fmaxf_f(rv(i, k, j) + CB * (c1(k) * mut(i, j - 1) + c2(k)), 0.f);
        t = t - rdy * vb * (v(i, k, j) - v(i, k, j - 1));
      }
    }
    if (((oxs && i == ids) || (oxe && i == ide - 1)) && inner_y) {
      const float mrdx = msfvy(i, j) * rdx;
      const int jp = min(jde - 1, j), jm = max(jds, j - 1);
      if (i == ids) {
        const float uw = 0.5f * (ru(i, k, jp) + ru(i, k, jm));
        const float ub = fminf_f(uw, 0.f);
        const float dup = ru(i + 1, k, jp) - ru(i, k, jp);
        const float dum = ru(i + 1, k, jm) - ru(i, k, jm);
        t = t - mrdx * (ub * (v(i + 1, k, j) - v(i, k, j)) + 0.5f * v(i, k, j) * (dup + dum));
      } else {
        const float uw = 0.5f * (ru(i + 1, k, jp) + ru(i + 1, k, jm));
        const float ub = fmaxf_f(uw, 0.f);
        const float dup = ru(i + 1, k, jp) - ru(i, k, jp);
        const float dum = ru(i + 1, k, jm) - ru(i, k, jm);
        t = t - mrdx * (ub * (v(i, k, j) - v(i - 1, k, j)) + 0.5f * v(i, k, j) * (dup + dum));
      }
    }
    auto vf = [&](int kk) -> float {
      if (kk == m.kts || kk == m.kte) return 0.f;
      if (kk == m.kts + 1 || kk == ktf)
        return 0.5f * (rom(i, kk, j) + rom(i, kk, j - 1)) * (fzm(kk) * v(i, kk, j) + fzp(kk) * v(i, kk - 1, j));
      float vel = 0.5f * (rom(i, kk, j) + rom(i, kk, j - 1));
      return vel * flux3(v(i, kk - 2, j), v(i, kk - 1, j), v(i, kk, j), v(i, kk + 1, j), -vel);
    };
    t = t - (msfvy(i, j) / msfvx(i, j)) * rdzw(k) * (vf(k + 1) - vf(k));
  }
  if (FL & TF_PG) {
    F3 ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT), p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB),
       al = f3(m, WRFGPU_AL), php = f3(m, WRFGPU_PHP), cqv = f3(m, WRFGPU_CQV);
    F2 muv = f2(m, WRFGPU_MUV), mu = f2(m, WRFGPU_MU_2);
    F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP),
       rdnw = f1(m, WRFGPU_RDNW);
    const int kde = m.kde;
    auto dpn = [&](int kk) -> float {
      if (kk == kde) {
        if (m.cf.top_lid)
          return .5f * (m.cfn * (p(i, kde - 1, j - 1) + p(i, kde - 1, j)) + m.cfn1 * (p(i, kde - 2, j - 1) + p(i, kde - 2, j)));
        return 0.f;
      }
      if (kk == 1)
        return .5f * (m.cf1 * (p(i, 1, j - 1) + p(i, 1, j)) + m.cf2 * (p(i, 2, j - 1) + p(i, 2, j)) +
                      m.cf3 * (p(i, 3, j - 1) + p(i, 3, j)));
      return .5f * (fnm(kk) * (p(i, kk, j - 1) + p(i, kk, j)) + fnp(kk) * (p(i, kk - 1, j - 1) + p(i, kk - 1, j)));
    };
    float dpy = (msfvy(i, j) / msfvx(i, j)) * .5f * rdy * (c1h(k) * muv(i, j) + c2h(k)) *
                ((ph(i, k + 1, j) - ph(i, k + 1, j - 1) + ph(i, k, j) - ph(i, k, j - 1)) +
                 (alt(i, k, j) + alt(i, k, j - 1)) * (p(i, k, j) - p(i, k, j - 1)) +
                 (al(i, k, j) + al(i, k, j - 1)) * (pb(i, k, j) - pb(i, k, j - 1)));
    dpy = dpy + (msfvy(i, j) / msfvx(i, j)) * rdy * (php(i, k, j) - php(i, k, j - 1)) *
                    (rdnw(k) * (dpn(k + 1) - dpn(k)) - .5f * ((c1h(k) * mu(i, j - 1)) + (c1h(k) * mu(i, j))));
    if (inner_y) t = t - cqv(i, k, j) * dpy;
  }
  if ((FL & TF_COR) && inner_y) {
    F2 f = f2(m, WRFGPU_F), e = f2(m, WRFGPU_E), sina = f2(m, WRFGPU_SINA);
    t = t - (msfvy(i, j) / msfvx(i, j)) * 0.5f * (f(i, j) + f(i, j - 1)) * 0.25f *
                (ru(i, k, j) + ru(i + 1, k, j) + ru(i, k, j - 1) + ru(i + 1, k, j - 1)) +
        (msfvy(i, j) / msfvx(i, j)) * 0.5f * (e(i, j) + e(i, j - 1)) * 0.5f * (sina(i, j) + sina(i, j - 1)) * 0.25f *
            (rw(i, k + 1, j - 1) + rw(i, k, j - 1) + rw(i, k + 1, j) + rw(i, k, j));
  }
  if ((FL & TF_CURV) && inner_y) {
    F3 u = f3(m, WRFGPU_U_2);
    F2 msfuy = f2(m, WRFGPU_MSFUY);
    auto vxgm = [&](int jj) {
      return 0.5f * (u(i, k, jj) + u(i + 1, k, jj)) * (msfvx(i, jj + 1) - msfvx(i, jj)) * rdy -
             0.5f * (v(i, k, jj) + v(i, k, jj + 1)) * (msfuy(i + 1, jj) - msfuy(i, jj)) * rdx;
    };
    t = t - 0.5f * (vxgm(j) + vxgm(j - 1)) * 0.25f * (ru(i, k, j) + ru(i + 1, k, j) + ru(i, k, j - 1) + ru(i + 1, k, j - 1)) -
        (msfvy(i, j) / msfvx(i, j)) * v(i, k, j) * RERADIUS * 0.25f *
            (rw(i, k + 1, j - 1) + rw(i, k, j - 1) + rw(i, k + 1, j) + rw(i, k, j));
  }
  tend(i, k, j) = t;
}

template <int FL>
__global__ void __launch_bounds__(BX* BY) k_tend_v(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  tend_v_point<FL>(m, bp.i, bp.j, bp.k);
}


// ---------------------------------------------------------------- rw_tend
// Column form: pg_buoy_w overwrites cqw(k) with 1/(1+cqw(k)) after the
// k = kde point has read the original cqw(kde-1), so each column is walked
// in order by one thread.  WCQ = false leaves cqw as it is (the edge-strip
// recomputation, which runs before the step's column kernel); it may then
// form any level range k0..k1 on its own (one level per thread), the values
// the column walk carries from the levels below loaded at the start.
template <int FL, bool WCQ = true>
__device__ __forceinline__ void tend_w_column(const Mem& m, const int i, const int j, int k0 = -1, int k1 = -1) {
  static_assert(WCQ || FL == TF_ALL, "level ranges are for the whole rk_tendency");
  if (k0 < 0) { k0 = m.kts; k1 = m.kte; }
  F3 tend = f3(m, WRFGPU_RW_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(m.kte, m.kde - 1);
  const bool in_acc = i >= m.its && i <= itf && j >= m.jts && j <= jtf;
  if (!in_acc) {
    if ((FL & TF_ZERO) && in_zero)
      for (int k = k0; k <= k1; ++k) tend(i, k, j) = 0.f;
    return;
  }
  F3 w = f3(m, WRFGPU_W_2), ru = f3(m, WRFGPU_RU), rv = f3(m, WRFGPU_RV), rom = f3(m, WRFGPU_WW);
  F3 p = f3(m, WRFGPU_P), cqw = f3(m, WRFGPU_CQW);
  F2 msftx = f2(m, WRFGPU_MSFTX), msfty = f2(m, WRFGPU_MSFTY);
  F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzu = f1(m, WRFGPU_RDN), rdnw = f1(m, WRFGPU_RDNW),
     c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F);
  const float rdx = m.rdx, rdy = m.rdy;
  const int kde = m.kde;
  // open lateral boundaries (module_advect_em.F:4784-5096, radiation :5689-5841)
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const bool ydiv = (!oys || j >= m.jds + 1) && (!oye || j <= m.jde - 2);
  const bool xdiv = (!oxs || i >= m.ids + 1) && (!oxe || i <= m.ide - 2);
  const float cqw_top = cqw(i, kde - 1, j);  // read before the k = kde-1 overwrite below
  auto vf = [&](int kk) -> float {
    if (kk == m.kts + 1 || kk == ktf + 1) return 0.25f * (rom(i, kk, j) + rom(i, kk - 1, j)) * (w(i, kk, j) + w(i, kk - 1, j));
    float vel = 0.5f * (rom(i, kk, j) + rom(i, kk - 1, j));
    return vel * flux3(w(i, kk - 2, j), w(i, kk - 1, j), w(i, kk, j), w(i, kk + 1, j), -vel);
  };
  // column constants, formed in the order of the per-level expressions
  const float mrdy = msftx(i, j) * rdy, mrdx = msftx(i, j) * rdx;
  const float rmg = (1.f / msfty(i, j)) * G;
  const float ratio = msftx(i, j) / msfty(i, j);
  float e_c = 0.f, cosa05 = 0.f, rsina05 = 0.f;
  if (FL & TF_COR) {
    e_c = f2(m, WRFGPU_E)(i, j);
    cosa05 = f2(m, WRFGPU_COSA)(i, j) * 0.5f;
    rsina05 = ratio * f2(m, WRFGPU_SINA)(i, j) * 0.5f;
  }
  const float ratio05 = ratio * 0.5f;
  float muf_c = 0.f, mub_c = 0.f;
  if (FL & TF_PG) { muf_c = f2(m, WRFGPU_MU_2)(i, j); mub_c = f2(m, WRFGPU_MUB)(i, j); }
  // the vertical flux of face k+1 is the lower face of level k+1
  float vf_lo = (FL & TF_ADV) && max(k0, m.kts + 1) <= ktf + 1 ? vf(max(k0, m.kts + 1)) : 0.f;
  // values of levels k, k-1, k-2 of the mass fluxes (and of u, v, p) at the
  // points the w-point stencils read, carried down the column instead of
  // re-read (the same values, so the same bits)
  F3 u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2);
  float ru0 = 0.f, ru1 = 0.f, ru0m = 0.f, ru1m = 0.f, ru0mm = 0.f, ru1mm = 0.f;  // ru(i | i+1, k | k-1 | k-2, j)
  float rv0 = 0.f, rv1 = 0.f, rv0m = 0.f, rv1m = 0.f, rv0mm = 0.f, rv1mm = 0.f;  // rv(i, k.., j | j+1)
  float u0 = 0.f, u1 = 0.f, u0m = 0.f, u1m = 0.f, v0 = 0.f, v1 = 0.f, v0m = 0.f, v1m = 0.f;
  float pk = 0.f, pkm = 0.f;
  if (k0 - 1 >= m.kts) {  // a range starting above kts: the carried values of the levels below
    ru0m = ru(i, k0 - 1, j); ru1m = ru(i + 1, k0 - 1, j); rv0m = rv(i, k0 - 1, j); rv1m = rv(i, k0 - 1, j + 1);
    if (FL & TF_CURV) { u0m = u(i, k0 - 1, j); u1m = u(i + 1, k0 - 1, j); v0m = v(i, k0 - 1, j); v1m = v(i, k0 - 1, j + 1); }
    if (FL & TF_PG) pkm = p(i, k0 - 1, j);
    if (k0 - 2 >= m.kts) {
      ru0mm = ru(i, k0 - 2, j); ru1mm = ru(i + 1, k0 - 2, j); rv0mm = rv(i, k0 - 2, j); rv1mm = rv(i, k0 - 2, j + 1);
    }
  }
  for (int k = k0; k <= k1; ++k) {
    ru0 = ru(i, k, j); ru1 = ru(i + 1, k, j); rv0 = rv(i, k, j); rv1 = rv(i, k, j + 1);
    if (FL & TF_CURV) { u0 = u(i, k, j); u1 = u(i + 1, k, j); v0 = v(i, k, j); v1 = v(i, k, j + 1); }
    if (FL & TF_PG) pk = p(i, k, j);
    float t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
    if (k >= m.kts + 1 && k <= ktf + 1) {
      if (FL & TF_ADV) {
        auto fy = [&](int jj, float r_k, float r_km, float r_kmm) {
          float vel = (k <= ktf) ? fzm(k) * r_k + fzp(k) * r_km : (2.f - fzm(k - 1)) * r_km - fzp(k - 1) * r_kmm;
          const int o = open_order_mass(jj, oys, oye, m.jds, m.jde);
          if (o == 2) return 0.5f * vel * (w(i, k, jj) + w(i, k, jj - 1));
          if (o == 3) return vel * flux3(w(i, k, jj - 2), w(i, k, jj - 1), w(i, k, jj), w(i, k, jj + 1), vel);
          return vel * flux5(w(i, k, jj - 3), w(i, k, jj - 2), w(i, k, jj - 1), w(i, k, jj), w(i, k, jj + 1), w(i, k, jj + 2), vel);
        };
        if (ydiv) t = t - mrdy * (fy(j + 1, rv1, rv1m, rv1mm) - fy(j, rv0, rv0m, rv0mm));
        auto fx = [&](int ii, float r_k, float r_km, float r_kmm) {
          float vel = (k <= ktf) ? fzm(k) * r_k + fzp(k) * r_km : (2.f - fzm(k - 1)) * r_km - fzp(k - 1) * r_kmm;
          const int o = open_order_mass(ii, oxs, oxe, m.ids, m.ide);
          if (o == 2) return 0.5f * vel * (w(ii, k, j) + w(ii - 1, k, j));
          if (o == 3) return vel * flux3(w(ii - 2, k, j), w(ii - 1, k, j), w(ii, k, j), w(ii + 1, k, j), vel);
          return vel * flux5(w(ii - 3, k, j), w(ii - 2, k, j), w(ii - 1, k, j), w(ii, k, j), w(ii + 1, k, j), w(ii + 2, k, j), vel);
        };
        if (xdiv) t = t - mrdx * (fx(i + 1, ru1, ru1m, ru1mm) - fx(i, ru0, ru0m, ru0mm));
        // radiation conditions of the open boundary rows: face sums and
        // differences of a mass flux between the own point (a) and its +i /
        // +j neighbour (b), the top level extrapolated
        if ((oxs && i == m.ids) || (oxe && i == m.ide - 1) || (oys && j == m.jds) || (oye && j == m.jde - 1)) {
          auto psum = [&](float a0, float b0, float am, float bm, float amm, float bmm) {
            return (k <= ktf) ? fzm(k) * (a0 + b0) + fzp(k) * (am + bm)
                              : (2.f - fzm(k - 1)) * (am + bm) - fzp(k - 1) * (amm + bmm);
          };
          auto pdif = [&](float a0, float b0, float am, float bm, float amm, float bmm) {
            return (k <= ktf) ? fzm(k) * (b0 - a0) + fzp(k) * (bm - am)
                              : (2.f - fzm(k - 1)) * (bm - am) - fzp(k - 1) * (bmm - amm);
          };
          if (oxs && i == m.ids) {
            const float ub = fminf_f(0.5f * psum(ru0, ru1, ru0m, ru1m, ru0mm, ru1mm), 0.f);
            t = t - rdx * (ub * (w(i + 1, k, j) - w(i, k, j)) + w(i, k, j) * pdif(ru0, ru1, ru0m, ru1m, ru0mm, ru1mm));
          }
          if (oxe && i == m.ide - 1) {
            const float ub = fmaxf_f(0.5f * psum(ru0, ru1, ru0m, ru1m, ru0mm, ru1mm), 0.f);
            t = t - rdx * (ub * (w(i, k, j) - w(i - 1, k, j)) + w(i, k, j) * pdif(ru0, ru1, ru0m, ru1m, ru0mm, ru1mm));
          }
          if (oys && j == m.jds) {
            const float vb = fminf_f(0.5f * psum(rv0, rv1, rv0m, rv1m, rv0mm, rv1mm), 0.f);
            t = t - rdy * (vb * (w(i, k, j + 1) - w(i, k, j)) + w(i, k, j) * pdif(rv0, rv1, rv0m, rv1m, rv0mm, rv1mm));
          }
          if (oye && j == m.jde - 1) {
            const float vb = fmaxf_f(0.5f * psum(rv0, rv1, rv0m, rv1m, rv0mm, rv1mm), 0.f);
            t = t - rdy * (vb * (w(i, k, j) - w(i, k, j - 1)) + w(i, k, j) * pdif(rv0, rv1, rv0m, rv1m, rv0mm, rv1mm));
          }
        }
        if (k <= ktf) {
          const float vf_hi = vf(k + 1);
          t = t - rdzu(k) * (vf_hi - vf_lo);
          vf_lo = vf_hi;
        } else {
          t = t + 2.f * rdzu(k - 1) * (vf_lo);
        }
      }
    }
    if (FL & TF_PG) {
      if (k == kde) {
        float cq1 = 1.f / (1.f + cqw_top);
        float cq2 = cqw_top * cq1;
        t = t + rmg * (cq1 * 2.f * rdnw(k - 1) * (-pkm) - (c1f(k) * muf_c) - cq2 * (c1f(k) * mub_c + c2f(k)));
      } else if (k >= 2) {
        const float cqk = cqw(i, k, j);
        float cq1 = 1.f / (1.f + cqk);
        float cq2 = cqk * cq1;
        if (WCQ) cqw(i, k, j) = cq1;
        t = t + rmg * (cq1 * rdzu(k) * (pk - pkm) - (c1f(k) * muf_c) - cq2 * (c1f(k) * mub_c + c2f(k)));
      }
    }
    // w_damp with w_damping = 1 (module_big_step_utilities_em.F:2687-2691),
    // after pg_buoy_w and before coriolis as rk_tendency calls them; part of
    // the whole rk_tendency only (the single-routine calls leave it out)
    if (FL == TF_ALL && m.cf.w_damping == 1 && k >= 2 && k <= kde - 1) {
      const float mutw = f2(m, WRFGPU_MUT)(i, j);
      const float vert_cfl = fabsf(rom(i, k, j) / (c1f(k) * mutw + c2f(k)) * rdnw(k) * m.dt);
      if (vert_cfl > W_BETA)
        t = t - sgn1(w(i, k, j)) * W_ALPHA * (vert_cfl - m.cf.w_crit_cfl) * (c1f(k) * mutw + c2f(k));
    }
    if (k >= m.kts + 1 && k <= ktf) {
      if (FL & TF_COR) {
        t = t + e_c * (cosa05 * (fzm(k) * (ru0 + ru1) + fzp(k) * (ru0m + ru1m)) -
                       rsina05 * (fzm(k) * (rv0 + rv1) + fzp(k) * (rv0m + rv1m)));
      }
    }
    if (k >= max(2, m.kts) && k <= ktf) {
      if (FL & TF_CURV) {
        t = t + RERADIUS * (0.5f * (fzm(k) * (ru0 + ru1) + fzp(k) * (ru0m + ru1m)) *
                                0.5f * (fzm(k) * (u0 + u1) + fzp(k) * (u0m + u1m)) +
                            ratio05 * (fzm(k) * (rv0 + rv1) + fzp(k) * (rv0m + rv1m)) *
                                0.5f * (fzm(k) * (v0 + v1) + fzp(k) * (v0m + v1m)));
      }
    }
    tend(i, k, j) = t;
    ru0mm = ru0m; ru1mm = ru1m; ru0m = ru0; ru1m = ru1;
    rv0mm = rv0m; rv1mm = rv1m; rv0m = rv0; rv1m = rv1;
    u0m = u0; u1m = u1; v0m = v0; v1m = v1;
    pkm = pk;
  }
}

template <int FL>
__global__ void __launch_bounds__(BX* BY, 5) k_tend_w(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  tend_w_column<FL>(m, bp.i, bp.j);
}

// ---------------------------------------------------------------- t_tend
template <int FL>
__device__ __forceinline__ void tend_t_point(const Mem& m, const int i, const int j, const int k) {
  F3 tend = f3(m, WRFGPU_T_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte && k >= m.kts && k <= m.kte;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(m.kte, m.kde - 1);
  if ((FL & TF_ZERO) && in_zero) {
    // zero_tend of the *_save arrays at the points small_step_prep does not
    // overwrite (module_em.F:395-428; module_small_step_em.F:170-245).
    const bool kt = k == m.kde, ie = i == m.ide, je = j == m.jde;
    if (kt || je) f3(m, WRFGPU_U_SAVE)(i, k, j) = 0.f;
    if (kt || ie) f3(m, WRFGPU_V_SAVE)(i, k, j) = 0.f;
    if (kt || ie || je) f3(m, WRFGPU_T_SAVE)(i, k, j) = 0.f;
    if (ie || je) { f3(m, WRFGPU_W_SAVE)(i, k, j) = 0.f; f3(m, WRFGPU_PH_SAVE)(i, k, j) = 0.f; }
    if (k == m.kts && (ie || je)) f2(m, WRFGPU_MU_SAVE)(i, j) = 0.f;
  }
  const bool in_acc = i >= m.its && i <= itf && j >= m.jts && j <= jtf && k >= m.kts && k <= ktf;
  if (!in_acc) {
    if ((FL & TF_ZERO) && in_zero) tend(i, k, j) = 0.f;
    return;
  }
  float t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
  if (FL & TF_ADV) {
    // advect_scalar ( t, t, t_tend, ... ): the old field is theta itself
    const F3 fld = f3(m, WRFGPU_T_2);
    const ScalarAdv a{fld, fld, f3(m, WRFGPU_RU), f3(m, WRFGPU_RV), f3(m, WRFGPU_WW), f2(m, WRFGPU_MSFTX),
                      f1(m, WRFGPU_FNM), f1(m, WRFGPU_FNP), f1(m, WRFGPU_RDNW)};
    t = adv_scalar_point(m, a, t, i, j, k);
  }
  tend(i, k, j) = t;
}

template <int FL>
__global__ void __launch_bounds__(BX* BY) k_tend_t(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  tend_t_point<FL>(m, bp.i, bp.j, bp.k);
}


// ---------------------------------------------------------------- ph_tend
template <int FL>
__device__ __forceinline__ void tend_ph_point(const Mem& m, const int i, const int j, const int k) {
  F3 tend = f3(m, WRFGPU_PH_TEND);
  const bool in_zero = i >= m.its && i <= m.ite && j >= m.jts && j <= m.jte && k >= m.kts && k <= m.kte;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1);
  const int kte = m.kte, kde = m.kde;
  const bool in_acc = i >= m.its && i <= itf && j >= m.jts && j <= jtf && k >= 2 && k <= kte;
  if (!in_acc) {
    if ((FL & TF_ZERO) && in_zero) tend(i, k, j) = 0.f;
    return;
  }
  if (!(FL & TF_ADV)) return;
  float t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
  F3 u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2), ww = f3(m, WRFGPU_WW), ph = f3(m, WRFGPU_PH_2),
     phb = f3(m, WRFGPU_PHB), w = f3(m, WRFGPU_W_2);
  F2 mut = f2(m, WRFGPU_MUT), muuf = f2(m, WRFGPU_MUU), muvf = f2(m, WRFGPU_MUV), msfux = f2(m, WRFGPU_MSFUX),
     msfvy = f2(m, WRFGPU_MSFVY), msfty = f2(m, WRFGPU_MSFTY);
  F1 c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F), fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP),
     rdnw = f1(m, WRFGPU_RDNW);
  // vertical advection of ph (:1396-1428)
  if (k <= kte - 1) {
    if (m.cf.phi_adv_z == 2) {
      auto wdwn = [&](int kk) { return rdnw(kk - 1) * (ph(i, kk, j) - ph(i, kk - 1, j) + phb(i, kk, j) - phb(i, kk - 1, j)); };
      t = t - ww(i, k, j) * (fnm(k) * wdwn(k + 1) + fnp(k) * wdwn(k));
    } else {
      auto wdwn = [&](int kk) {
        return .5f * (ww(i, kk, j) + ww(i, kk - 1, j)) * rdnw(kk - 1) * (ph(i, kk, j) - ph(i, kk - 1, j) + phb(i, kk, j) - phb(i, kk - 1, j));
      };
      t = t - (fnm(k) * wdwn(k + 1) + fnp(k) * wdwn(k));
    }
  }
  // "gw" term (:1432-1446)
  if (m.cf.non_hydrostatic) {
    if (k == kde) t = 0.f;
    t = t + (c1f(k) * mut(i, j) + c2f(k)) * G * w(i, k, j) / msfty(i, j);
  }
  // horizontal advection (:1768-2075): the 6th-order centred stencil on
  // ph + phb, next to an open boundary 4th order two rows in and 2nd order
  // one row in, nothing on the boundary row itself; y, then x
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const int ids = m.ids, ide = m.ide, jds = m.jds, jde = m.jde;
  auto order = [](int c, bool os, bool oe, int lo, int hi) {
    if (os && c == lo) return 0;
    if (oe && c == hi - 1) return 0;
    if ((os && c == lo + 1) || (oe && c == hi - 2)) return 2;
    if ((os && c == lo + 2) || (oe && c == hi - 3)) return 4;
    return 6;
  };
  const float cfn = m.cfn, cfn1 = m.cfn1;
  const bool top = k == kte;
  auto term = [&](int di, int dj, int ord) -> float {
    // the two face mass fluxes of the direction and the metric factor
    float fp, fm, c;
    if (dj) {
      auto vv = [&](int jj) {
        return top ? (cfn * v(i, k - 1, jj) + cfn1 * v(i, k - 2, jj)) : (v(i, k, jj) + v(i, k - 1, jj));
      };
      c = (top ? 0.5f : 0.25f) * m.rdy / msfty(i, j);
      fp = (c1f(k) * muvf(i, j + 1) + c2f(k)) * vv(j + 1) * msfvy(i, j + 1);
      fm = (c1f(k) * muvf(i, j) + c2f(k)) * vv(j) * msfvy(i, j);
    } else {
      auto uu = [&](int ii) {
        return top ? (cfn * u(ii, k - 1, j) + cfn1 * u(ii, k - 2, j)) : (u(ii, k, j) + u(ii, k - 1, j));
      };
      c = (top ? 0.5f : 0.25f) * m.rdx / msfty(i, j);
      fp = (c1f(k) * muuf(i + 1, j) + c2f(k)) * uu(i + 1) * msfux(i + 1, j);
      fm = (c1f(k) * muuf(i, j) + c2f(k)) * uu(i) * msfux(i, j);
    }
    auto P = [&](int s) { return ph(i + s * di, k, j + s * dj); };
    auto B = [&](int s) { return phb(i + s * di, k, j + s * dj); };
    if (ord == 6)
      return c * ((fp + fm) * (1.f / 60.f) *
                  (45.f * (P(1) - P(-1)) - 9.f * (P(2) - P(-2)) + (P(3) - P(-3)) + 45.f * (B(1) - B(-1)) -
                   9.f * (B(2) - B(-2)) + (B(3) - B(-3))));
    if (ord == 4)
      return c * ((fp + fm) * (1.f / 12.f) *
                  (8.f * (P(1) - P(-1)) - (P(2) - P(-2)) + 8.f * (B(1) - B(-1)) - (B(2) - B(-2))));
    return c * (fp * (B(1) - B(0) + P(1) - P(0)) + fm * (B(0) - B(-1) + P(0) - P(-1)));
  };
  const int oy = order(j, oys, oye, jds, jde), ox = order(i, oxs, oxe, ids, ide);
  if (oy) t = t - term(0, 1, oy);
  if (ox) t = t - term(1, 0, ox);
  // lateral open boundary terms (:2077-2176), ph_old is ph in rk_tendency
  if ((oys && j == jds) || (oye && j == jde - 1)) {
    const int kz = min(k, kde - 1);
    const float vb = .5f * (fnm(kz) * (v(i, kz, j + 1) + v(i, kz, j)) + fnp(kz) * (v(i, kz - 1, j + 1) + v(i, kz - 1, j)));
    if (j == jds) t = t - m.rdy * (c1f(k) * mut(i, j) + c2f(k)) * (fminf_f(vb, 0.f) * (ph(i, k, j + 1) - ph(i, k, j)));
    else t = t - m.rdy * (c1f(k) * mut(i, j) + c2f(k)) * (fmaxf_f(vb, 0.f) * (ph(i, k, j) - ph(i, k, j - 1)));
  }
  if ((oxs && i == ids) || (oxe && i == ide - 1)) {
    const F2 msftx = f2(m, WRFGPU_MSFTX);
    // the west boundary takes its top level at kde, the east one at kde-1 (:2137, :2163)
    const int kz = (i == ids) ? k : (k < kde ? k : kde - 1);
    const float ub = .5f * (fnm(kz) * (u(i + 1, kz, j) + u(i, kz, j)) + fnp(kz) * (u(i + 1, kz - 1, j) + u(i, kz - 1, j)));
    if (i == ids)
      t = t - (msftx(i, j) / msfty(i, j)) * m.rdx * (c1f(k) * mut(i, j) + c2f(k)) * (fminf_f(ub, 0.f) * (ph(i + 1, k, j) - ph(i, k, j)));
    else
      t = t - (msftx(i, j) / msfty(i, j)) * m.rdx * (c1f(k) * mut(i, j) + c2f(k)) * (fmaxf_f(ub, 0.f) * (ph(i, k, j) - ph(i - 1, k, j)));
  }
  tend(i, k, j) = t;
}

template <int FL>
__global__ void __launch_bounds__(BX* BY) k_tend_ph(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  tend_ph_point<FL>(m, bp.i, bp.j, bp.k);
}


// ---------------------------------------------------------------- edge strips
// The large step's tendencies at the points next to an open boundary
// (open_adv.cuh), recomputed with the point functions: u, v, theta and ph
// after the tile kernels, from the same inputs, overwriting theirs; w before
// its tile kernel, which overwrites cqw and leaves the strip's rw_tend alone.
__global__ void __launch_bounds__(STRIP_THREADS) k_strip_tend(StripLaunch L) {
  const StripPos sp = strip_pos(L);
  const Mem& m = block_member(L.mem, sp.m);
  if (!sp.valid) return;
  tend_u_point<TF_ALL>(m, sp.i, sp.j, sp.k);
  tend_v_point<TF_ALL>(m, sp.i, sp.j, sp.k);
  tend_t_point<TF_ZERO | TF_ADV>(m, sp.i, sp.j, sp.k);
  tend_ph_point<TF_ZERO | TF_ADV>(m, sp.i, sp.j, sp.k);
}
__global__ void __launch_bounds__(STRIP_THREADS) k_strip_tend_w(StripLaunch L) {
  const StripPos sp = strip_pos(L);
  const Mem& m = block_member(L.mem, sp.m);
  if (!sp.valid || sp.k < m.kts || sp.k > m.kte) return;
  tend_w_column<TF_ALL, false>(m, sp.i, sp.j, sp.k, sp.k);
}
void launch_strip_tend(const StripLaunch& L, int nb, cudaStream_t s) {
  if (nb > 0) k_strip_tend<<<nb, STRIP_THREADS, 0, s>>>(L);
}
void launch_strip_tend_w(const StripLaunch& L, int nb, cudaStream_t s) {
  if (nb > 0) k_strip_tend_w<<<nb, STRIP_THREADS, 0, s>>>(L);
}

// ---------------------------------------------------------------- launchers
#define DISPATCH_FL(KERNEL, GRID, BLOCK, S, FLAGS)                                       \
  switch (FLAGS) {                                                                      \
    case TF_ALL: KERNEL<TF_ALL><<<GRID, BLOCK, 0, S>>>(L); break;                       \
    case TF_ZERO | TF_ADV: KERNEL<TF_ZERO | TF_ADV><<<GRID, BLOCK, 0, S>>>(L); break;   \
    case TF_ADV: KERNEL<TF_ADV><<<GRID, BLOCK, 0, S>>>(L); break;                       \
    case TF_PG: KERNEL<TF_PG><<<GRID, BLOCK, 0, S>>>(L); break;                         \
    case TF_COR: KERNEL<TF_COR><<<GRID, BLOCK, 0, S>>>(L); break;                       \
    case TF_CURV: KERNEL<TF_CURV><<<GRID, BLOCK, 0, S>>>(L); break;                     \
    case TF_ZERO: KERNEL<TF_ZERO><<<GRID, BLOCK, 0, S>>>(L); break;                     \
    default: break;                                                                     \
  }

void launch_tend_u(const Launch& L, int nb, int flags, cudaStream_t s) { DISPATCH_FL(k_tend_u, nb, dim3(BX, BY), s, flags) }
void launch_tend_v(const Launch& L, int nb, int flags, cudaStream_t s) { DISPATCH_FL(k_tend_v, nb, dim3(BX, BY), s, flags) }
void launch_tend_w(const Launch& L, int nb, int flags, cudaStream_t s) { DISPATCH_FL(k_tend_w, nb, dim3(BX, BY), s, flags) }
void launch_tend_t(const Launch& L, int nb, int flags, cudaStream_t s) { DISPATCH_FL(k_tend_t, nb, dim3(BX, BY), s, flags) }
void launch_tend_ph(const Launch& L, int nb, int flags, cudaStream_t s) { DISPATCH_FL(k_tend_ph, nb, dim3(BX, BY), s, flags) }

}  // namespace wrfgpu
