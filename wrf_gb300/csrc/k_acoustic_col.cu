// Column-marching forms of the acoustic-step kernels used by the fused
// solver (the routine kernels of k_small.cu stay for routine-level calls).
//
// A block owns a TX x TY tile of columns and each thread marches its column
// up k.  The inputs of level k+1 are loaded into registers before level k
// is computed and stored, so every thread keeps a whole level of loads in
// flight instead of waiting behind its own stores (the stores may alias the
// loads as far as the compiler knows).  The per-point arithmetic is the
// reference's, in its order: results are bit-identical to k_small.cu.
//
//   k_sumflux_p_rho_col  sumflux (module_small_step_em.F:1473-1633) on the
//                        u, v and w points of the column + calc_p_rho
//                        (:438-568) on its mass points; tiles cover the
//                        staggered extents so the u point i = ide and the v
//                        point j = jde are included.
#include "common.cuh"
#include "kernels.h"
#include "ffmath.h"

namespace wrfgpu {

namespace {
struct SFLevel {
  float rum, rvm, wwm;      // accumulated mass fluxes (0 at the first iteration)
  float u, v, ww;           // current u, v, omega
  float us, vs, ww1;        // linear parts (last iteration only)
  float ph1, alt, t2, t1, c2a, pm1;  // calc_p_rho inputs (ph at k+1)
};
}  // namespace

// One block per (staggered tile, chunk of levels: gridDim.y chunks); the
// levels are independent but for ph(k), carried from the level below within
// a chunk and read at a chunk's first level.
template <int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_sumflux_p_rho_col(TileLaunch L, int rk_step, int iteration) {
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const Stage st = stage_of(m, rk_step);
  if (iteration > st.nsmall) return;  // members with fewer acoustic steps
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  if (i > m.ite || j > m.jte) return;
  const int ns = st.nsmall;
  const bool first = iteration == 1, last = iteration == ns;
  const int mini = min(m.ide - 1, m.ite), minj = min(m.jde - 1, m.jte), mink = min(m.kde - 1, m.kte);
  const int kts = m.kts, kte = m.kte;
  const bool ucol = j <= minj, vcol = i <= mini, mcol = ucol && vcol;
  MassImages img;  // the halo images of al and p (mass columns)
  img.init(m, i, j);
  F3 ru_m = f3(m, WRFGPU_RU_M), rv_m = f3(m, WRFGPU_RV_M), ww_m = f3(m, WRFGPU_WW_M);
  F3 u2 = f3(m, WRFGPU_U_2), v2 = f3(m, WRFGPU_V_2), ww = f3(m, WRFGPU_WW), us = f3(m, WRFGPU_U_SAVE),
     vs = f3(m, WRFGPU_V_SAVE), ww1 = f3(m, WRFGPU_WW1);
  F3 al = f3(m, WRFGPU_AL), p = f3(m, WRFGPU_P), ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT),
     t_2 = f3(m, WRFGPU_T_2), t_1 = f3(m, WRFGPU_T_SAVE), c2a = f3(m, WRFGPU_C2A), pm1 = f3(m, WRFGPU_PM1);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), rdnw = f1(m, WRFGPU_RDNW);
  float muu = 0.f, muv = 0.f, msfuy = 1.f, msfvx_inv = 1.f, muij = 0.f, mutij = 0.f;
  if (last && ucol) { muu = f2(m, WRFGPU_MUU).ro(i, j); msfuy = f2(m, WRFGPU_MSFUY).ro(i, j); }
  if (last && vcol) { muv = f2(m, WRFGPU_MUV).ro(i, j); msfvx_inv = f2(m, WRFGPU_MSFVX_INV).ro(i, j); }
  if (mcol) { muij = f2(m, WRFGPU_MU_2).ro(i, j); mutij = f2(m, WRFGPU_MUTS).ro(i, j); }
  const float smdiv = m.smdiv;

  auto load = [&](int k, SFLevel& v) {
    const bool ru_acc = ucol && k <= mink, rv_acc = vcol && k <= mink, mass = mcol && k <= mink;
    v.rum = (!first && ru_acc) ? ru_m(i, k, j) : 0.f;
    v.rvm = (!first && rv_acc) ? rv_m(i, k, j) : 0.f;
    v.wwm = (!first && mcol) ? ww_m(i, k, j) : 0.f;
    v.u = ru_acc ? u2.ro(i, k, j) : 0.f;
    v.v = rv_acc ? v2.ro(i, k, j) : 0.f;
    v.ww = mcol ? ww.ro(i, k, j) : 0.f;
    v.us = (last && ru_acc) ? us.ro(i, k, j) : 0.f;
    v.vs = (last && rv_acc) ? vs.ro(i, k, j) : 0.f;
    v.ww1 = (last && mcol) ? ww1.ro(i, k, j) : 0.f;
    if (mass) {
      v.ph1 = ph.ro(i, k + 1, j);
      v.alt = alt.ro(i, k, j); v.t2 = t_2.ro(i, k, j); v.t1 = t_1.ro(i, k, j); v.c2a = c2a.ro(i, k, j);
      v.pm1 = pm1(i, k, j);
    } else {
      v.ph1 = v.alt = v.t2 = v.t1 = v.c2a = v.pm1 = 0.f;
    }
  };
  const int per = (kte - kts + 1 + (int)gridDim.y - 1) / (int)gridDim.y;
  const int k0 = kts + (int)blockIdx.y * per, k1 = min(kte, k0 + per - 1);
  if (k0 > k1) return;
  SFLevel cur, nxt;
  load(k0, cur);
  float ph_k = mcol ? ph.ro(i, k0, j) : 0.f;
  for (int k = k0; k <= k1; ++k) {
    if (k + 1 <= k1) load(k + 1, nxt);
    const bool ru_acc = ucol && k <= mink, rv_acc = vcol && k <= mink;
    // sumflux
    float rum = cur.rum, rvm = cur.rvm, wwm = cur.wwm;
    if (ru_acc) {
      rum = rum + cur.u;
      if (last) rum = rum / float(ns) + (c1h(k) * muu + c2h(k)) * cur.us / msfuy;
    }
    if (rv_acc) {
      rvm = rvm + cur.v;
      if (last) rvm = rvm / float(ns) + (c1h(k) * muv + c2h(k)) * cur.vs * msfvx_inv;
    }
    if (mcol) {
      wwm = wwm + cur.ww;
      if (last) wwm = wwm / float(ns) + cur.ww1;
    }
    if (first || ru_acc) ru_m(i, k, j) = rum;
    if (first || rv_acc) rv_m(i, k, j) = rvm;
    if (first || mcol) ww_m(i, k, j) = wwm;
    // calc_p_rho on the mass point
    if (mcol && k <= mink) {
      const float a = cur.alt, t1 = cur.t1;
      float alv = -1.f / (c1h(k) * mutij + c2h(k)) * (a * (c1h(k) * muij) + rdnw(k) * (cur.ph1 - ph_k));
      img.store([&](int ii, int jj) { al(ii, k, jj) = alv; });
      float pv = cur.c2a * (a * (cur.t2 - (c1h(k) * muij) * t1) / ((c1h(k) * mutij + c2h(k)) * (T0 + t1)) - alv);
      if (iteration == 0) {
        pm1(i, k, j) = pv;
      } else {
        const float ptmp = pv;
        pv = pv + smdiv * (pv - cur.pm1);
        pm1(i, k, j) = ptmp;
      }
      img.store([&](int ii, int jj) { p(ii, k, jj) = pv; });
      ph_k = cur.ph1;
    }
    cur = nxt;
  }
}

// variant parameter: 10 x blocks per SM + level chunks
void launch_sumflux_p_rho_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, cudaStream_t s, int var) {
  const int p = TUNE_PARAM[TU_SUMF][var], chunks = p % 10;
  if (p / 10 == 4) k_sumflux_p_rho_col<4><<<dim3(nblocks, chunks), dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
  else k_sumflux_p_rho_col<3><<<dim3(nblocks, chunks), dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
}

// ---------------------------------------------------------------------------
// advance_uv (module_small_step_em.F:654-967) on the u and v points of the
// column, plus sumflux's accumulation of ru_m / rv_m left to
// k_sumflux_p_rho_col.  Horizontal neighbours i-1 (u) and j-1 (v) are read
// directly (L1); p and ph of level k are kept from the previous level.
// ---------------------------------------------------------------------------
namespace {
struct UVLevel {
  float u, rut, cqu, v, rvt, cqv;  // own u / v point
  float p1, ph1, pb, php, alt, al;           // (i, j):   p, ph at k+1; the rest at k
  float p1x, ph1x, pbx, phpx, altx, alx;     // (i-1, j)
  float p1y, ph1y, pby, phpy, alty, aly;     // (i, j-1)
};
}  // namespace

template <int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_advance_uv_col(TileLaunch L, int rk_step, int iteration) {
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const Stage st = stage_of(m, rk_step);
  if (iteration > st.nsmall) return;
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  if (i > m.ite || j > m.jte) return;
  const float dts = st.dts_rk;
  const WrfDynConfig& cf = m.cf;
  const int i_start = m.its, i_end = min(m.ite, m.ide - 1), j_start = m.jts, i_endu = m.ite, j_endv = m.jte;
  int i_start_up = i_start, i_end_up = i_endu, j_start_vp = j_start, j_end_vp = j_endv;
  if ((cf.open_xs || cf.symmetric_xs) && m.its == m.ids) i_start_up = i_start_up + 1;
  if ((cf.open_xe || cf.symmetric_xe) && m.ite == m.ide) i_end_up = i_end_up - 1;
  if ((cf.open_ys || cf.symmetric_ys || cf.polar) && m.jts == m.jds) j_start_vp = j_start_vp + 1;
  if ((cf.open_ye || cf.symmetric_ye || cf.polar) && m.jte == m.jde) j_end_vp = j_end_vp - 1;
  int i_start_u_tend = i_start, i_end_u_tend = i_endu, j_start_v_tend = j_start, j_end_v_tend = j_endv;
  if (cf.symmetric_xs && m.its == m.ids) i_start_u_tend = i_start_u_tend + 1;
  if (cf.symmetric_xe && m.ite == m.ide) i_end_u_tend = i_end_u_tend - 1;
  if (cf.symmetric_ys && m.jts == m.jds) j_start_v_tend = j_start_v_tend + 1;
  if (cf.symmetric_ye && m.jte == m.jde) j_end_v_tend = j_end_v_tend - 1;
  const bool upt = j >= j_start && j <= min(m.jte, m.jde - 1) && i >= min(i_start_u_tend, i_start_up) &&
                   i <= max(i_end_u_tend, i_end_up);
  const bool u_tend = upt && i >= i_start_u_tend && i <= i_end_u_tend;
  const bool u_pg = upt && i >= i_start_up && i <= i_end_up;
  const bool vpt = j >= j_start_v_tend && j <= j_end_v_tend && i >= i_start && i <= i_end;
  const bool v_pg = vpt && j >= j_start_vp && j <= j_end_vp;
  if (!upt && !vpt) return;
  F3 p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB), ph = f3(m, WRFGPU_PH_2), php = f3(m, WRFGPU_PHP),
     alt = f3(m, WRFGPU_ALT), al = f3(m, WRFGPU_AL);
  F3 u = f3(m, WRFGPU_U_2), ru_tend = f3(m, WRFGPU_RU_TEND), cqu = f3(m, WRFGPU_CQU);
  F3 v = f3(m, WRFGPU_V_2), rv_tend = f3(m, WRFGPU_RV_TEND), cqv = f3(m, WRFGPU_CQV);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP),
     rdnw = f1(m, WRFGPU_RDNW);
  const float rdx = m.rdx, rdy = m.rdy, emdiv = m.emdiv, cf1 = m.cf1, cf2 = m.cf2, cf3 = m.cf3;
  const int kde = m.kde, k_start = m.kts, k_end = m.kte - 1;
  // per-column factors (the reference's left-to-right products, split where they start)
  F2 MU = f2(m, WRFGPU_MU_2), MUDF = f2(m, WRFGPU_MUDF);
  float ua = 0.f, uc = 0.f, mudf_u = 0.f, muu = 0.f, mu_i = 0.f, mu_im = 0.f;
  float va = 0.f, vc = 0.f, mudf_v = 0.f, muv = 0.f, mu_jm = 0.f;
  if (u_pg) {
    const float msfux = f2(m, WRFGPU_MSFUX).ro(i, j), msfuy = f2(m, WRFGPU_MSFUY).ro(i, j);
    const float dx = 1.f / rdx;
    mudf_u = -emdiv * dx * (MUDF.ro(i, j) - MUDF.ro(i - 1, j)) / msfuy;
    ua = (msfux / msfuy) * .5f * rdx;
    uc = (msfux / msfuy) * rdx;
    muu = f2(m, WRFGPU_MUU).ro(i, j);
    mu_i = MU.ro(i, j); mu_im = MU.ro(i - 1, j);
  }
  if (vpt) {
    const float msfvx_inv = f2(m, WRFGPU_MSFVX_INV).ro(i, j);
    const float dy = 1.f / rdy;
    mudf_v = -emdiv * dy * (MUDF.ro(i, j) - MUDF.ro(i, j - 1)) * msfvx_inv;
    if (v_pg) {
      const float msfvx = f2(m, WRFGPU_MSFVX).ro(i, j), msfvy = f2(m, WRFGPU_MSFVY).ro(i, j);
      va = (msfvy / msfvx) * .5f * rdy;
      vc = (msfvy / msfvx) * rdy;
      muv = f2(m, WRFGPU_MUV).ro(i, j);
      mu_i = MU.ro(i, j); mu_jm = MU.ro(i, j - 1);
    }
  }
  const bool need_x = u_pg, need_y = v_pg, need_c = u_pg || v_pg;
  auto load = [&](int k, UVLevel& d) {
    d.u = upt ? u(i, k, j) : 0.f;
    d.rut = u_tend ? ru_tend.ro(i, k, j) : 0.f;
    d.cqu = u_pg ? cqu.ro(i, k, j) : 0.f;
    d.v = vpt ? v(i, k, j) : 0.f;
    d.rvt = vpt ? rv_tend.ro(i, k, j) : 0.f;
    d.cqv = v_pg ? cqv.ro(i, k, j) : 0.f;
    const bool top = k + 1 <= kde - 1;  // p exists up to kde-1
    if (need_c) {
      d.p1 = top ? p.ro(i, k + 1, j) : 0.f; d.ph1 = ph.ro(i, k + 1, j);
      d.pb = pb.ro(i, k, j); d.php = php.ro(i, k, j); d.alt = alt.ro(i, k, j); d.al = al.ro(i, k, j);
    }
    if (need_x) {
      d.p1x = top ? p.ro(i - 1, k + 1, j) : 0.f; d.ph1x = ph.ro(i - 1, k + 1, j);
      d.pbx = pb.ro(i - 1, k, j); d.phpx = php.ro(i - 1, k, j); d.altx = alt.ro(i - 1, k, j); d.alx = al.ro(i - 1, k, j);
    }
    if (need_y) {
      d.p1y = top ? p.ro(i, k + 1, j - 1) : 0.f; d.ph1y = ph.ro(i, k + 1, j - 1);
      d.pby = pb.ro(i, k, j - 1); d.phpy = php.ro(i, k, j - 1); d.alty = alt.ro(i, k, j - 1); d.aly = al.ro(i, k, j - 1);
    }
  };
  // this block's chunk of levels (gridDim.y chunks); the levels are
  // independent but for the carried p, ph and dpn of the level below
  const int per = (k_end - k_start + 1 + (int)gridDim.y - 1) / (int)gridDim.y;
  const int k0 = k_start + (int)blockIdx.y * per, k1 = min(k_end, k0 + per - 1);
  if (k0 > k1) return;
  // level k0 values of p and ph, and dpn(k0) (dpn(1) has its own formula)
  float p0 = 0.f, ph0 = 0.f, p0x = 0.f, ph0x = 0.f, p0y = 0.f, ph0y = 0.f, dpn_u = 0.f, dpn_v = 0.f;
  if (need_c) { p0 = p.ro(i, k0, j); ph0 = ph.ro(i, k0, j); }
  if (need_x) {
    p0x = p.ro(i - 1, k0, j); ph0x = ph.ro(i - 1, k0, j);
    if (k0 == 1)
      dpn_u = .5f * (cf1 * (p.ro(i, 1, j) + p.ro(i - 1, 1, j)) + cf2 * (p.ro(i, 2, j) + p.ro(i - 1, 2, j)) +
                     cf3 * (p.ro(i, 3, j) + p.ro(i - 1, 3, j)));
    else
      dpn_u = .5f * (fnm(k0) * (p0 + p0x) + fnp(k0) * (p.ro(i, k0 - 1, j) + p.ro(i - 1, k0 - 1, j)));
  }
  if (need_y) {
    p0y = p.ro(i, k0, j - 1); ph0y = ph.ro(i, k0, j - 1);
    if (k0 == 1)
      dpn_v = .5f * (cf1 * (p.ro(i, 1, j) + p.ro(i, 1, j - 1)) + cf2 * (p.ro(i, 2, j) + p.ro(i, 2, j - 1)) +
                     cf3 * (p.ro(i, 3, j) + p.ro(i, 3, j - 1)));
    else
      dpn_v = .5f * (fnm(k0) * (p0 + p0y) + fnp(k0) * (p.ro(i, k0 - 1, j) + p.ro(i, k0 - 1, j - 1)));
  }
  // top value of dpn (kde): zero unless the lid is rigid
  float dpn_u_top = 0.f, dpn_v_top = 0.f;
  if (cf.top_lid) {
    if (need_x)
      dpn_u_top = .5f * (cf1 * (p.ro(i - 1, kde - 1, j) + p.ro(i, kde - 1, j)) + cf2 * (p.ro(i - 1, kde - 2, j) + p.ro(i, kde - 2, j)) +
                         cf3 * (p.ro(i - 1, kde - 3, j) + p.ro(i, kde - 3, j)));
    if (need_y)
      dpn_v_top = .5f * (cf1 * (p.ro(i, kde - 1, j - 1) + p.ro(i, kde - 1, j)) + cf2 * (p.ro(i, kde - 2, j - 1) + p.ro(i, kde - 2, j)) +
                         cf3 * (p.ro(i, kde - 3, j - 1) + p.ro(i, kde - 3, j)));
  }
  UVLevel cur, nxt;
  load(k0, cur);
  for (int k = k0; k <= k1; ++k) {
    if (k + 1 <= k1) load(k + 1, nxt);
    const int kk = k + 1;
    // u
    if (upt) {
      float uv = cur.u;
      if (u_tend) uv = uv + dts * cur.rut;
      float dpn_hi = 0.f;
      if (u_pg) {
        dpn_hi = (kk == kde) ? dpn_u_top : .5f * (fnm(kk) * (cur.p1 + cur.p1x) + fnp(kk) * (p0 + p0x));
        float dpxy = ua * (c1h(k) * muu + c2h(k)) *
                     (((cur.ph1 - cur.ph1x) + (ph0 - ph0x)) + (cur.alt + cur.altx) * (p0 - p0x) +
                      (cur.al + cur.alx) * (cur.pb - cur.pbx));
        dpxy = dpxy + uc * (cur.php - cur.phpx) *
                          (rdnw(k) * (dpn_hi - dpn_u) - .5f * ((c1h(k) * mu_im) + (c1h(k) * mu_i)));
        uv = uv - dts * cur.cqu * dpxy + (c1h(k) * mudf_u);
        dpn_u = dpn_hi;
      }
      u(i, k, j) = uv;
    }
    // v
    if (vpt) {
      float vv = cur.v + dts * cur.rvt;
      if (v_pg) {
        const float dpn_hi = (kk == kde) ? dpn_v_top : .5f * (fnm(kk) * (cur.p1 + cur.p1y) + fnp(kk) * (p0 + p0y));
        float dpxy = va * (c1h(k) * muv + c2h(k)) *
                     (((cur.ph1 - cur.ph1y) + (ph0 - ph0y)) + (cur.alt + cur.alty) * (p0 - p0y) +
                      (cur.al + cur.aly) * (cur.pb - cur.pby));
        dpxy = dpxy + vc * (cur.php - cur.phpy) *
                          (rdnw(k) * (dpn_hi - dpn_v) - .5f * ((c1h(k) * mu_jm) + (c1h(k) * mu_i)));
        vv = vv - dts * cur.cqv * dpxy + (c1h(k) * mudf_v);
        dpn_v = dpn_hi;
      }
      v(i, k, j) = vv;
    }
    p0 = cur.p1; ph0 = cur.ph1; p0x = cur.p1x; ph0x = cur.ph1x; p0y = cur.p1y; ph0y = cur.ph1y;
    cur = nxt;
  }
}

// variant parameter: 10 x blocks per SM + level chunks
void launch_advance_uv_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, cudaStream_t s, int var) {
  const int p = TUNE_PARAM[TU_AUV][var], chunks = p % 10;
  if (p / 10 == 4) k_advance_uv_col<4><<<dim3(nblocks, chunks), dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
  else k_advance_uv_col<3><<<dim3(nblocks, chunks), dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
}



// ---------------------------------------------------------------------------
// advance_mu_t (module_small_step_em.F:969-1175), one thread per mass column:
// pass 1 the column divergence (kept per level) and its sum, then mu, and
// pass 2 omega by upward recursion and theta.  RC: accumulation type of the
// column sum and the recursion (float: the reference; double: mixed form).
// ---------------------------------------------------------------------------
constexpr int KCOL = 129;  // column scratch (kde <= 128)

template <typename RC, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_advance_mu_t_col(TileLaunch L, int rk_step, int iteration) {
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const Stage st = stage_of(m, rk_step);
  if (iteration > st.nsmall) return;
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  const int i_end = min(m.ite, m.ide - 1), j_end = min(m.jte, m.jde - 1);
  if (i > i_end || j > j_end) return;
  const int k_start = m.kts, k_end = m.kte - 1, kde = m.kde;
  const float dts = st.dts_rk, epssm = m.epssm, rdx = m.rdx, rdy = m.rdy;
  F3 ww = f3(m, WRFGPU_WW), ww_1 = f3(m, WRFGPU_WW1), u = f3(m, WRFGPU_U_2), u_1 = f3(m, WRFGPU_U_SAVE),
     v = f3(m, WRFGPU_V_2), v_1 = f3(m, WRFGPU_V_SAVE), t = f3(m, WRFGPU_T_2), t_1 = f3(m, WRFGPU_T_SAVE),
     t_ave = f3(m, WRFGPU_T_2SAVE), ft = f3(m, WRFGPU_T_TEND);
  F2 MU = f2(m, WRFGPU_MU_2), MUT = f2(m, WRFGPU_MUT), MUAVE = f2(m, WRFGPU_MUAVE), MUTS = f2(m, WRFGPU_MUTS),
     muu = f2(m, WRFGPU_MUU), muv = f2(m, WRFGPU_MUV), MUDF = f2(m, WRFGPU_MUDF), MU_TEND = f2(m, WRFGPU_MU_TEND),
     msfuy = f2(m, WRFGPU_MSFUY), msfvx_inv = f2(m, WRFGPU_MSFVX_INV), msftx = f2(m, WRFGPU_MSFTX),
     msfty = f2(m, WRFGPU_MSFTY);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), dnw = f1(m, WRFGPU_DNW), fnm = f1(m, WRFGPU_FNM),
     fnp = f1(m, WRFGPU_FNP), rdnw = f1(m, WRFGPU_RDNW);
  const float mxy = msftx.ro(i, j) * msfty.ro(i, j);
  const float muv0 = muv.ro(i, j), muv1 = muv.ro(i, j + 1), muu0 = muu.ro(i, j), muu1 = muu.ro(i + 1, j);
  const float vi0 = msfvx_inv.ro(i, j), vi1 = msfvx_inv.ro(i, j + 1), uy0 = msfuy.ro(i, j), uy1 = msfuy.ro(i + 1, j);
  // pass 1: dvdxi(k) and dmdt
  struct D1 { float v1, v0, vo1, vo0, u1, u0, uo1, uo0; };
  auto load1 = [&](int k, D1& d) {
    d.v1 = v.ro(i, k, j + 1); d.vo1 = v_1.ro(i, k, j + 1); d.v0 = v.ro(i, k, j); d.vo0 = v_1.ro(i, k, j);
    d.u1 = u.ro(i + 1, k, j); d.uo1 = u_1.ro(i + 1, k, j); d.u0 = u.ro(i, k, j); d.uo0 = u_1.ro(i, k, j);
  };
  float dv[KCOL];
  RC dmdt = RC(0.);
  // the levels' loads are independent: four levels in flight at a time; the
  // sum is still taken in k order
  chunked_levels<4, D1>(k_start, k_end, load1, [&](int k, const D1& cur) {
    const float d = mxy * (rdy * ((cur.v1 + (c1h(k) * muv1 + c2h(k)) * cur.vo1 * vi1) -
                                  (cur.v0 + (c1h(k) * muv0 + c2h(k)) * cur.vo0 * vi0)) +
                           rdx * ((cur.u1 + (c1h(k) * muu1 + c2h(k)) * cur.uo1 / uy1) -
                                  (cur.u0 + (c1h(k) * muu0 + c2h(k)) * cur.uo0 / uy0)));
    dv[k] = d;
    if constexpr (sizeof(RC) == 8) dmdt = fma((RC)dnw(k), (RC)d, dmdt);  // mixed form: one FP64 fma per level
    else dmdt = dmdt + (RC)dnw(k) * (RC)d;
  });
  const float mu_tend = MU_TEND.ro(i, j);
  const float muave = MU(i, j);
  const float mu = (float)((RC)muave + (RC)dts * (dmdt + (RC)mu_tend));
  const float mudf = (float)(dmdt + (RC)mu_tend), muts = MUT.ro(i, j) + mu;
  MassImages img;
  img.init(m, i, j);
  img.store([&](int ii, int jj) { MU(ii, jj) = mu; MUDF(ii, jj) = mudf; MUTS(ii, jj) = muts; });
  MUAVE(i, j) = .5f * ((1.f + epssm) * mu + (1.f - epssm) * muave);
  const float my = msfty.ro(i, j), mx = msftx.ro(i, j);
  const RC rmy = rcp_rc<RC>((RC)my);  // mixed form only
  // pass 2: omega (recursion one level ahead of theta) and theta
  struct D2 { float ww1, t, ft, t1, t1xm, t1xp, t1ym, t1yp, u0, u1, v0, v1; };
  auto load2 = [&](int k, D2& d) {
    d.ww1 = ww_1.ro(i, k, j); d.t = t(i, k, j); d.ft = ft.ro(i, k, j);
    d.t1 = t_1.ro(i, k, j); d.t1xm = t_1.ro(i - 1, k, j); d.t1xp = t_1.ro(i + 1, k, j);
    d.t1ym = t_1.ro(i, k, j - 1); d.t1yp = t_1.ro(i, k, j + 1);
    d.u0 = u.ro(i, k, j); d.u1 = u.ro(i + 1, k, j); d.v0 = v.ro(i, k, j); d.v1 = v.ro(i, k, j + 1);
  };
  RC wwk = (RC)ww(i, 1, j);
  // mixed form: the recursion factored into fmas, c1h (dmdt + mu_tend) + dv
  // times dnw / my (FP64 runs at 1/64 of the FP32 rate on this part)
  const RC dm_mt = (RC)dmdt + (RC)mu_tend;
  // final omega of level 1 (the recursion starts from the unchanged ww(1))
  float wwf_k = ww(i, 1, j) - ww_1.ro(i, 1, j);
  float wdtn_lo = 0.f;  // wdtn(1) = 0
  D2 cur, nxt;
  load2(k_start, cur);
  for (int k = k_start; k <= k_end; ++k) {
    if (k + 1 <= k_end) load2(k + 1, nxt);
    // omega of level k+1 (recursion from level k), needed by wdtn(k+1)
    float wwf_kp1 = 0.f;
    if (k + 1 <= k_end) {
      const int kk = k + 1, kl = kk - 1;
      if constexpr (sizeof(RC) == 8)
        wwk = fma(-fma((RC)c1h(kl), dm_mt, (RC)dv[kk - 1]), (RC)dnw(kk - 1) * rmy, wwk);
      else
        wwk = wwk - (RC)dnw(kk - 1) * (((RC)c1h(kl) * dmdt) + (RC)dv[kk - 1] + ((RC)c1h(kl) * (RC)mu_tend)) / (RC)my;
      wwf_kp1 = (float)wwk - nxt.ww1;
    }
    ww(i, k, j) = wwf_k;
    // theta of level k
    const float tv = cur.t;
    t_ave(i, k, j) = tv;
    float tt = tv + my * dts * cur.ft;
    const float wdtn_hi = (k + 1 == kde) ? 0.f : wwf_kp1 * (fnm(k + 1) * (k + 1 <= k_end ? nxt.t1 : 0.f) + fnp(k + 1) * cur.t1);
    tt = tt - dts * my *
                  (mx * (.5f * rdy * (cur.v1 * (cur.t1yp + cur.t1) - cur.v0 * (cur.t1 + cur.t1ym)) +
                         .5f * rdx * (cur.u1 * (cur.t1xp + cur.t1) - cur.u0 * (cur.t1 + cur.t1xm))) +
                   rdnw(k) * (wdtn_hi - wdtn_lo));
    t(i, k, j) = tt;
    wdtn_lo = wdtn_hi;
    wwf_k = wwf_kp1;
    cur = nxt;
  }
}

// ---------------------------------------------------------------------------
// advance_w (module_small_step_em.F:1178-1469), one thread per mass column.
// Upward pass: at level L, t_2ave(L), the raw right-hand side of L+1, the
// omega advection term that completes rhs(L), and the explicit w and forward
// elimination of level L-1 (which needs rhs(L)); everything the elimination
// reads from neighbouring levels sits in register windows.  Downward pass:
// back substitution and the geopotential update.  RC as above (the mixed
// form keeps a, alpha, gamma in FP64).
// ---------------------------------------------------------------------------
// Level inputs of advance_w staged by TMA: plane index of each field in a
// ring slot (the FP64 a / alpha of the mixed form are read from global
// memory instead, so that form stages the first 13).
enum AwPlane { AW_T2 = 0, AW_T2A, AW_T1, AW_PH, AW_W, AW_RWT, AW_CQW, AW_C2A, AW_ALT, AW_PHT, AW_WW, AW_PH1, AW_PHB,
               AW_A, AW_AL, AW_NPLANE };
// Ring depth: levels L, L+1 resident and L+2, L+3 in flight; at four
// blocks per SM (which the shared memory of four slots does not allow) only
// L+2 is in flight.
template <typename RC, int NSLOT> struct AwCfg {
  static constexpr int NF = sizeof(RC) == 8 ? AW_A : AW_NPLANE;
  using Ring = TileRing<NF, NSLOT>;
};

template <typename RC, int MINB, bool DAMP>
__global__ void __launch_bounds__(TX* TY, MINB) k_advance_w_col(TileLaunch L, int rk_step, int iteration) {
  constexpr int AW_RING = MINB >= 4 ? 3 : 4;
  using Ring = typename AwCfg<RC, AW_RING>::Ring;
  constexpr int NF = AwCfg<RC, AW_RING>::NF;
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const Stage st = stage_of(m, rk_step);
  if (iteration > st.nsmall) return;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx, po = ty * TX + tx;
  const int i = tp.i0 + tx, j = tp.j0 + ty;
  const int i_end = min(m.ite, m.ide - 1), j_end = min(m.jte, m.jde - 1);
  // every thread takes part in the ring's barriers; only columns of the
  // domain compute and store
  const bool act = i <= i_end && j <= j_end;
  const int ic = act ? i : tp.i0, jc = act ? j : tp.j0;  // in-range indices for the column loads
  const int k_end = m.kte - 1, kde = m.kde;
  const float dts = st.dts_rk, epssm = m.epssm, rdx = m.rdx, rdy = m.rdy;

  Ring ring;
  ring.init(smem, 1);
  {
    const int ids[AW_NPLANE] = {WRFGPU_T_2, WRFGPU_T_2SAVE, WRFGPU_T_SAVE, WRFGPU_PH_2, WRFGPU_W_2, WRFGPU_RW_TEND,
                                WRFGPU_CQW, WRFGPU_C2A, WRFGPU_ALT, WRFGPU_PH_TEND, WRFGPU_WW, WRFGPU_PH_SAVE,
                                WRFGPU_PHB, WRFGPU_A, WRFGPU_ALPHA};
    const CUtensorMap* maps[NF];
    for (int f = 0; f < NF; ++f) maps[f] = tmap_of(m, ids[f], BOX_TILE);
    const int x0 = tp.i0 - m.ims, z0 = tp.j0 - m.jms;
    if (tid == 0) {
      ring.init_barriers();
      mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int k = 1; k <= min(AW_RING - 1, kde); ++k) ring.issue(k, maps, x0, z0, m.kms);
    bool ok = true;

    F3 w = f3(m, WRFGPU_W_2), t_2ave = f3(m, WRFGPU_T_2SAVE), ph = f3(m, WRFGPU_PH_2), u = f3(m, WRFGPU_U_2),
       v = f3(m, WRFGPU_V_2);
    F2 ht = f2(m, WRFGPU_HT), msftx = f2(m, WRFGPU_MSFTX), msfty = f2(m, WRFGPU_MSFTY);
    F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F),
       fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP), rdnw = f1(m, WRFGPU_RDNW), rdn = f1(m, WRFGPU_RDN);
    const bool fp64 = sizeof(RC) == 8;
    const bool adv2 = m.cf.phi_adv_z == 2;
    const float msft_inv = 1.f / msfty.ro(ic, jc);
    const float my = msfty.ro(ic, jc), mx = msftx.ro(ic, jc), mutij = f2(m, WRFGPU_MUT).ro(ic, jc),
                mua = f2(m, WRFGPU_MUAVE).ro(ic, jc), mts = f2(m, WRFGPU_MUTS).ro(ic, jc);
    auto P = [&](int k, int f) -> float { return ring.plane(k, f)[po]; };
    auto Acoef = [&](int k) -> RC {
      if (fp64) return (RC)__ldg(&d3(m, m.wd[0])(ic, k, jc));
      return (RC)P(k, AW_A < NF ? AW_A : 0);
    };
    auto ALcoef = [&](int k) -> RC {
      if (fp64) return (RC)__ldg(&d3(m, m.wd[1])(ic, k, jc));
      return (RC)P(k, AW_AL < NF ? AW_AL : 0);
    };
    auto GAcoef = [&](int k) -> RC {
      return fp64 ? (RC)__ldg(&d3(m, m.wd[2])(ic, k, jc)) : (RC)f3(m, WRFGPU_GAMMA).ro(ic, k, jc);
    };
    const float eps1 = 1.f + epssm, eps0 = 1.f - epssm;

    // surface w (needs only u, v of the lowest levels)
    const float cf1 = m.cf1, cf2 = m.cf2, cf3 = m.cf3;
    const int I = ic, J = jc;
    const float w1 = (my * .5f * rdy *
                          ((ht.ro(I, J + 1) - ht.ro(I, J)) * (cf1 * v.ro(I, 1, J + 1) + cf2 * v.ro(I, 2, J + 1) + cf3 * v.ro(I, 3, J + 1)) +
                           (ht.ro(I, J) - ht.ro(I, J - 1)) * (cf1 * v.ro(I, 1, J) + cf2 * v.ro(I, 2, J) + cf3 * v.ro(I, 3, J))) +
                      mx * .5f * rdx *
                          ((ht.ro(I + 1, J) - ht.ro(I, J)) * (cf1 * u.ro(I + 1, 1, J) + cf2 * u.ro(I + 1, 2, J) + cf3 * u.ro(I + 1, 3, J)) +
                           (ht.ro(I, J) - ht.ro(I - 1, J)) * (cf1 * u.ro(I, 1, J) + cf2 * u.ro(I, 2, J) + cf3 * u.ro(I, 3, J))));

    // explicit w of level k (FP32, the reference's expression) and forward
    // elimination (RC: FP64 in the mixed form)
    RC wprev = (RC)w1;
    RC wcol[KCOL];
    auto sweep = [&](int k, float wk_in, float rwt, float cqwk, float c2ak, float altk, RC ak, RC alk, float tak,
                     float c2am, float altm, float tam, float r_p1, float r_0, float r_m1, float ph_p1, float ph_0,
                     float ph_m1) {
      const float wkf = wk_in + dts * rwt +
                        msft_inv * cqwk *
                            (+.5f * dts * G * rdn(k) *
                             (c2ak * rdnw(k) / (c1h(k) * mutij + c2h(k)) * (eps1 * (r_p1 - r_0) + eps0 * (ph_p1 - ph_0)) -
                              c2am * rdnw(k - 1) / (c1h(k - 1) * mutij + c2h(k - 1)) *
                                  (eps1 * (r_0 - r_m1) + eps0 * (ph_0 - ph_m1)))) +
                        dts * G * msft_inv * (rdn(k) * (c2ak * altk * tak - c2am * altm * tam) - (c1f(k) * mua));
      RC wk;
      if constexpr (sizeof(RC) == 8) wk = fma(-ak, wprev, (RC)wkf) * alk;  // mixed form: one FP64 fma
      else wk = ((RC)wkf - ak * wprev) * alk;
      wcol[k] = wk;
      wprev = wk;
    };
    float rhs[KCOL];
    rhs[1] = 0.f;
    // windows: level L-1 and L-2 values of what the elimination reads
    float r_m1 = 0.f, r_m2 = 0.f;          // rhs(L-1), rhs(L-2)
    float ph_m1 = 0.f, ph_m2 = 0.f;        // ph(L-1), ph(L-2)
    float ta_m1 = 0.f, ta_m2 = 0.f;        // t_2ave(L-1), t_2ave(L-2)
    float c2a_m1 = 0.f, c2a_m2 = 0.f, alt_m1 = 0.f, alt_m2 = 0.f;
    float w_m1 = 0.f, rwt_m1 = 0.f, cqw_m1 = 0.f;
    RC a_m1 = RC(0.), al_m1 = RC(0.);
    float wd_k = 0.f;   // wdwn(L)
    float rr_k = 0.f;   // raw rhs(L)
    ok = ring.wait(1) && ok;
    float ww_k = P(1, AW_WW), ph1_k = P(1, AW_PH1), phb_k = P(1, AW_PHB);
    for (int Lk = 1; Lk <= k_end; ++Lk) {
      __syncthreads();  // level Lk-1's slot is free
      if (tid == 0 && Lk + AW_RING - 1 <= kde) ring.issue(Lk + AW_RING - 1, maps, x0, z0, m.kms);
      ok = ring.wait(Lk + 1) && ok;
      const float c_t2 = P(Lk, AW_T2), c_t2a = P(Lk, AW_T2A), c_t1 = P(Lk, AW_T1), c_ph = P(Lk, AW_PH);
      const float c_w = P(Lk, AW_W), c_rwt = P(Lk, AW_RWT), c_cqw = P(Lk, AW_CQW), c_c2a = P(Lk, AW_C2A),
                  c_alt = P(Lk, AW_ALT);
      const RC c_a = Acoef(Lk), c_al = ALcoef(Lk);
      const float c_pht1 = P(Lk + 1, AW_PHT), c_w1 = P(Lk + 1, AW_W), c_ww1 = P(Lk + 1, AW_WW),
                  c_ph11 = P(Lk + 1, AW_PH1), c_phb1 = P(Lk + 1, AW_PHB);
      // t_2ave(L)
      float tav = .5f * ((1.f + epssm) * c_t2 + (1.f - epssm) * c_t2a);
      tav = (tav + (c1h(Lk) * mua) * T0) / ((c1h(Lk) * mts + c2h(Lk)) * (T0 + c_t1));
      if (act) t_2ave(i, Lk, j) = tav;
      // raw rhs(L+1), wdwn(L+1)
      const float rr_next = dts * (c_pht1 + .5f * G * (1.f - epssm) * c_w1);
      float wd_hi;
      if (adv2) wd_hi = rdnw(Lk) * (c_ph11 - ph1_k + c_phb1 - phb_k);
      else wd_hi = .5f * (c_ww1 + ww_k) * rdnw(Lk) * (c_ph11 - ph1_k + c_phb1 - phb_k);
      // rhs(L) complete
      float r_0 = 0.f;
      if (Lk >= 2) {
        float r = rr_k;
        if (adv2) r = r - (dts * ww_k * (fnm(Lk) * wd_hi + fnp(Lk) * wd_k));
        else r = r - (dts * (fnm(Lk) * wd_hi + fnp(Lk) * wd_k));
        r = c_ph + my * r / (c1f(Lk) * mutij + c2f(Lk));
        rhs[Lk] = r;
        r_0 = r;
      }
      // elimination of level L-1
      if (Lk >= 3)
        sweep(Lk - 1, w_m1, rwt_m1, cqw_m1, c2a_m1, alt_m1, a_m1, al_m1, ta_m1, c2a_m2, alt_m2, ta_m2, r_0, r_m1,
              r_m2, c_ph, ph_m1, ph_m2);
      // slide
      r_m2 = r_m1; r_m1 = r_0;
      ph_m2 = ph_m1; ph_m1 = c_ph;
      ta_m2 = ta_m1; ta_m1 = tav;
      c2a_m2 = c2a_m1; c2a_m1 = c_c2a; alt_m2 = alt_m1; alt_m1 = c_alt;
      w_m1 = c_w; rwt_m1 = c_rwt; cqw_m1 = c_cqw; a_m1 = c_a; al_m1 = c_al;
      ww_k = c_ww1; ph1_k = c_ph11; phb_k = c_phb1;
      wd_k = wd_hi; rr_k = rr_next;
    }
    // top: rhs(kde) has no omega term (level kde is resident: waited at Lk = k_end)
    const int kt = k_end + 1;
    const float ph_top = P(kt, AW_PH);
    float r_top = ph_top + my * rr_k / (c1f(kt) * mutij + c2f(kt));
    if (m.cf.top_lid) r_top = 0.f;
    rhs[kt] = r_top;
    // elimination of level k_end
    sweep(k_end, w_m1, rwt_m1, cqw_m1, c2a_m1, alt_m1, a_m1, al_m1, ta_m1, c2a_m2, alt_m2, ta_m2, r_top, r_m1, r_m2,
          ph_top, ph_m1, ph_m2);
    {  // level kde
      const int k = kt;
      const float r = rdnw(k - 1);
      float wkf = P(k, AW_W) + dts * P(k, AW_RWT) +
                  msft_inv * (-.5f * dts * G / (c1h(k - 1) * mutij + c2h(k - 1)) * (r * r) * 2.f * c2a_m1 *
                                  (eps1 * (r_top - r_m1) + eps0 * (ph_top - ph_m1)) -
                              dts * G * (2.f * rdnw(k - 1) * c2a_m1 * alt_m1 * ta_m1 + (c1f(k) * mua)));
      if (m.cf.top_lid) wkf = 0.f;
      RC wk;
      if constexpr (sizeof(RC) == 8) wk = fma(-Acoef(k), wprev, (RC)wkf) * ALcoef(k);
      else wk = ((RC)wkf - Acoef(k) * wprev) * ALcoef(k);
      wcol[k] = wk;
    }
    if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
    if (!act) return;
    MassImages img;  // the halo images of ph
    img.init(m, i, j);
    w(i, 1, j) = w1;
    // ---- damp_opt = 3 (module_small_step_em.F:1445-1458): after the back
    // substitution, w relaxes toward w_save in the top zdamp metres with
    // weight dampmag sin^2(pi/2 (h - hbot) / zdamp); the geopotential then
    // takes the damped w.  The recursion itself runs on the undamped values.
    // DAMP: compiled in only when some member uses it (the launcher's choice)
    const bool damp3 = DAMP && m.cf.damp_opt == 3;
    const F3 w_save = f3(m, WRFGPU_W_SAVE), ph_1 = f3(m, WRFGPU_PH_SAVE), phb = f3(m, WRFGPU_PHB);
    const float hdepth = m.cf.zdamp, dampmag = dts * m.cf.dampcoef;
    const float htop = damp3 ? (ph_1.ro(i, kt, j) + phb.ro(i, kt, j)) / G : 0.f;
    auto damped = [&](int k, float wk, float ph1k, float phbk, float wsk) -> float {
      const float hk = (ph1k + phbk) / G;
      const float hbot = htop - hdepth;
      float dampwt = 0.f;
      if (hk >= hbot) {
        const float sn = wrfgpu_ff::sinf_cr(.5f * PI_F * (hk - hbot) / hdepth);
        dampwt = dampmag * sn * sn;
      }
      return (wk - dampwt * (c1f(k) * mutij + c2f(k)) * wsk) / (1.f + dampwt);
    };
    // ---- back substitution (RC) and geopotential (FP32, from the new w)
    RC wup = wcol[kt];
    {
      float wst = (float)wup;
      if (damp3) wst = damped(kt, wst, ph_1.ro(i, kt, j), phb.ro(i, kt, j), w_save.ro(i, kt, j));
      w(i, kt, j) = wst;
      const float phv = rhs[kt] + my * .5f * dts * G * eps1 * wst / (c1f(kt) * mts + c2f(kt));
      img.store([&](int ii, int jj) { ph(ii, kt, jj) = phv; });
    }
    // four levels at a time: their gamma, eliminated w and rhs (global and
    // local-memory loads, independent of the recursion) go out first
    for (int kb = k_end; kb >= 2; kb -= 4) {
      RC gv[4], wv[4];
      float rv[4], p1v[4], pbv[4], wsv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = kb - q;
        if (k >= 2) {
          gv[q] = GAcoef(k); wv[q] = wcol[k]; rv[q] = rhs[k];
          if (damp3) { p1v[q] = ph_1.ro(i, k, j); pbv[q] = phb.ro(i, k, j); wsv[q] = w_save.ro(i, k, j); }
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = kb - q;
        if (k >= 2) {
          RC wk;
          if constexpr (sizeof(RC) == 8) wk = fma(-gv[q], wup, wv[q]);
          else wk = wv[q] - gv[q] * wup;
          float wst = (float)wk;
          if (damp3) wst = damped(k, wst, p1v[q], pbv[q], wsv[q]);
          w(i, k, j) = wst;
          const float phv = rv[q] + my * .5f * dts * G * eps1 * wst / (c1f(k) * mts + c2f(k));
          img.store([&](int ii, int jj) { ph(ii, k, jj) = phv; });
          wup = wk;
        }
      }
    }
  }
}

void launch_advance_mu_t_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, bool fp64, cudaStream_t s,
                             int var) {
  const int minb = TUNE_PARAM[TU_AMUT][var];
  if (fp64) {
    if (minb == 2) k_advance_mu_t_col<double, 2><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
    else if (minb == 3) k_advance_mu_t_col<double, 3><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
    else if (minb == 4) k_advance_mu_t_col<double, 4><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
    else k_advance_mu_t_col<double, 5><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
  } else {
    if (minb == 2) k_advance_mu_t_col<float, 2><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
    else if (minb == 3) k_advance_mu_t_col<float, 3><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
    else if (minb == 4) k_advance_mu_t_col<float, 4><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
    else k_advance_mu_t_col<float, 5><<<nblocks, dim3(TX, TY), 0, s>>>(L, rk_step, iteration);
  }
}
template <bool DAMP>
static void launch_advance_w_var(const TileLaunch& L, int nblocks, int rk_step, int iteration, bool fp64,
                                 cudaStream_t s, int minb) {
  static bool attr = false;
  constexpr size_t S32 = AwCfg<float, 4>::Ring::SMEM, S64 = AwCfg<double, 4>::Ring::SMEM;
  constexpr size_t S32_3 = AwCfg<float, 3>::Ring::SMEM, S64_3 = AwCfg<double, 3>::Ring::SMEM;
  if (!attr) {
    cudaFuncSetAttribute(k_advance_w_col<float, 2, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S32);
    cudaFuncSetAttribute(k_advance_w_col<float, 3, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S32);
    cudaFuncSetAttribute(k_advance_w_col<float, 4, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S32_3);
    cudaFuncSetAttribute(k_advance_w_col<double, 2, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S64);
    cudaFuncSetAttribute(k_advance_w_col<double, 3, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S64);
    cudaFuncSetAttribute(k_advance_w_col<double, 4, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S64_3);
    attr = true;
  }
  if (fp64) {
    if (minb == 2) k_advance_w_col<double, 2, DAMP><<<nblocks, dim3(TX, TY), S64, s>>>(L, rk_step, iteration);
    else if (minb == 3) k_advance_w_col<double, 3, DAMP><<<nblocks, dim3(TX, TY), S64, s>>>(L, rk_step, iteration);
    else k_advance_w_col<double, 4, DAMP><<<nblocks, dim3(TX, TY), S64_3, s>>>(L, rk_step, iteration);
  } else {
    if (minb == 2) k_advance_w_col<float, 2, DAMP><<<nblocks, dim3(TX, TY), S32, s>>>(L, rk_step, iteration);
    else if (minb == 3) k_advance_w_col<float, 3, DAMP><<<nblocks, dim3(TX, TY), S32, s>>>(L, rk_step, iteration);
    else k_advance_w_col<float, 4, DAMP><<<nblocks, dim3(TX, TY), S32_3, s>>>(L, rk_step, iteration);
  }
}
void launch_advance_w_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, bool fp64, cudaStream_t s,
                          int var, bool damp) {
  const int minb = TUNE_PARAM[TU_AW][var];
  if (damp) launch_advance_w_var<true>(L, nblocks, rk_step, iteration, fp64, s, minb);
  else launch_advance_w_var<false>(L, nblocks, rk_step, iteration, fp64, s, minb);
}

}  // namespace wrfgpu
