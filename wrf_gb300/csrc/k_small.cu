// Acoustic (small) step kernels: dyn_em/module_small_step_em.F
//   small_step_prep   :16-290   column kernel (2-D mass bookkeeping + 3-D recoupling)
//   calc_p_rho        :438-568  point kernel
//   calc_coef_w       :570-652  column kernel (tridiagonal coefficients)
//   advance_uv        :654-967  point kernel
//   advance_mu_t      :969-1175 column kernel (column mass divergence, omega recursion, theta)
//   advance_w         :1178-1469 column kernel (explicit w + Thomas solve + ph update)
//   sumflux           :1473-1633 point kernel (fused with calc_p_rho of the same tile loop)
//   small_step_finish :295-434 with calc_mu_uv_1 (module_big_step_utilities_em.F:184-326)
// Column recursions are templated on their accumulation type RC: float in
// the plain form (the reference's REAL), double in the mixed-precision form
// (FP64 column sums, omega recursion, tridiagonal coefficients and solve).
// Roofline: HBM-bound; advance_w reads ~20 arrays per cell and is the
// largest acoustic kernel.
#include "common.cuh"
#include "kernels.h"
#include "ffmath.h"

namespace wrfgpu {

constexpr int KMAX = 128;  // column scratch (kde <= KMAX, checked at domain creation)

// ------------------------------------------------------------ small_step_prep
// Two kernels.  The 2-D part (mu_1, mu_2, muts, muus, muvs, mu_save, mudf)
// runs once per column; the 3-D part is elementwise in k and runs one block
// per (staggered tile, chunk of levels), reading muts / muus / muvs as the
// 2-D kernel stored them (the same values the reference's loops use).
__global__ void __launch_bounds__(BX* BY) k_small_step_prep_2d(Launch L, int rk_step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j;
  const int i_start = m.its, i_end = min(m.ite, m.ide - 1), j_start = m.jts, j_end = min(m.jte, m.jde - 1);
  const int i_endu = m.ite, j_endv = m.jte;
  if (i < i_start || i > i_endu || j < j_start || j > j_endv) return;
  const bool mass = i <= i_end && j <= j_end, upt = i <= i_endu && j <= j_end, vpt = i <= i_end && j <= j_endv;
  F2 mub = f2(m, WRFGPU_MUB), MU_1 = f2(m, WRFGPU_MU_1), MU_2 = f2(m, WRFGPU_MU_2), MUU = f2(m, WRFGPU_MUU),
     MUUS = f2(m, WRFGPU_MUUS), MUV = f2(m, WRFGPU_MUV), MUVS = f2(m, WRFGPU_MUVS), MUTS = f2(m, WRFGPU_MUTS),
     MUDF = f2(m, WRFGPU_MUDF), MU_SAVE = f2(m, WRFGPU_MU_SAVE);
  if (rk_step == 1) {
    if (mass) { MU_1(i, j) = MU_2(i, j); MUDF(i, j) = 0.f; }
    if (mass) MUTS(i, j) = mub.ro(i, j) + MU_2(i, j);
    if (upt) MUUS(i, j) = MUU.ro(i, j);
    if (vpt) MUVS(i, j) = MUV.ro(i, j);
    if (mass) { MU_SAVE(i, j) = MU_2(i, j); MU_2(i, j) = 0.f; }
  } else {
    if (mass) MUTS(i, j) = mub.ro(i, j) + MU_1(i, j);
    if (upt) MUUS(i, j) = 0.5f * (mub.ro(i, j) + MU_1(i, j) + mub.ro(i - 1, j) + MU_1(i - 1, j));
    if (vpt) MUVS(i, j) = 0.5f * (mub.ro(i, j) + MU_1(i, j) + mub.ro(i, j - 1) + MU_1(i, j - 1));
    if (mass) { MU_SAVE(i, j) = MU_2(i, j); MU_2(i, j) = MU_1(i, j) - MU_2(i, j); }
  }
}

// levels [k0, k1] split into gridDim.y chunks: this block's part
__device__ __forceinline__ void level_chunk(int k0, int k1, int* c0, int* c1) {
  const int per = (k1 - k0 + 1 + gridDim.y - 1) / gridDim.y;
  *c0 = k0 + blockIdx.y * per;
  *c1 = min(k1, *c0 + per - 1);
}

// (a minimum of three blocks per SM holds it to 63 registers, four resident blocks)
__global__ void __launch_bounds__(TX* TY, 3) k_small_step_prep_3d(TileLaunch L, int rk_step) {
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  const int i_end = min(m.ite, m.ide - 1), j_end = min(m.jte, m.jde - 1);
  const int k_start = m.kts, k_end = min(m.kte, m.kde - 1), i_endu = m.ite, j_endv = m.jte, kde = m.kde;
  if (i > i_endu || j > j_endv) return;
  const bool mass = i <= i_end && j <= j_end, upt = i <= i_endu && j <= j_end, vpt = i <= i_end && j <= j_endv;
  F3 u_1 = f3(m, WRFGPU_U_1), u_2 = f3(m, WRFGPU_U_2), v_1 = f3(m, WRFGPU_V_1), v_2 = f3(m, WRFGPU_V_2),
     w_1 = f3(m, WRFGPU_W_1), w_2 = f3(m, WRFGPU_W_2), t_1 = f3(m, WRFGPU_T_1), t_2 = f3(m, WRFGPU_T_2),
     ph_1 = f3(m, WRFGPU_PH_1), ph_2 = f3(m, WRFGPU_PH_2), u_save = f3(m, WRFGPU_U_SAVE),
     v_save = f3(m, WRFGPU_V_SAVE), w_save = f3(m, WRFGPU_W_SAVE), t_save = f3(m, WRFGPU_T_SAVE),
     ph_save = f3(m, WRFGPU_PH_SAVE), ww = f3(m, WRFGPU_WW), ww_save = f3(m, WRFGPU_WW1), c2a = f3(m, WRFGPU_C2A),
     pb = f3(m, WRFGPU_PB), p = f3(m, WRFGPU_P), alt = f3(m, WRFGPU_ALT);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F);
  const bool rk1 = rk_step == 1;
  int c0, c1;
  level_chunk(k_start, k_end, &c0, &c1);
  // levels are independent: inputs of a chunk of levels are loaded first.
  // At the first stage *_1 = *_2 (the copies the reference makes first).
  struct L2 { float x2, x1; };
  if (upt) {
    const float muus = f2(m, WRFGPU_MUUS)(i, j), muu = f2(m, WRFGPU_MUU).ro(i, j), my = f2(m, WRFGPU_MSFUY).ro(i, j);
    chunked_levels<8, L2>(
        c0, c1, [&](int k, L2& d) { d.x2 = u_2(i, k, j); d.x1 = rk1 ? d.x2 : u_1(i, k, j); },
        [&](int k, const L2& d) {
          if (rk1) u_1(i, k, j) = d.x2;
          u_save(i, k, j) = d.x2;
          u_2(i, k, j) = ((c1h(k) * muus + c2h(k)) * d.x1 - (c1h(k) * muu + c2h(k)) * d.x2) / my;
        });
  }
  if (vpt) {
    const float muvs = f2(m, WRFGPU_MUVS)(i, j), muv = f2(m, WRFGPU_MUV).ro(i, j),
                mxi = f2(m, WRFGPU_MSFVX_INV).ro(i, j);
    chunked_levels<8, L2>(
        c0, c1, [&](int k, L2& d) { d.x2 = v_2(i, k, j); d.x1 = rk1 ? d.x2 : v_1(i, k, j); },
        [&](int k, const L2& d) {
          if (rk1) v_1(i, k, j) = d.x2;
          v_save(i, k, j) = d.x2;
          v_2(i, k, j) = ((c1h(k) * muvs + c2h(k)) * d.x1 - (c1h(k) * muv + c2h(k)) * d.x2) * mxi;
        });
  }
  if (mass) {
    const float muts = f2(m, WRFGPU_MUTS)(i, j), mt = f2(m, WRFGPU_MUT).ro(i, j), my = f2(m, WRFGPU_MSFTY).ro(i, j);
    struct LT { float t2, t1, pb, p, alt; };
    chunked_levels<8, LT>(
        c0, c1,
        [&](int k, LT& d) {
          d.t2 = t_2(i, k, j); d.t1 = rk1 ? d.t2 : t_1(i, k, j);
          d.pb = pb.ro(i, k, j); d.p = p.ro(i, k, j); d.alt = alt.ro(i, k, j);
        },
        [&](int k, const LT& d) {
          if (rk1) t_1(i, k, j) = d.t2;
          c2a(i, k, j) = CPOVCV * (d.pb + d.p) / d.alt;
          t_save(i, k, j) = d.t2;
          t_2(i, k, j) = (c1h(k) * muts + c2h(k)) * d.t1 - (c1h(k) * mt + c2h(k)) * d.t2;
        });
    int w0, w1;
    level_chunk(k_start, kde, &w0, &w1);
    struct LW { float w2, w1, p2, p1, ww; };
    chunked_levels<6, LW>(
        w0, w1,
        [&](int k, LW& d) {
          d.w2 = w_2(i, k, j); d.w1 = rk1 ? d.w2 : w_1(i, k, j);
          d.p2 = ph_2(i, k, j); d.p1 = rk1 ? d.p2 : ph_1(i, k, j);
          d.ww = ww.ro(i, k, j);
        },
        [&](int k, const LW& d) {
          if (rk1) { w_1(i, k, j) = d.w2; ph_1(i, k, j) = d.p2; }
          w_save(i, k, j) = d.w2;
          w_2(i, k, j) = ((c1f(k) * muts + c2f(k)) * d.w1 - (c1f(k) * mt + c2f(k)) * d.w2) / my;
          ph_save(i, k, j) = d.p2;
          ph_2(i, k, j) = d.p1 - d.p2;
          ww_save(i, k, j) = d.ww;
        });
  }
}

// ------------------------------------------------------------ calc_p_rho
__device__ __forceinline__ void calc_p_rho_point(const Mem& m, int i, int k, int j, int step) {
  F3 al = f3(m, WRFGPU_AL), p = f3(m, WRFGPU_P), ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT),
     t_2 = f3(m, WRFGPU_T_2), t_1 = f3(m, WRFGPU_T_SAVE), c2a = f3(m, WRFGPU_C2A), pm1 = f3(m, WRFGPU_PM1);
  F2 mu = f2(m, WRFGPU_MU_2), Mut = f2(m, WRFGPU_MUTS);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), rdnw = f1(m, WRFGPU_RDNW);
  const float a = alt.ro(i, k, j), muij = mu.ro(i, j), mutij = Mut.ro(i, j), t1 = t_1.ro(i, k, j);
  float alv = -1.f / (c1h(k) * mutij + c2h(k)) * (a * (c1h(k) * muij) + rdnw(k) * (ph.ro(i, k + 1, j) - ph.ro(i, k, j)));
  al(i, k, j) = alv;
  float pv = c2a.ro(i, k, j) * (a * (t_2.ro(i, k, j) - (c1h(k) * muij) * t1) / ((c1h(k) * mutij + c2h(k)) * (T0 + t1)) - alv);
  if (step == 0) {
    pm1(i, k, j) = pv;
  } else {
    float ptmp = pv;
    pv = pv + m.smdiv * (pv - pm1(i, k, j));
    pm1(i, k, j) = ptmp;
  }
  p(i, k, j) = pv;
}

__global__ void __launch_bounds__(BX* BY) k_calc_p_rho(Launch L, int step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (i < m.its || i > min(m.ite, m.ide - 1) || j < m.jts || j > min(m.jte, m.jde - 1) || k < m.kts ||
      k > min(m.kte, m.kde - 1))
    return;
  calc_p_rho_point(m, i, k, j, step);
}

// Column form over mass tiles x level chunks: the levels of a chunk are
// independent, so their loads go out four levels at a time; the arithmetic
// of each point is calc_p_rho_point's.
__global__ void __launch_bounds__(TX* TY) k_calc_p_rho_col(TileLaunch L, int step) {
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  if (i > min(m.ite, m.ide - 1) || j > min(m.jte, m.jde - 1)) return;
  int c0, c1;
  level_chunk(m.kts, min(m.kte, m.kde - 1), &c0, &c1);
  F3 al = f3(m, WRFGPU_AL), p = f3(m, WRFGPU_P), ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT),
     t_2 = f3(m, WRFGPU_T_2), t_1 = f3(m, WRFGPU_T_SAVE), c2a = f3(m, WRFGPU_C2A), pm1 = f3(m, WRFGPU_PM1);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), rdnw = f1(m, WRFGPU_RDNW);
  const float muij = f2(m, WRFGPU_MU_2).ro(i, j), mutij = f2(m, WRFGPU_MUTS).ro(i, j), smdiv = m.smdiv;
  struct LP { float a, t1, t2, c2a, ph0, ph1, pm1; };
  chunked_levels<4, LP>(
      c0, c1,
      [&](int k, LP& d) {
        d.a = alt.ro(i, k, j); d.t1 = t_1.ro(i, k, j); d.t2 = t_2.ro(i, k, j); d.c2a = c2a.ro(i, k, j);
        d.ph0 = ph.ro(i, k, j); d.ph1 = ph.ro(i, k + 1, j); d.pm1 = step == 0 ? 0.f : pm1(i, k, j);
      },
      [&](int k, const LP& d) {
        const float alv = -1.f / (c1h(k) * mutij + c2h(k)) * (d.a * (c1h(k) * muij) + rdnw(k) * (d.ph1 - d.ph0));
        al(i, k, j) = alv;
        float pv = d.c2a * (d.a * (d.t2 - (c1h(k) * muij) * d.t1) / ((c1h(k) * mutij + c2h(k)) * (T0 + d.t1)) - alv);
        if (step == 0) {
          pm1(i, k, j) = pv;
        } else {
          const float ptmp = pv;
          pv = pv + smdiv * (pv - d.pm1);
          pm1(i, k, j) = ptmp;
        }
        p(i, k, j) = pv;
      });
}

// ------------------------------------------------------------ calc_coef_w
// One column of calc_coef_w at (i, j).
template <typename RC>
__device__ __forceinline__ void coef_w_column(const Mem& m, int i, int j, int rk_step) {
  const Stage st = stage_of(m, rk_step);
  F3 cqw = f3(m, WRFGPU_CQW), c2a = f3(m, WRFGPU_C2A);
  F2 MUTf = f2(m, WRFGPU_MUT);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F),
     rdn = f1(m, WRFGPU_RDN), rdnw = f1(m, WRFGPU_RDNW);
  const int kde = m.kde;
  // a, b, c in FP32 (the reference's expressions and rounding); the
  // recursion alpha = 1 / (b - a gamma), gamma = c alpha in RC
  const float MUT = MUTf(i, j);
  const float lid_flag = m.cf.top_lid ? 0.f : 1.f;
  const float tt = (.5f * st.dts_rk * G * (1.f + m.epssm));
  const float cof = tt * tt;
  auto A = [&](int k) -> RC& {
    if (sizeof(RC) == 8) return *(RC*)&d3(m, m.wd[0])(i, k, j);
    return *(RC*)&f3(m, WRFGPU_A)(i, k, j);
  };
  auto AL = [&](int k) -> RC& {
    if (sizeof(RC) == 8) return *(RC*)&d3(m, m.wd[1])(i, k, j);
    return *(RC*)&f3(m, WRFGPU_ALPHA)(i, k, j);
  };
  auto GA = [&](int k) -> RC& {
    if (sizeof(RC) == 8) return *(RC*)&d3(m, m.wd[2])(i, k, j);
    return *(RC*)&f3(m, WRFGPU_GAMMA)(i, k, j);
  };
  // one pass up the column: A(k) (the reference forms all of A first; A
  // does not depend on the recursion, so the values are the same), B, C and
  // the recursion, with the loads of four levels in flight
  A(2) = RC(0.);
  GA(1) = RC(0.);
  RC gprev = RC(0.);
  struct LC { float cqw, c2a, c2am; };
  chunked_levels<4, LC>(
      2, kde - 1,
      [&](int k, LC& d) { d.cqw = cqw.ro(i, k, j); d.c2a = c2a.ro(i, k, j); d.c2am = c2a.ro(i, k - 1, j); },
      [&](int k, const LC& d) {
        float a_k = 0.f;
        if (k >= 3) {
          const int kl = k - 1;
          a_k = -d.cqw * cof * rdn(k) * rdnw(k - 1) * d.c2am / ((c1h(kl) * MUT + c2h(kl)) * (c1f(kl) * MUT + c2f(kl)));
          A(k) = (RC)a_k;
        }
        const float b = 1.f + d.cqw * cof * rdn(k) *
                                  (rdnw(k) * d.c2a / ((c1h(k) * MUT + c2h(k)) * (c1f(k) * MUT + c2f(k))) +
                                   rdnw(k - 1) * d.c2am / ((c1h(k - 1) * MUT + c2h(k - 1)) * (c1f(k) * MUT + c2f(k))));
        const float c = -d.cqw * cof * rdn(k) * rdnw(k) * d.c2a /
                        ((c1h(k) * MUT + c2h(k)) * (c1f(k + 1) * MUT + c2f(k + 1)));
        // the mixed form fuses b - a gamma into one FP64 fma
        RC den;
        if constexpr (sizeof(RC) == 8) den = fma(-(RC)a_k, gprev, (RC)b);
        else den = (RC)b - (RC)a_k * gprev;
        RC al = rcp_rc<RC>(den);
        AL(k) = al;
        gprev = (RC)c * al;
        GA(k) = gprev;
      });
  float a_top;
  {
    int k = kde - 1;
    float r = rdnw(kde - 1);
    a_top = -2.f * cof * (r * r) * c2a.ro(i, kde - 1, j) * lid_flag /
            ((c1h(k) * MUT + c2h(k)) * (c1f(k) * MUT + c2f(k)));
    A(kde) = (RC)a_top;
  }
  {
    int k = kde;
    float r = rdnw(kde - 1);
    const float b = 1.f + 2.f * cof * (r * r) * c2a.ro(i, kde - 1, j) /
                              ((c1h(k - 1) * MUT + c2h(k - 1)) * (c1f(k) * MUT + c2f(k)));
    RC den;
    if constexpr (sizeof(RC) == 8) den = fma(-(RC)a_top, gprev, (RC)b);
    else den = (RC)b - (RC)a_top * gprev;
    RC al = rcp_rc<RC>(den);
    AL(kde) = al;
    GA(kde) = RC(0.) * al;
  }
}

template <typename RC>
__global__ void __launch_bounds__(BX* BY) k_calc_coef_w(Launch L, int rk_step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j;
  if (i < m.its || i > min(m.ite, m.ide - 1) || j < m.jts || j > min(m.jte, m.jde - 1)) return;
  coef_w_column<RC>(m, i, j, rk_step);
}

// the same over mass tiles (32 x 8 columns per block)
template <typename RC>
__global__ void __launch_bounds__(TX* TY) k_calc_coef_w_col(TileLaunch L, int rk_step) {
  const TilePos tp = tile_pos(L, false, false);
  const Mem& m = block_member(L.mem, tp.m);
  const int i = tp.i0 + threadIdx.x, j = tp.j0 + threadIdx.y;
  if (i > min(m.ite, m.ide - 1) || j > min(m.jte, m.jde - 1)) return;
  coef_w_column<RC>(m, i, j, rk_step);
}

// ------------------------------------------------------------ advance_uv
__global__ void __launch_bounds__(BX* BY) k_advance_uv(Launch L, int rk_step, int iteration) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (iteration > stage_of(m, rk_step).nsmall) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  const int k_start = m.kts, k_end = m.kte - 1;
  if (k < k_start || k > k_end) return;
  const Stage st = stage_of(m, rk_step);
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
  F3 p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB), ph = f3(m, WRFGPU_PH_2), php = f3(m, WRFGPU_PHP),
     alt = f3(m, WRFGPU_ALT), al = f3(m, WRFGPU_AL);
  F2 mu = f2(m, WRFGPU_MU_2), MUDF = f2(m, WRFGPU_MUDF);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP),
     rdnw = f1(m, WRFGPU_RDNW);
  const float rdx = m.rdx, rdy = m.rdy, emdiv = m.emdiv;
  const int kde = m.kde;
  // u
  if (j >= j_start && j <= min(m.jte, m.jde - 1) && i >= min(i_start_u_tend, i_start_up) &&
      i <= max(i_end_u_tend, i_end_up)) {
    F3 u = f3(m, WRFGPU_U_2), ru_tend = f3(m, WRFGPU_RU_TEND), cqu = f3(m, WRFGPU_CQU);
    F2 muu = f2(m, WRFGPU_MUU), msfux = f2(m, WRFGPU_MSFUX), msfuy = f2(m, WRFGPU_MSFUY);
    float uv = u(i, k, j);
    if (i >= i_start_u_tend && i <= i_end_u_tend) uv = uv + dts * ru_tend.ro(i, k, j);
    if (i >= i_start_up && i <= i_end_up) {
      const float dx = 1.f / rdx;
      float mudf_xy = -emdiv * dx * (MUDF.ro(i, j) - MUDF.ro(i - 1, j)) / msfuy.ro(i, j);
      float dpxy = (msfux.ro(i, j) / msfuy.ro(i, j)) * .5f * rdx * (c1h(k) * muu.ro(i, j) + c2h(k)) *
                   (((ph.ro(i, k + 1, j) - ph.ro(i - 1, k + 1, j)) + (ph.ro(i, k, j) - ph.ro(i - 1, k, j))) +
                    (alt.ro(i, k, j) + alt.ro(i - 1, k, j)) * (p.ro(i, k, j) - p.ro(i - 1, k, j)) +
                    (al.ro(i, k, j) + al.ro(i - 1, k, j)) * (pb.ro(i, k, j) - pb.ro(i - 1, k, j)));
      auto dpn = [&](int kk) -> float {
        if (kk == kde) {
          if (cf.top_lid)
            return .5f * (m.cf1 * (p.ro(i - 1, kde - 1, j) + p.ro(i, kde - 1, j)) + m.cf2 * (p.ro(i - 1, kde - 2, j) + p.ro(i, kde - 2, j)) +
                          m.cf3 * (p.ro(i - 1, kde - 3, j) + p.ro(i, kde - 3, j)));
          return 0.f;
        }
        if (kk == 1)
          return .5f * (m.cf1 * (p.ro(i, 1, j) + p.ro(i - 1, 1, j)) + m.cf2 * (p.ro(i, 2, j) + p.ro(i - 1, 2, j)) +
                        m.cf3 * (p.ro(i, 3, j) + p.ro(i - 1, 3, j)));
        return .5f * (fnm(kk) * (p.ro(i, kk, j) + p.ro(i - 1, kk, j)) + fnp(kk) * (p.ro(i, kk - 1, j) + p.ro(i - 1, kk - 1, j)));
      };
      dpxy = dpxy + (msfux.ro(i, j) / msfuy.ro(i, j)) * rdx * (php.ro(i, k, j) - php.ro(i - 1, k, j)) *
                        (rdnw(k) * (dpn(k + 1) - dpn(k)) - .5f * ((c1h(k) * mu.ro(i - 1, j)) + (c1h(k) * mu.ro(i, j))));
      uv = uv - dts * cqu.ro(i, k, j) * dpxy + (c1h(k) * mudf_xy);
    }
    u(i, k, j) = uv;
  }
  // v
  if (j >= j_start_v_tend && j <= j_end_v_tend && i >= i_start && i <= i_end) {
    F3 v = f3(m, WRFGPU_V_2), rv_tend = f3(m, WRFGPU_RV_TEND), cqv = f3(m, WRFGPU_CQV);
    F2 muv = f2(m, WRFGPU_MUV), msfvx = f2(m, WRFGPU_MSFVX), msfvx_inv = f2(m, WRFGPU_MSFVX_INV),
       msfvy = f2(m, WRFGPU_MSFVY);
    float vv = v(i, k, j) + dts * rv_tend.ro(i, k, j);
    const float dy = 1.f / rdy;
    float mudf_xy = -emdiv * dy * (MUDF.ro(i, j) - MUDF.ro(i, j - 1)) * msfvx_inv.ro(i, j);
    if (j >= j_start_vp && j <= j_end_vp) {
      float dpxy = (msfvy.ro(i, j) / msfvx.ro(i, j)) * .5f * rdy * (c1h(k) * muv.ro(i, j) + c2h(k)) *
                   (((ph.ro(i, k + 1, j) - ph.ro(i, k + 1, j - 1)) + (ph.ro(i, k, j) - ph.ro(i, k, j - 1))) +
                    (alt.ro(i, k, j) + alt.ro(i, k, j - 1)) * (p.ro(i, k, j) - p.ro(i, k, j - 1)) +
                    (al.ro(i, k, j) + al.ro(i, k, j - 1)) * (pb.ro(i, k, j) - pb.ro(i, k, j - 1)));
      auto dpn = [&](int kk) -> float {
        if (kk == kde) {
          if (cf.top_lid)
            return .5f * (m.cf1 * (p.ro(i, kde - 1, j - 1) + p.ro(i, kde - 1, j)) + m.cf2 * (p.ro(i, kde - 2, j - 1) + p.ro(i, kde - 2, j)) +
                          m.cf3 * (p.ro(i, kde - 3, j - 1) + p.ro(i, kde - 3, j)));
          return 0.f;
        }
        if (kk == 1)
          return .5f * (m.cf1 * (p.ro(i, 1, j) + p.ro(i, 1, j - 1)) + m.cf2 * (p.ro(i, 2, j) + p.ro(i, 2, j - 1)) +
                        m.cf3 * (p.ro(i, 3, j) + p.ro(i, 3, j - 1)));
        return .5f * (fnm(kk) * (p.ro(i, kk, j) + p.ro(i, kk, j - 1)) + fnp(kk) * (p.ro(i, kk - 1, j) + p.ro(i, kk - 1, j - 1)));
      };
      dpxy = dpxy + (msfvy.ro(i, j) / msfvx.ro(i, j)) * rdy * (php.ro(i, k, j) - php.ro(i, k, j - 1)) *
                        (rdnw(k) * (dpn(k + 1) - dpn(k)) - .5f * ((c1h(k) * mu.ro(i, j - 1)) + (c1h(k) * mu.ro(i, j))));
      vv = vv - dts * cqv.ro(i, k, j) * dpxy + (c1h(k) * mudf_xy);
    }
    v(i, k, j) = vv;
  }
}

// ------------------------------------------------------------ advance_mu_t
template <typename RC>
__global__ void __launch_bounds__(BX* BY) k_advance_mu_t(Launch L, int rk_step, int iteration) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (iteration > stage_of(m, rk_step).nsmall) return;
  const int i = bp.i, j = bp.j;
  const int i_start = m.its, i_end = min(m.ite, m.ide - 1), j_start = m.jts, j_end = min(m.jte, m.jde - 1);
  if (i < i_start || i > i_end || j < j_start || j > j_end) return;
  const int k_start = m.kts, k_end = m.kte - 1, kde = m.kde;
  const Stage st = stage_of(m, rk_step);
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
  auto dvdxi = [&](int k) -> float {
    return mxy * (rdy * ((v.ro(i, k, j + 1) + (c1h(k) * muv1 + c2h(k)) * v_1.ro(i, k, j + 1) * vi1) -
                         (v.ro(i, k, j) + (c1h(k) * muv0 + c2h(k)) * v_1.ro(i, k, j) * vi0)) +
                  rdx * ((u.ro(i + 1, k, j) + (c1h(k) * muu1 + c2h(k)) * u_1.ro(i + 1, k, j) / uy1) -
                         (u.ro(i, k, j) + (c1h(k) * muu0 + c2h(k)) * u_1.ro(i, k, j) / uy0)));
  };
  RC dmdt = RC(0.);
  for (int k = k_start; k <= k_end; ++k) dmdt = dmdt + (RC)dnw(k) * (RC)dvdxi(k);
  const float mu_tend = MU_TEND.ro(i, j);
  float muave = MU(i, j);
  float mu = (float)((RC)MU(i, j) + (RC)dts * (dmdt + (RC)mu_tend));
  MU(i, j) = mu;
  MUDF(i, j) = (float)(dmdt + (RC)mu_tend);
  MUTS(i, j) = MUT.ro(i, j) + mu;
  MUAVE(i, j) = .5f * ((1.f + epssm) * mu + (1.f - epssm) * muave);
  const float my = msfty.ro(i, j);
  // omega by upward recursion, then subtract the saved omega
  RC wwk = (RC)ww(i, 1, j);
  for (int kk = 2; kk <= k_end; ++kk) {
    int k = kk - 1;
    wwk = wwk - (RC)dnw(kk - 1) * (((RC)c1h(k) * dmdt) + (RC)dvdxi(kk - 1) + ((RC)c1h(k) * (RC)mu_tend)) / (RC)my;
    ww(i, kk, j) = (float)wwk;
  }
  for (int k = 1; k <= k_end; ++k) ww(i, k, j) = ww(i, k, j) - ww_1.ro(i, k, j);
  // theta
  for (int k = 1; k <= k_end; ++k) {
    float tv = t(i, k, j);
    t_ave(i, k, j) = tv;
    t(i, k, j) = tv + my * dts * ft.ro(i, k, j);
  }
  const float mx = msftx.ro(i, j);
  auto wdtn = [&](int k) -> float {
    if (k == 1 || k == kde) return 0.f;
    return ww(i, k, j) * (fnm(k) * t_1.ro(i, k, j) + fnp(k) * t_1.ro(i, k - 1, j));
  };
  for (int k = 1; k <= k_end; ++k) {
    t(i, k, j) = t(i, k, j) - dts * my *
                                  (mx * (.5f * rdy * (v.ro(i, k, j + 1) * (t_1.ro(i, k, j + 1) + t_1.ro(i, k, j)) - v.ro(i, k, j) * (t_1.ro(i, k, j) + t_1.ro(i, k, j - 1))) +
                                         .5f * rdx * (u.ro(i + 1, k, j) * (t_1.ro(i + 1, k, j) + t_1.ro(i, k, j)) - u.ro(i, k, j) * (t_1.ro(i, k, j) + t_1.ro(i - 1, k, j)))) +
                                   rdnw(k) * (wdtn(k + 1) - wdtn(k)));
  }
}

// ------------------------------------------------------------ advance_w
template <typename RC>
__global__ void __launch_bounds__(BX* BY) k_advance_w(Launch L, int rk_step, int iteration) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  if (iteration > stage_of(m, rk_step).nsmall) return;
  const int i = bp.i, j = bp.j;
  const int i_start = m.its, i_end = min(m.ite, m.ide - 1), j_start = m.jts, j_end = min(m.jte, m.jde - 1);
  if (i < i_start || i > i_end || j < j_start || j > j_end) return;
  const int k_end = m.kte - 1;
  const Stage st = stage_of(m, rk_step);
  const float dts = st.dts_rk, epssm = m.epssm, rdx = m.rdx, rdy = m.rdy;
  F3 w = f3(m, WRFGPU_W_2), rw_tend = f3(m, WRFGPU_RW_TEND), ww = f3(m, WRFGPU_WW), u = f3(m, WRFGPU_U_2),
     v = f3(m, WRFGPU_V_2), t_2ave = f3(m, WRFGPU_T_2SAVE), t_2 = f3(m, WRFGPU_T_2), t_1 = f3(m, WRFGPU_T_SAVE),
     ph = f3(m, WRFGPU_PH_2), ph_1 = f3(m, WRFGPU_PH_SAVE), phb = f3(m, WRFGPU_PHB), ph_tend = f3(m, WRFGPU_PH_TEND),
     c2a = f3(m, WRFGPU_C2A), cqw = f3(m, WRFGPU_CQW), alt = f3(m, WRFGPU_ALT);
  F2 mut = f2(m, WRFGPU_MUT), muave = f2(m, WRFGPU_MUAVE), muts = f2(m, WRFGPU_MUTS), ht = f2(m, WRFGPU_HT),
     msftx = f2(m, WRFGPU_MSFTX), msfty = f2(m, WRFGPU_MSFTY);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F),
     fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP), rdnw = f1(m, WRFGPU_RDNW), rdn = f1(m, WRFGPU_RDN);
  RC rhs[KMAX + 1];
  const float msft_inv = 1.f / msfty.ro(i, j);
  const float my = msfty.ro(i, j), mx = msftx.ro(i, j), mutij = mut.ro(i, j), mua = muave.ro(i, j), mts = muts.ro(i, j);
  rhs[1] = RC(0.);
  for (int k = 1; k <= k_end; ++k) {
    float ta = .5f * ((1.f + epssm) * t_2.ro(i, k, j) + (1.f - epssm) * t_2ave(i, k, j));
    ta = (ta + (c1h(k) * mua) * T0) / ((c1h(k) * mts + c2h(k)) * (T0 + t_1.ro(i, k, j)));
    t_2ave(i, k, j) = ta;
    rhs[k + 1] = (RC)(dts * (ph_tend.ro(i, k + 1, j) + .5f * G * (1.f - epssm) * w(i, k + 1, j)));
  }
  if (m.cf.phi_adv_z == 2) {
    auto wdwn = [&](int kk) {  // kk = k+1
      int k = kk - 1;
      return rdnw(k) * (ph_1.ro(i, k + 1, j) - ph_1.ro(i, k, j) + phb.ro(i, k + 1, j) - phb.ro(i, k, j));
    };
    for (int k = 2; k <= k_end; ++k)
      rhs[k] = rhs[k] - (RC)(dts * ww.ro(i, k, j) * (fnm(k) * wdwn(k + 1) + fnp(k) * wdwn(k)));
  } else {
    auto wdwn = [&](int kk) {
      int k = kk - 1;
      return .5f * (ww.ro(i, k + 1, j) + ww.ro(i, k, j)) * rdnw(k) * (ph_1.ro(i, k + 1, j) - ph_1.ro(i, k, j) + phb.ro(i, k + 1, j) - phb.ro(i, k, j));
    };
    float wd_lo = wdwn(2);
    for (int k = 2; k <= k_end; ++k) {
      float wd_hi = wdwn(k + 1);
      rhs[k] = rhs[k] - (RC)(dts * (fnm(k) * wd_hi + fnp(k) * wd_lo));
      wd_lo = wd_hi;
    }
  }
  for (int k = 2; k <= k_end + 1; ++k) {
    rhs[k] = (RC)ph(i, k, j) + (RC)my * rhs[k] / ((RC)c1f(k) * (RC)mutij + (RC)c2f(k));
    if (m.cf.top_lid && k == k_end + 1) rhs[k] = RC(0.);
  }
  const float cf1 = m.cf1, cf2 = m.cf2, cf3 = m.cf3;
  RC w1 = (RC)(my * .5f * rdy *
                   ((ht.ro(i, j + 1) - ht.ro(i, j)) * (cf1 * v.ro(i, 1, j + 1) + cf2 * v.ro(i, 2, j + 1) + cf3 * v.ro(i, 3, j + 1)) +
                    (ht.ro(i, j) - ht.ro(i, j - 1)) * (cf1 * v.ro(i, 1, j) + cf2 * v.ro(i, 2, j) + cf3 * v.ro(i, 3, j))) +
               mx * .5f * rdx *
                   ((ht.ro(i + 1, j) - ht.ro(i, j)) * (cf1 * u.ro(i + 1, 1, j) + cf2 * u.ro(i + 1, 2, j) + cf3 * u.ro(i + 1, 3, j)) +
                    (ht.ro(i, j) - ht.ro(i - 1, j)) * (cf1 * u.ro(i, 1, j) + cf2 * u.ro(i, 2, j) + cf3 * u.ro(i, 3, j))));
  w(i, 1, j) = (float)w1;
  // explicit part and forward elimination in one upward sweep
  const RC eps1 = RC(1.) + (RC)epssm, eps0 = RC(1.) - (RC)epssm;
  RC wprev = w1;
  const bool fp64 = sizeof(RC) == 8;
  auto Acoef = [&](int k) -> RC { return fp64 ? (RC)d3(m, m.wd[0])(i, k, j) : (RC)f3(m, WRFGPU_A)(i, k, j); };
  auto ALcoef = [&](int k) -> RC { return fp64 ? (RC)d3(m, m.wd[1])(i, k, j) : (RC)f3(m, WRFGPU_ALPHA)(i, k, j); };
  auto GAcoef = [&](int k) -> RC { return fp64 ? (RC)d3(m, m.wd[2])(i, k, j) : (RC)f3(m, WRFGPU_GAMMA)(i, k, j); };
  RC wcol[KMAX + 1];
  for (int k = 2; k <= k_end; ++k) {
    RC wk = (RC)w(i, k, j) + (RC)dts * (RC)rw_tend.ro(i, k, j) +
            (RC)msft_inv * (RC)cqw.ro(i, k, j) *
                (+RC(.5) * (RC)dts * (RC)G * (RC)rdn(k) *
                 ((RC)c2a.ro(i, k, j) * (RC)rdnw(k) / ((RC)c1h(k) * (RC)mutij + (RC)c2h(k)) *
                      (eps1 * (rhs[k + 1] - rhs[k]) + eps0 * ((RC)ph(i, k + 1, j) - (RC)ph(i, k, j))) -
                  (RC)c2a.ro(i, k - 1, j) * (RC)rdnw(k - 1) / ((RC)c1h(k - 1) * (RC)mutij + (RC)c2h(k - 1)) *
                      (eps1 * (rhs[k] - rhs[k - 1]) + eps0 * ((RC)ph(i, k, j) - (RC)ph(i, k - 1, j))))) +
            (RC)dts * (RC)G * (RC)msft_inv *
                ((RC)rdn(k) * ((RC)c2a.ro(i, k, j) * (RC)alt.ro(i, k, j) * (RC)t_2ave(i, k, j) -
                               (RC)c2a.ro(i, k - 1, j) * (RC)alt.ro(i, k - 1, j) * (RC)t_2ave(i, k - 1, j)) -
                 ((RC)c1f(k) * (RC)mua));
    if (!fp64) wk = (RC)(float)wk;
    wk = (wk - Acoef(k) * wprev) * ALcoef(k);
    wcol[k] = wk;
    wprev = wk;
  }
  {
    int k = k_end + 1;
    RC r = (RC)rdnw(k - 1);
    RC wk = (RC)w(i, k, j) + (RC)dts * (RC)rw_tend.ro(i, k, j) +
            (RC)msft_inv * (-RC(.5) * (RC)dts * (RC)G / ((RC)c1h(k - 1) * (RC)mutij + (RC)c2h(k - 1)) * (r * r) * RC(2.) *
                                (RC)c2a.ro(i, k - 1, j) * (eps1 * (rhs[k] - rhs[k - 1]) + eps0 * ((RC)ph(i, k, j) - (RC)ph(i, k - 1, j))) -
                            (RC)dts * (RC)G * (RC(2.) * (RC)rdnw(k - 1) * (RC)c2a.ro(i, k - 1, j) * (RC)alt.ro(i, k - 1, j) * (RC)t_2ave(i, k - 1, j) +
                                               ((RC)c1f(k) * (RC)mua)));
    if (m.cf.top_lid) wk = RC(0.);
    if (!fp64) wk = (RC)(float)wk;
    wk = (wk - Acoef(k) * wprev) * ALcoef(k);
    wcol[k] = wk;
  }
  // damp_opt = 3 (module_small_step_em.F:1445-1458): w relaxes toward w_save
  // in the top zdamp metres after the back substitution (which runs on the
  // undamped values); the geopotential takes the damped w
  const bool damp3 = m.cf.damp_opt == 3;
  const F3 w_save = f3(m, WRFGPU_W_SAVE);
  const float hdepth = m.cf.zdamp, dampmag = dts * m.cf.dampcoef;
  const float htop = damp3 ? (ph_1.ro(i, k_end + 1, j) + phb.ro(i, k_end + 1, j)) / G : 0.f;
  auto damped = [&](int k, RC wk) -> RC {
    if (!damp3) return wk;
    const float hk = (ph_1.ro(i, k, j) + phb.ro(i, k, j)) / G;
    const float hbot = htop - hdepth;
    float dampwt = 0.f;
    if (hk >= hbot) {
      const float sn = wrfgpu_ff::sinf_cr(.5f * PI_F * (hk - hbot) / hdepth);
      dampwt = dampmag * sn * sn;
    }
    return (RC)(((float)wk - dampwt * (c1f(k) * mutij + c2f(k)) * w_save.ro(i, k, j)) / (1.f + dampwt));
  };
  // back substitution and geopotential update (downward)
  RC wup = wcol[k_end + 1];
  {
    const RC wd = damped(k_end + 1, wup);
    w(i, k_end + 1, j) = (float)wd;
    ph(i, k_end + 1, j) = (float)(rhs[k_end + 1] + (RC)my * RC(.5) * (RC)dts * (RC)G * eps1 * wd /
                                                       ((RC)c1f(k_end + 1) * (RC)mts + (RC)c2f(k_end + 1)));
  }
  for (int k = k_end; k >= 2; --k) {
    RC wk = wcol[k] - GAcoef(k) * wup;
    const RC wd = damped(k, wk);
    w(i, k, j) = (float)wd;
    ph(i, k, j) = (float)(rhs[k] + (RC)my * RC(.5) * (RC)dts * (RC)G * eps1 * wd / ((RC)c1f(k) * (RC)mts + (RC)c2f(k)));
    wup = wk;
  }
}

// ------------------------------------------------------------ sumflux (+ calc_p_rho)
__global__ void __launch_bounds__(BX* BY) k_sumflux_p_rho(Launch L, int rk_step, int iteration, int do_p_rho) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (i < m.its || i > m.ite || j < m.jts || j > m.jte || k < m.kts || k > m.kte) return;
  const Stage st = stage_of(m, rk_step);
  if (iteration > st.nsmall) return;  // members with fewer acoustic steps
  const int ns = st.nsmall;
  const int mini = min(m.ide - 1, m.ite), minj = min(m.jde - 1, m.jte), mink = min(m.kde - 1, m.kte);
  F3 ru_m = f3(m, WRFGPU_RU_M), rv_m = f3(m, WRFGPU_RV_M), ww_m = f3(m, WRFGPU_WW_M);
  float rum = iteration == 1 ? 0.f : ru_m(i, k, j);
  float rvm = iteration == 1 ? 0.f : rv_m(i, k, j);
  float wwm = iteration == 1 ? 0.f : ww_m(i, k, j);
  const bool ru_acc = j <= minj && k <= mink;            // i its..ite
  const bool rv_acc = i <= mini && k <= mink;            // j jts..jte
  const bool ww_acc = i <= mini && j <= minj;            // k kts..kte
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H);
  if (ru_acc) {
    rum = rum + f3(m, WRFGPU_U_2).ro(i, k, j);
    if (iteration == ns)
      rum = rum / float(ns) + (c1h(k) * f2(m, WRFGPU_MUU).ro(i, j) + c2h(k)) * f3(m, WRFGPU_U_SAVE).ro(i, k, j) / f2(m, WRFGPU_MSFUY).ro(i, j);
  }
  if (rv_acc) {
    rvm = rvm + f3(m, WRFGPU_V_2).ro(i, k, j);
    if (iteration == ns)
      rvm = rvm / float(ns) + (c1h(k) * f2(m, WRFGPU_MUV).ro(i, j) + c2h(k)) * f3(m, WRFGPU_V_SAVE).ro(i, k, j) * f2(m, WRFGPU_MSFVX_INV).ro(i, j);
  }
  if (ww_acc) {
    wwm = wwm + f3(m, WRFGPU_WW).ro(i, k, j);
    if (iteration == ns) wwm = wwm / float(ns) + f3(m, WRFGPU_WW1).ro(i, k, j);
  }
  if (iteration == 1 || ru_acc) ru_m(i, k, j) = rum;
  if (iteration == 1 || rv_acc) rv_m(i, k, j) = rvm;
  if (iteration == 1 || ww_acc) ww_m(i, k, j) = wwm;
  if (do_p_rho && i <= mini && j <= minj && k <= mink) calc_p_rho_point(m, i, k, j, iteration);
}

// ------------------------------------------------------------ small_step_finish
// calc_mus: form muus, muvs from muts here (calc_mu_uv_1, which solve_em
// calls right before small_step_finish, solve_em.F:1732); otherwise take the
// caller's (the routine's own interface: it reads them).
template <int MINB>
__global__ void __launch_bounds__(BX* BY, MINB) k_small_step_finish(Launch L, int rk_step, bool calc_mus) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j;
  const int i_start = m.its, i_end = min(m.ite, m.ide - 1), j_start = m.jts, j_end = min(m.jte, m.jde - 1);
  const int i_endu = m.ite, j_endv = m.jte;
  if (i < i_start || i > i_endu || j < j_start || j > j_endv) return;
  const bool px = m.cf.periodic_x, py = m.cf.periodic_y;
  const Stage st = stage_of(m, rk_step);
  F2 MU = f2(m, WRFGPU_MUTS), MUU = f2(m, WRFGPU_MUUS), MUV = f2(m, WRFGPU_MUVS);
  // calc_mu_uv_1 on (muts -> muus, muvs)
  float muus = 0.f, muvs = 0.f;
  const bool upt = j <= j_end, vpt = i <= i_end;
  if (upt && !calc_mus) muus = MUU(i, j);
  if (vpt && !calc_mus) muvs = MUV(i, j);
  if (upt && calc_mus) {
    if (i == m.ids && m.its == m.ids) { int im = px ? i - 1 : i; muus = 0.5f * (MU(i, j) + MU(im, j)); }
    else if (i == m.ide && m.ite == m.ide) { int im = px ? i : i - 1; muus = 0.5f * (MU(i - 1, j) + MU(im, j)); }
    else muus = 0.5f * (MU(i, j) + MU(i - 1, j));
    MUU(i, j) = muus;
  }
  if (vpt && calc_mus) {
    if (j == m.jds && m.jts == m.jds) { int jm = py ? j - 1 : j; muvs = 0.5f * (MU(i, j) + MU(i, jm)); }
    else if (j == m.jde && m.jte == m.jde) { int jm = py ? j : j - 1; muvs = 0.5f * (MU(i, j - 1) + MU(i, jm)); }
    else muvs = 0.5f * (MU(i, j) + MU(i, j - 1));
    MUV(i, j) = muvs;
  }
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F);
  // levels are independent: inputs of a chunk of levels are loaded first
  struct L2 { float x, s; };
  if (vpt) {
    F3 v_2 = f3(m, WRFGPU_V_2), v_save = f3(m, WRFGPU_V_SAVE);
    const float muv = f2(m, WRFGPU_MUV).ro(i, j), mx = f2(m, WRFGPU_MSFVX).ro(i, j);
    chunked_levels<8, L2>(
        m.kds, m.kde - 1, [&](int k, L2& d) { d.x = v_2(i, k, j); d.s = v_save.ro(i, k, j); },
        [&](int k, const L2& d) { v_2(i, k, j) = (mx * d.x + d.s * (c1h(k) * muv + c2h(k))) / (c1h(k) * muvs + c2h(k)); });
  }
  if (upt) {
    F3 u_2 = f3(m, WRFGPU_U_2), u_save = f3(m, WRFGPU_U_SAVE);
    const float muu = f2(m, WRFGPU_MUU).ro(i, j), my = f2(m, WRFGPU_MSFUY).ro(i, j);
    chunked_levels<8, L2>(
        m.kds, m.kde - 1, [&](int k, L2& d) { d.x = u_2(i, k, j); d.s = u_save.ro(i, k, j); },
        [&](int k, const L2& d) { u_2(i, k, j) = (my * d.x + d.s * (c1h(k) * muu + c2h(k))) / (c1h(k) * muus + c2h(k)); });
  }
  if (upt && vpt) {
    F3 w_2 = f3(m, WRFGPU_W_2), w_save = f3(m, WRFGPU_W_SAVE), ph_2 = f3(m, WRFGPU_PH_2), ph_save = f3(m, WRFGPU_PH_SAVE),
       ww = f3(m, WRFGPU_WW), ww1 = f3(m, WRFGPU_WW1), t_2 = f3(m, WRFGPU_T_2), t_save = f3(m, WRFGPU_T_SAVE),
       h_diabatic = f3(m, WRFGPU_H_DIABATIC);
    const float mt = f2(m, WRFGPU_MUT).ro(i, j), mts = MU(i, j), my = f2(m, WRFGPU_MSFTY).ro(i, j);
    const bool last = rk_step >= m.cf.rk_ord;
    struct LW { float w, ws, p, ps, ww, ww1, t, ts, hd; };
    chunked_levels<6, LW>(
        m.kds, m.kde,
        [&](int k, LW& d) {
          d.w = w_2(i, k, j); d.ws = w_save.ro(i, k, j); d.p = ph_2(i, k, j); d.ps = ph_save.ro(i, k, j);
          d.ww = ww(i, k, j); d.ww1 = ww1.ro(i, k, j);
          if (k <= m.kde - 1) {
            d.t = t_2(i, k, j); d.ts = t_save.ro(i, k, j); d.hd = last ? h_diabatic.ro(i, k, j) : 0.f;
          }
        },
        [&](int k, const LW& d) {
          w_2(i, k, j) = (my * d.w + d.ws * (c1f(k) * mt + c2f(k))) / (c1f(k) * mts + c2f(k));
          ph_2(i, k, j) = d.p + d.ps;
          ww(i, k, j) = d.ww + d.ww1;
          if (k <= m.kde - 1) {
            if (!last)
              t_2(i, k, j) = (d.t + d.ts * (c1h(k) * mt + c2h(k))) / (c1h(k) * mts + c2h(k));
            else
              t_2(i, k, j) = (d.t - st.dts_rk * float(st.nsmall) * (c1h(k) * mt + c2h(k)) * d.hd +
                              d.ts * (c1h(k) * mt + c2h(k))) / (c1h(k) * mts + c2h(k));
          }
        });
    F2 mu_2 = f2(m, WRFGPU_MU_2);
    mu_2(i, j) = mu_2(i, j) + f2(m, WRFGPU_MU_SAVE)(i, j);
  }
}

// ------------------------------------------------------------ launchers
void launch_small_step_prep(const Launch& L2, int nb2, const TileLaunch& LST, int nb_st, StepArgs a, cudaStream_t s,
                            int var) {
  k_small_step_prep_2d<<<nb2, dim3(BX, BY), 0, s>>>(L2, a.rk_step);
  k_small_step_prep_3d<<<dim3(nb_st, TUNE_PARAM[TU_SSP][var]), dim3(TX, TY), 0, s>>>(LST, a.rk_step);
}
void launch_calc_p_rho(const Launch& L, int nb, StepArgs a, cudaStream_t s) {
  k_calc_p_rho<<<nb, dim3(BX, BY), 0, s>>>(L, a.iteration);
}
void launch_calc_p_rho_col(const TileLaunch& L, int nb, StepArgs a, cudaStream_t s) {
  k_calc_p_rho_col<<<dim3(nb, 4), dim3(TX, TY), 0, s>>>(L, a.iteration);
}
void launch_calc_coef_w_col(const TileLaunch& L, int nb, StepArgs a, bool fp64, cudaStream_t s) {
  if (fp64) k_calc_coef_w_col<double><<<nb, dim3(TX, TY), 0, s>>>(L, a.rk_step);
  else k_calc_coef_w_col<float><<<nb, dim3(TX, TY), 0, s>>>(L, a.rk_step);
}
void launch_calc_coef_w(const Launch& L, int nb, StepArgs a, bool fp64, cudaStream_t s) {
  if (fp64) k_calc_coef_w<double><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step);
  else k_calc_coef_w<float><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step);
}
void launch_advance_uv(const Launch& L, int nb, StepArgs a, cudaStream_t s) {
  k_advance_uv<<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, a.iteration);
}
void launch_advance_mu_t(const Launch& L, int nb, StepArgs a, bool fp64, cudaStream_t s) {
  if (fp64) k_advance_mu_t<double><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, a.iteration);
  else k_advance_mu_t<float><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, a.iteration);
}
void launch_advance_w(const Launch& L, int nb, StepArgs a, bool fp64, cudaStream_t s) {
  if (fp64) k_advance_w<double><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, a.iteration);
  else k_advance_w<float><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, a.iteration);
}
void launch_sumflux_p_rho(const Launch& L, int nb, StepArgs a, bool do_p_rho, cudaStream_t s) {
  k_sumflux_p_rho<<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, a.iteration, do_p_rho ? 1 : 0);
}
void launch_sumflux(const Launch& L, int nb, StepArgs a, cudaStream_t s) { launch_sumflux_p_rho(L, nb, a, false, s); }
void launch_small_step_finish(const Launch& L, int nb, StepArgs a, cudaStream_t s, int var, bool calc_mus) {
  // 4 blocks of 128 threads per SM leave the registers free (~80); 8 hold them to 64
  if (var == 0) k_small_step_finish<4><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, calc_mus);
  else k_small_step_finish<8><<<nb, dim3(BX, BY), 0, s>>>(L, a.rk_step, calc_mus);
}

}  // namespace wrfgpu
