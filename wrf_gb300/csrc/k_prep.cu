// rk_step_prep (dyn_em/module_em.F:37-186) as one column kernel: one thread
// per (i,j) column computes mut, muu, muv, the coupled momenta ru/rv/rw, the
// column-integrated omega ww, cqu/cqv/cqw, alt and php for its own point.
// Roofline: HBM-bound; per mass cell it reads u, v, w, ph, phb, al, alb, qv
// (8 x 4 B) and writes ru, rv, rw, ww, php, alt, cqu, cqv, cqw (9 x 4 B).
#include "common.cuh"
#include "kernels.h"

namespace wrfgpu {

__global__ void __launch_bounds__(BX* BY) k_rk_step_prep(Launch L) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j;
  const bool px = m.cf.periodic_x, py = m.cf.periodic_y;
  F2 MU = f2(m, WRFGPU_MU_2), MUB = f2(m, WRFGPU_MUB), MUT = f2(m, WRFGPU_MUT), MUU = f2(m, WRFGPU_MUU),
     MUV = f2(m, WRFGPU_MUV);
  F2 msftx = f2(m, WRFGPU_MSFTX), msfty = f2(m, WRFGPU_MSFTY), msfuy = f2(m, WRFGPU_MSFUY),
     msfvx_inv = f2(m, WRFGPU_MSFVX_INV);
  F3 u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2), w = f3(m, WRFGPU_W_2), ph = f3(m, WRFGPU_PH_2);
  F3 ru = f3(m, WRFGPU_RU), rv = f3(m, WRFGPU_RV), rw = f3(m, WRFGPU_RW), ww = f3(m, WRFGPU_WW);
  F3 php = f3(m, WRFGPU_PHP), alt = f3(m, WRFGPU_ALT), phb = f3(m, WRFGPU_PHB), al = f3(m, WRFGPU_AL),
     alb = f3(m, WRFGPU_ALB);
  F3 cqu = f3(m, WRFGPU_CQU), cqv = f3(m, WRFGPU_CQV), cqw = f3(m, WRFGPU_CQW);
  F3 qv = f3p(m, m.q[0]);
  F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H), c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F),
     dnw = f1(m, WRFGPU_DNW);
  const int ktf = min(m.kte, m.kde - 1);
  const int itf_m = min(m.ite, m.ide - 1), jtf_m = min(m.jte, m.jde - 1);
  const float rdx = m.rdx, rdy = m.rdy;

  // calculate_full (module_big_step_utilities_em.F:3587-3636)
  float mut_ij = 0.f;
  const bool at_mass_ext = i >= m.its - 1 && i <= itf_m && j >= m.jts - 1 && j <= jtf_m;
  if (at_mass_ext) { mut_ij = MUB(i, j) + MU(i, j); MUT(i, j) = mut_ij; }
  // calc_mu_uv (module_big_step_utilities_em.F:26-181)
  float muu_ij = 0.f, muv_ij = 0.f;
  const bool at_u = i >= m.its && i <= m.ite && j >= m.jts && j <= jtf_m;
  const bool at_v = i >= m.its && i <= itf_m && j >= m.jts && j <= m.jte;
  if (at_u) {
    if (i == m.ids && m.its == m.ids) {
      int im = px ? i - 1 : i;
      muu_ij = 0.5f * (MU(i, j) + MU(im, j) + MUB(i, j) + MUB(im, j));
    } else if (i == m.ide && m.ite == m.ide) {
      int im = px ? i : i - 1;
      muu_ij = 0.5f * (MU(i - 1, j) + MU(im, j) + MUB(i - 1, j) + MUB(im, j));
    } else {
      muu_ij = 0.5f * (MU(i, j) + MU(i - 1, j) + MUB(i, j) + MUB(i - 1, j));
    }
    MUU(i, j) = muu_ij;
  }
  if (at_v) {
    if (j == m.jds && m.jts == m.jds) {
      int jm = py ? j - 1 : j;
      muv_ij = 0.5f * (MU(i, j) + MU(i, jm) + MUB(i, j) + MUB(i, jm));
    } else if (j == m.jde && m.jte == m.jde) {
      int jm = py ? j : j - 1;
      muv_ij = 0.5f * (MU(i, j - 1) + MU(i, jm) + MUB(i, j - 1) + MUB(i, jm));
    } else {
      muv_ij = 0.5f * (MU(i, j) + MU(i, j - 1) + MUB(i, j) + MUB(i, j - 1));
    }
    MUV(i, j) = muv_ij;
  }
  // couple_momentum (:329-391)
  if (at_u)
    for (int k = m.kts; k <= ktf; ++k) ru(i, k, j) = u(i, k, j) * (c1h(k) * muu_ij + c2h(k)) / msfuy(i, j);
  if (at_v)
    for (int k = m.kts; k <= ktf; ++k) rv(i, k, j) = v(i, k, j) * (c1h(k) * muv_ij + c2h(k)) * msfvx_inv(i, j);
  const bool at_t = i >= m.its && i <= itf_m && j >= m.jts && j <= jtf_m;
  if (at_t)
    for (int k = m.kts; k <= m.kte; ++k) rw(i, k, j) = w(i, k, j) * (c1f(k) * mut_ij + c2f(k)) / msfty(i, j);
  // calc_ww_cp (:640-784); the staggered mass averages are formed locally.
  if (i >= m.its && i <= m.ite && j >= m.jts && j <= jtf_m) {
    ww(i, 1, j) = 0.f;
    ww(i, m.kte, j) = 0.f;
  }
  if (at_t) {
    const float muu0 = 0.5f * (MU(i, j) + MUB(i, j) + MU(i - 1, j) + MUB(i - 1, j));
    const float muu1 = 0.5f * (MU(i + 1, j) + MUB(i + 1, j) + MU(i, j) + MUB(i, j));
    const float muv0 = 0.5f * (MU(i, j) + MUB(i, j) + MU(i, j - 1) + MUB(i, j - 1));
    const float muv1 = 0.5f * (MU(i, j + 1) + MUB(i, j + 1) + MU(i, j) + MUB(i, j));
    const float mx = msftx(i, j), uy0 = msfuy(i, j), uy1 = msfuy(i + 1, j);
    const float vi0 = msfvx_inv(i, j), vi1 = msfvx_inv(i, j + 1);
    auto divv = [&](int k) -> float {
      return mx * dnw(k) *
             (rdx * ((c1h(k) * muu1 + c2h(k)) * u(i + 1, k, j) / uy1 - (c1h(k) * muu0 + c2h(k)) * u(i, k, j) / uy0) +
              rdy * ((c1h(k) * muv1 + c2h(k)) * v(i, k, j + 1) * vi1 - (c1h(k) * muv0 + c2h(k)) * v(i, k, j) * vi0));
    };
    float dmdt = 0.f;
    for (int k = m.kts; k <= ktf; ++k) dmdt = dmdt + divv(k);
    float wwk = ww(i, 1, j);
    for (int k = 2; k <= ktf; ++k) {
      wwk = wwk - dnw(k - 1) * c1h(k - 1) * dmdt - divv(k - 1);
      ww(i, k, j) = wwk;
    }
  }
  // calc_cq (:787-907) with qv the only moist species
  if (at_u)
    for (int k = m.kts; k <= ktf; ++k) {
      float qtot = 0.f + qv(i, k, j) + qv(i - 1, k, j);
      cqu(i, k, j) = 1.f / (1.f + 0.5f * qtot);
    }
  if (at_v)
    for (int k = m.kts; k <= ktf; ++k) {
      float qtot = 0.f + qv(i, k, j) + qv(i, k, j - 1);
      cqv(i, k, j) = 1.f / (1.f + 0.5f * qtot);
    }
  if (at_t) {
    for (int k = m.kts + 1; k <= ktf; ++k) {
      float qtot = 0.f + qv(i, k, j) + qv(i, k - 1, j);
      cqw(i, k, j) = 0.5f * qtot;
    }
    // calc_alt (:910-950), calc_php (:1227-1262)
    for (int k = m.kts; k <= ktf; ++k) {
      alt(i, k, j) = al(i, k, j) + alb(i, k, j);
      php(i, k, j) = 0.5f * (phb(i, k, j) + phb(i, k + 1, j) + ph(i, k, j) + ph(i, k + 1, j));
    }
  }
}

void launch_rk_step_prep(const Launch& L, int nblocks, cudaStream_t s) {
  k_rk_step_prep<<<nblocks, dim3(BX, BY), 0, s>>>(L);
}

}  // namespace wrfgpu
