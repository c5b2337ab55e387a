// rk_step_prep (dyn_em/module_em.F:37-186) as one column kernel: one thread
// per (i,j) column computes mut, muu, muv, the coupled momenta ru/rv/rw, the
// column-integrated omega ww, cqu/cqv/cqw, alt and php for its own point.
// Roofline: HBM-bound; per mass cell it reads u, v, w, ph, phb, al, alb, qv
// (8 x 4 B) and writes ru, rv, rw, ww, php, alt, cqu, cqv, cqw (9 x 4 B).
#include "common.cuh"
#include "kernels.h"

namespace wrfgpu {

template <int MINB>
__global__ void __launch_bounds__(BX* BY, MINB) k_rk_step_prep(Launch L) {
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
  // couple_momentum (:329-391) and calc_cq (:787-907, qv the only moist
  // species) on the u and v points: levels loaded in chunks (independent levels)
  if (at_u) {
    const float my = msfuy.ro(i, j);
    struct LU { float u, q0, q1; };
    chunked_levels<8, LU>(
        m.kts, ktf, [&](int k, LU& d) { d.u = u.ro(i, k, j); d.q0 = qv.ro(i, k, j); d.q1 = qv.ro(i - 1, k, j); },
        [&](int k, const LU& d) {
          ru(i, k, j) = d.u * (c1h(k) * muu_ij + c2h(k)) / my;
          float qtot = 0.f + d.q0 + d.q1;
          cqu(i, k, j) = 1.f / (1.f + 0.5f * qtot);
        });
  }
  if (at_v) {
    const float mxi = msfvx_inv.ro(i, j);
    struct LV { float v, q0, q1; };
    chunked_levels<8, LV>(
        m.kts, ktf, [&](int k, LV& d) { d.v = v.ro(i, k, j); d.q0 = qv.ro(i, k, j); d.q1 = qv.ro(i, k, j - 1); },
        [&](int k, const LV& d) {
          rv(i, k, j) = d.v * (c1h(k) * muv_ij + c2h(k)) * mxi;
          float qtot = 0.f + d.q0 + d.q1;
          cqv(i, k, j) = 1.f / (1.f + 0.5f * qtot);
        });
  }
  const bool at_t = i >= m.its && i <= itf_m && j >= m.jts && j <= jtf_m;
  // calc_ww_cp (:640-784); the staggered mass averages are formed locally.
  if (i >= m.its && i <= m.ite && j >= m.jts && j <= jtf_m) {
    ww(i, 1, j) = 0.f;
    ww(i, m.kte, j) = 0.f;
  }
  if (at_t) {
    const float muu0 = 0.5f * (MU.ro(i, j) + MUB.ro(i, j) + MU.ro(i - 1, j) + MUB.ro(i - 1, j));
    const float muu1 = 0.5f * (MU.ro(i + 1, j) + MUB.ro(i + 1, j) + MU.ro(i, j) + MUB.ro(i, j));
    const float muv0 = 0.5f * (MU.ro(i, j) + MUB.ro(i, j) + MU.ro(i, j - 1) + MUB.ro(i, j - 1));
    const float muv1 = 0.5f * (MU.ro(i, j + 1) + MUB.ro(i, j + 1) + MU.ro(i, j) + MUB.ro(i, j));
    const float mx = msftx.ro(i, j), uy0 = msfuy.ro(i, j), uy1 = msfuy.ro(i + 1, j);
    const float vi0 = msfvx_inv.ro(i, j), vi1 = msfvx_inv.ro(i, j + 1);
    float dv[129];
    float dmdt = 0.f;
    struct LD { float u0, u1, v0, v1; };
    chunked_levels<8, LD>(
        m.kts, ktf,
        [&](int k, LD& d) { d.u0 = u.ro(i, k, j); d.u1 = u.ro(i + 1, k, j); d.v0 = v.ro(i, k, j); d.v1 = v.ro(i, k, j + 1); },
        [&](int k, const LD& d) {
          const float dvv =
              mx * dnw(k) *
              (rdx * ((c1h(k) * muu1 + c2h(k)) * d.u1 / uy1 - (c1h(k) * muu0 + c2h(k)) * d.u0 / uy0) +
               rdy * ((c1h(k) * muv1 + c2h(k)) * d.v1 * vi1 - (c1h(k) * muv0 + c2h(k)) * d.v0 * vi0));
          dv[k] = dvv;
          dmdt = dmdt + dvv;
        });
    float wwk = 0.f;  // ww(i, 1, j), set to zero above by this thread
    // the recursion's loads (dv sits in local memory) go out eight levels at a time
    chunked_levels<8, float>(
        2, ktf, [&](int k, float& d) { d = dv[k - 1]; },
        [&](int k, const float& d) {
          wwk = wwk - dnw(k - 1) * c1h(k - 1) * dmdt - d;
          ww(i, k, j) = wwk;
        });
    // couple_momentum rw (:329-391), calc_cq cqw, calc_alt (:910-950), calc_php (:1227-1262)
    const float my = msfty.ro(i, j);
    struct LT { float w, q0, qm, al, alb, phb0, phb1, ph0, ph1; };
    chunked_levels<6, LT>(
        m.kts, m.kte,
        [&](int k, LT& d) {
          d.w = w.ro(i, k, j);
          if (k <= ktf) {
            d.q0 = qv.ro(i, k, j); d.qm = k > m.kts ? qv.ro(i, k - 1, j) : 0.f;
            d.al = al.ro(i, k, j); d.alb = alb.ro(i, k, j);
            d.phb0 = phb.ro(i, k, j); d.phb1 = phb.ro(i, k + 1, j); d.ph0 = ph.ro(i, k, j); d.ph1 = ph.ro(i, k + 1, j);
          }
        },
        [&](int k, const LT& d) {
          rw(i, k, j) = d.w * (c1f(k) * mut_ij + c2f(k)) / my;
          if (k <= ktf) {
            if (k >= m.kts + 1) {
              float qtot = 0.f + d.q0 + d.qm;
              cqw(i, k, j) = 0.5f * qtot;
            }
            alt(i, k, j) = d.al + d.alb;
            php(i, k, j) = 0.5f * (d.phb0 + d.phb1 + d.ph0 + d.ph1);
          }
        });
  }
}

void launch_rk_step_prep(const Launch& L, int nblocks, cudaStream_t s, int var) {
  // 3 blocks of 128 threads per SM leave the register count free (88);
  // 8 hold it to 64 for twice the resident warps
  if (var == 0) k_rk_step_prep<3><<<nblocks, dim3(BX, BY), 0, s>>>(L);
  else k_rk_step_prep<8><<<nblocks, dim3(BX, BY), 0, s>>>(L);
}

}  // namespace wrfgpu
