// Column-marching forms of the u and v large-step tendencies (rk_tendency,
// module_em.F:129-560 with advect_u / advect_v, module_advect_em.F:205-1700
// for 5th/3rd order; horizontal_pressure_gradient, module_big_step_utilities_em.F:1585-1718;
// coriolis :3106-3215; curvature :3234-3363).
//
// One thread per (i, j) column of a 32 x 8 tile of the staggered extents,
// levels kts..kte in order (or one chunk of them per block along y).  For u
// and v, the advected field and the mass fluxes ru, rv of each level arrive
// by TMA as halo planes, several levels ahead, and every horizontal face
// flux is formed once, in shared memory, instead of once by each of the two
// columns it separates.  The per-point arithmetic is that of the point
// kernels in k_tend.cu, term for term and in the same order, with three
// exact reuses across levels:
//   * the vertical flux of face k+1 is the lower face of level k+1,
//   * dpn(k+1) of the pressure-gradient correction is dpn(k) one level up,
//   * values at level k+1 (p, ph, rw of the two columns) carry down,
// and the column-invariant products of map factors, Coriolis parameters and
// grid constants are formed once per column, in the reference's order of
// operations (so every rounding is unchanged).  The next levels' own-column
// inputs are prefetched into L2 two levels ahead.
#include "common.cuh"
#include "kernels.h"
#include "open_adv.cuh"

namespace wrfgpu {

// Staged planes of the advected field and the two mass fluxes: the tile plus
// a 4-point halo, (TX + 8) x (TY + 8) from (i0 - 4, j0 - 4), TEND_RING levels
// in flight; the x and y face fluxes of a level are formed once each into
// shared memory (double-buffered), so one block barrier per level suffices.
constexpr int HALO_W = TX + 2 * TMA_HALO, HALO_H = TY + 2 * TMA_HALO;
constexpr int TEND_RING = 4;
using HaloRing = LevelRing<3, TEND_RING, HALO_W, HALO_H>;
constexpr int FXN = TY * (TX + 1), FYN = (TY + 1) * TX;
constexpr size_t TEND_SMEM = HaloRing::SMEM + 2 * (FXN + FYN) * 4;

// The tile's x faces (columns i0 .. i0+TX of rows j0 .. j0+TY-1) and y faces
// (rows j0 .. j0+TY of columns i0 .. i0+TX-1) of one level: 5th-order fluxes
// of Q with the face velocity vx(o) / vy(o), o the face's upper point in the
// halo plane.  Each thread forms its cell's left and bottom faces; the last
// column's right faces go to warp TY-1, the last row's top faces to warp TY-2.
template <class VX, class VY>
__device__ __forceinline__ void tile_faces(const float* Q, float* FX, float* FY, VX vx, VY vy, int tx, int ty) {
  auto xface = [&](int r, int c) {
    const int o = (r + TMA_HALO) * HALO_W + c + TMA_HALO;
    const float vel = vx(o);
    FX[r * (TX + 1) + c] = vel * flux5(Q[o - 3], Q[o - 2], Q[o - 1], Q[o], Q[o + 1], Q[o + 2], vel);
  };
  auto yface = [&](int r, int c) {
    const int o = (r + TMA_HALO) * HALO_W + c + TMA_HALO;
    const float vel = vy(o);
    FY[r * TX + c] = vel * flux5(Q[o - 3 * HALO_W], Q[o - 2 * HALO_W], Q[o - HALO_W], Q[o], Q[o + HALO_W],
                                 Q[o + 2 * HALO_W], vel);
  };
  xface(ty, tx);
  yface(ty, tx);
  if (ty == TY - 1 && tx < TY) xface(tx, TX);
  if (ty == TY - 2) yface(TY, tx);
}

// Level chunk of this block (gridDim.y chunks of kts..ktf).
struct Chunk { int k0, k1; };
__device__ __forceinline__ Chunk level_chunk_of(int kts, int ktf) {
  const int per = (ktf - kts + 1 + (int)gridDim.y - 1) / (int)gridDim.y;
  const int k0 = kts + (int)blockIdx.y * per;
  return Chunk{k0, min(ktf, k0 + per - 1)};
}

// ---------------------------------------------------------------- ru_tend
// A level's point inputs of the u (v) tendency beyond the staged planes, with
// the sums and differences of the two columns formed as the reference's
// expressions form them (so every rounding is unchanged): the tendency so
// far, the advected field three levels up, the omega sum of the face above,
// rw, p and ph one level up, alt, al, pb, php and cqu (cqv) of the two
// columns, and the two sums of the cross velocity for the curvature term.
struct LevelIn {
  float t, f3, romsum, rw_l1, rw_r1, p_l1, p_r1, ph_l1, ph_r1, altsum, alsum, pbd, phpd, cq, cs_r, cs_l;
};
// They are loaded together, right before the level's arithmetic, so their
// latencies overlap one another (interleaved with the arithmetic that uses
// them, the kernel took 1.63 instead of 1.31 ms per 512x512x80 step).
template <int FL, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_tend_u_col(TileLaunch L) {
  static_assert(FL & TF_ADV, "the staged form includes advection");
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i = tp.i0 + tx, j = tp.j0 + ty;
  const F3 tend = f3(m, WRFGPU_RU_TEND);
  const int kts = m.kts, kte = m.kte, kde = m.kde, kme = m.kme, ktf = min(kte, kde - 1);
  const int jacc = min(m.jte, m.jde - 1);
  const bool inside = i <= m.ite && j <= m.jte;
  const bool acc = inside && j <= jacc;
  if ((FL & TF_ZERO) && inside && !acc && blockIdx.y == 0)
    for (int k = kts; k <= kte; ++k) tend(i, k, j) = 0.f;
  const Chunk ch = level_chunk_of(kts, ktf);
  const int k0 = ch.k0, k1 = ch.k1;
  if (tp.i0 <= m.ite && tp.j0 <= jacc && k0 <= k1) {  // block-uniform
    const F3 u = f3(m, WRFGPU_U_2), rw = f3(m, WRFGPU_RW), rom = f3(m, WRFGPU_WW);
    const F3 ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT), p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB),
             al = f3(m, WRFGPU_AL), php = f3(m, WRFGPU_PHP), cqu = f3(m, WRFGPU_CQU), v = f3(m, WRFGPU_V_2);
    const F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzw = f1(m, WRFGPU_RDNW), c1h = f1(m, WRFGPU_C1H),
             c2h = f1(m, WRFGPU_C2H);
    const float rdx = m.rdx, rdy = m.rdy;
    HaloRing ring;
    ring.init(smem, k0);
    float* FXb = (float*)(smem + HaloRing::SMEM);
    float* FYb = FXb + 2 * FXN;
    const CUtensorMap* maps[3] = {tmap_of(m, WRFGPU_U_2, BOX_HALO), tmap_of(m, WRFGPU_RU, BOX_HALO),
                                  tmap_of(m, WRFGPU_RV, BOX_HALO)};
    const int x0 = tp.i0 - TMA_HALO - m.ims, z0 = tp.j0 - TMA_HALO - m.jms;
    if (tid == 0) {
      ring.init_barriers();
      mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int d = 0; d < TEND_RING - 1 && k0 + d <= k1; ++d) ring.issue(k0 + d, maps, x0, z0, m.kms);
    // column constants
    float mrdy = 0.f, mrdx = 0.f, ratio = 0.f, pgA = 0.f, pgB = 0.f;
    float muu_c = 0.f, mu_l = 0.f, mu_r = 0.f, corA = 0.f, corB = 0.f;
    float dvx_l = 0.f, dvx_r = 0.f, duy_l = 0.f, duy_r = 0.f;
    // own-column window of u for the vertical flux u(k-1 .. k+2), the vertical
    // flux of face k, and the pressure-gradient / rw carries (formed afresh at
    // the chunk's first level k0, with the same expressions as one level down)
    float um1 = 0.f, u0 = 0.f, up1 = 0.f, up2 = 0.f, vf_lo = 0.f;
    float p_l = 0.f, p_r = 0.f, ph_l = 0.f, ph_r = 0.f, dpn_lo = 0.f, rw_l = 0.f, rw_r = 0.f;
    if (acc) {
      const F2 msfux = f2(m, WRFGPU_MSFUX), msfuy = f2(m, WRFGPU_MSFUY);
      const float msfux_c = msfux(i, j), msfuy_c = msfuy(i, j);
      mrdy = msfux_c * rdy; mrdx = msfux_c * rdx;
      ratio = msfux_c / msfuy_c;
      pgA = ratio * .5f * rdx; pgB = ratio * rdx;
      if (FL & TF_PG) {
        muu_c = f2(m, WRFGPU_MUU)(i, j);
        mu_l = f2(m, WRFGPU_MU_2)(i - 1, j);
        mu_r = f2(m, WRFGPU_MU_2)(i, j);
      }
      if (FL & TF_COR) {
        const F2 f = f2(m, WRFGPU_F), e = f2(m, WRFGPU_E), cosa = f2(m, WRFGPU_COSA);
        corA = ratio * 0.5f * (f(i, j) + f(i - 1, j)) * 0.25f;
        corB = 0.5f * (e(i, j) + e(i - 1, j)) * 0.5f * (cosa(i, j) + cosa(i - 1, j)) * 0.25f;
      }
      if (FL & TF_CURV) {
        const F2 msfvx = f2(m, WRFGPU_MSFVX);
        dvx_r = msfvx(i, j + 1) - msfvx(i, j);
        dvx_l = msfvx(i - 1, j + 1) - msfvx(i - 1, j);
        duy_r = msfuy(i + 1, j) - msfuy(i, j);
        duy_l = msfuy(i, j) - msfuy(i - 1, j);
      }
      um1 = (k0 - 1 >= kts) ? u(i, k0 - 1, j) : 0.f; u0 = u(i, k0, j); up1 = u(i, k0 + 1, j);
      up2 = (k0 + 2 <= kme) ? u(i, k0 + 2, j) : 0.f;
      {
        const int kk = k0;
        if (kk == kts || kk == kte) vf_lo = 0.f;
        else if (kk == kts + 1 || kk == ktf)
          vf_lo = 0.5f * (rom(i, kk, j) + rom(i - 1, kk, j)) * (fzm(kk) * u0 + fzp(kk) * um1);
        else {
          const float vel = 0.5f * (rom(i - 1, kk, j) + rom(i, kk, j));
          vf_lo = vel * flux3(u(i, kk - 2, j), um1, u0, up1, -vel);
        }
      }
      if (FL & TF_PG) {
        p_l = p(i - 1, k0, j); p_r = p(i, k0, j);
        ph_l = ph(i - 1, k0, j); ph_r = ph(i, k0, j);
        if (k0 == 1)
          dpn_lo = .5f * (m.cf1 * (p(i - 1, 1, j) + p(i, 1, j)) + m.cf2 * (p(i - 1, 2, j) + p(i, 2, j)) +
                          m.cf3 * (p(i - 1, 3, j) + p(i, 3, j)));
        else
          dpn_lo = .5f * (fzm(k0) * (p_l + p_r) + fzp(k0) * (p(i - 1, k0 - 1, j) + p(i, k0 - 1, j)));
      }
      if (FL & (TF_COR | TF_CURV)) { rw_l = rw(i - 1, k0, j); rw_r = rw(i, k0, j); }
    }
    const int o = (ty + TMA_HALO) * HALO_W + tx + TMA_HALO;  // own point in the halo planes
    auto load_in = [&](int k) {
      LevelIn q;
      q.t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
      q.f3 = (k + 3 <= kme) ? u(i, k + 3, j) : 0.f;
      const int kk = k + 1;
      // rom(i) + rom(i-1) = rom(i-1) + rom(i) exactly: IEEE addition commutes
      q.romsum = (kk == kts || kk == kte) ? 0.f : rom(i, kk, j) + rom(i - 1, kk, j);
      q.rw_l1 = q.rw_r1 = 0.f;
      if (FL & (TF_COR | TF_CURV)) { q.rw_l1 = rw(i - 1, k + 1, j); q.rw_r1 = rw(i, k + 1, j); }
      q.p_l1 = q.p_r1 = q.ph_l1 = q.ph_r1 = q.altsum = q.alsum = q.pbd = q.phpd = q.cq = 0.f;
      if (FL & TF_PG) {
        if (kk != kde) { q.p_l1 = p(i - 1, kk, j); q.p_r1 = p(i, kk, j); }
        q.ph_l1 = ph(i - 1, k + 1, j); q.ph_r1 = ph(i, k + 1, j);
        q.altsum = alt(i, k, j) + alt(i - 1, k, j);
        q.alsum = al(i, k, j) + al(i - 1, k, j);
        q.pbd = pb(i, k, j) - pb(i - 1, k, j);
        q.phpd = php(i, k, j) - php(i - 1, k, j);
        q.cq = cqu(i, k, j);
      }
      q.cs_r = q.cs_l = 0.f;
      if (FL & TF_CURV) { q.cs_r = v(i, k, j) + v(i, k, j + 1); q.cs_l = v(i - 1, k, j) + v(i - 1, k, j + 1); }
      return q;
    };
    bool ok = true;
    for (int k = k0; k <= k1; ++k) {
      ok = ring.wait(k) && ok;
      const float* U = ring.plane(k, 0);
      const float* RU = ring.plane(k, 1);
      const float* RV = ring.plane(k, 2);
      float* FX = FXb + (k & 1) * FXN;
      float* FY = FYb + (k & 1) * FYN;
      tile_faces(U, FX, FY, [&](int q) { return 0.5f * (RU[q] + RU[q - 1]); },
                 [&](int q) { return 0.5f * (RV[q] + RV[q - 1]); }, tx, ty);
      __syncthreads();
      // the slot of level k-1, which every thread has finished with
      if (tid == 0 && k + TEND_RING - 1 <= k1) ring.issue(k + TEND_RING - 1, maps, x0, z0, m.kms);
      if (!acc) continue;
      if (k + 2 <= kme) {
        prefetch_l2(&rom(i, k + 2, j)); prefetch_l2(&p(i, k + 2, j)); prefetch_l2(&ph(i, k + 2, j));
        prefetch_l2(&alt(i, k + 2, j)); prefetch_l2(&al(i, k + 2, j)); prefetch_l2(&pb(i, k + 2, j));
        prefetch_l2(&php(i, k + 2, j)); prefetch_l2(&cqu(i, k + 2, j)); prefetch_l2(&rw(i, k + 2, j));
        prefetch_l2(&v(i, k + 2, j)); prefetch_l2(&tend(i, k + 2, j));
      }
      const LevelIn q = load_in(k);
      float t = q.t;
      t = t - mrdy * (FY[(ty + 1) * TX + tx] - FY[ty * TX + tx]);
      t = t - mrdx * (FX[ty * (TX + 1) + tx + 1] - FX[ty * (TX + 1) + tx]);
      {  // vertical flux of face k+1
        const int kk = k + 1;
        float vf_hi;
        if (kk == kts || kk == kte) vf_hi = 0.f;
        else if (kk == kts + 1 || kk == ktf)
          vf_hi = 0.5f * q.romsum * (fzm(kk) * up1 + fzp(kk) * u0);
        else {
          const float vel = 0.5f * q.romsum;
          vf_hi = vel * flux3(um1, u0, up1, up2, -vel);
        }
        t = t - rdzw(k) * (vf_hi - vf_lo);
        vf_lo = vf_hi;
      }
      if (FL & TF_PG) {
        const int kk = k + 1;
        float dpn_hi;
        if (kk == kde) {
          if (m.cf.top_lid)
            dpn_hi = .5f * (m.cfn * (p(i - 1, kde - 1, j) + p(i, kde - 1, j)) +
                            m.cfn1 * (p(i - 1, kde - 2, j) + p(i, kde - 2, j)));
          else dpn_hi = 0.f;
        } else {
          dpn_hi = .5f * (fzm(kk) * (q.p_l1 + q.p_r1) + fzp(kk) * (p_l + p_r));
        }
        float dpx = pgA * (c1h(k) * muu_c + c2h(k)) *
                    ((q.ph_r1 - q.ph_l1 + ph_r - ph_l) + q.altsum * (p_r - p_l) + q.alsum * q.pbd);
        dpx = dpx + pgB * q.phpd * (rdzw(k) * (dpn_hi - dpn_lo) - .5f * ((c1h(k) * mu_l) + (c1h(k) * mu_r)));
        t = t - q.cq * dpx;
        dpn_lo = dpn_hi;
        p_l = q.p_l1; p_r = q.p_r1; ph_l = q.ph_l1; ph_r = q.ph_r1;
      }
      if (FL & (TF_COR | TF_CURV)) {
        const float rvsum = RV[o + HALO_W - 1] + RV[o + HALO_W] + RV[o - 1] + RV[o];
        const float rwsum = q.rw_l1 + rw_l + q.rw_r1 + rw_r;
        if (FL & TF_COR) t = t + corA * rvsum - corB * rwsum;
        if (FL & TF_CURV) {
          const float vx_r = 0.5f * (u0 + U[o + 1]) * dvx_r * rdy - 0.5f * q.cs_r * duy_r * rdx;
          const float vx_l = 0.5f * (U[o - 1] + u0) * dvx_l * rdy - 0.5f * q.cs_l * duy_l * rdx;
          t = t + 0.5f * (vx_r + vx_l) * 0.25f * rvsum - u0 * RERADIUS * 0.25f * rwsum;
        }
      }
      rw_l = q.rw_l1; rw_r = q.rw_r1;
      tend(i, k, j) = t;
      um1 = u0; u0 = up1; up1 = up2; up2 = q.f3;
    }
    if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
  }
  if ((FL & TF_ZERO) && acc && blockIdx.y == gridDim.y - 1)
    for (int k = ktf + 1; k <= kte; ++k) tend(i, k, j) = 0.f;
}

// ---------------------------------------------------------------- rv_tend
template <int FL, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_tend_v_col(TileLaunch L) {
  static_assert(FL & TF_ADV, "the staged form includes advection");
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i = tp.i0 + tx, j = tp.j0 + ty;
  const F3 tend = f3(m, WRFGPU_RV_TEND);
  const int kts = m.kts, kte = m.kte, kde = m.kde, kme = m.kme, ktf = min(kte, kde - 1);
  const int iacc = min(m.ite, m.ide - 1);
  const bool inside = i <= m.ite && j <= m.jte;
  const bool acc = inside && i <= iacc;
  if ((FL & TF_ZERO) && inside && !acc && blockIdx.y == 0)
    for (int k = kts; k <= kte; ++k) tend(i, k, j) = 0.f;
  const Chunk ch = level_chunk_of(kts, ktf);
  const int k0 = ch.k0, k1 = ch.k1;
  if (tp.i0 <= iacc && tp.j0 <= m.jte && k0 <= k1) {  // block-uniform
    const F3 v = f3(m, WRFGPU_V_2), rw = f3(m, WRFGPU_RW), rom = f3(m, WRFGPU_WW);
    const F3 ph = f3(m, WRFGPU_PH_2), alt = f3(m, WRFGPU_ALT), p = f3(m, WRFGPU_P), pb = f3(m, WRFGPU_PB),
             al = f3(m, WRFGPU_AL), php = f3(m, WRFGPU_PHP), cqv = f3(m, WRFGPU_CQV), u = f3(m, WRFGPU_U_2);
    const F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzw = f1(m, WRFGPU_RDNW), c1h = f1(m, WRFGPU_C1H),
             c2h = f1(m, WRFGPU_C2H);
    const float rdx = m.rdx, rdy = m.rdy;
    HaloRing ring;
    ring.init(smem, k0);
    float* FXb = (float*)(smem + HaloRing::SMEM);
    float* FYb = FXb + 2 * FXN;
    const CUtensorMap* maps[3] = {tmap_of(m, WRFGPU_V_2, BOX_HALO), tmap_of(m, WRFGPU_RU, BOX_HALO),
                                  tmap_of(m, WRFGPU_RV, BOX_HALO)};
    const int x0 = tp.i0 - TMA_HALO - m.ims, z0 = tp.j0 - TMA_HALO - m.jms;
    if (tid == 0) {
      ring.init_barriers();
      mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int d = 0; d < TEND_RING - 1 && k0 + d <= k1; ++d) ring.issue(k0 + d, maps, x0, z0, m.kms);
    float mrdy = 0.f, mrdx = 0.f, ratio = 0.f, pgA = 0.f, pgB = 0.f;
    float muv_c = 0.f, mu_l = 0.f, mu_r = 0.f, corA = 0.f, corB = 0.f;
    float dvx_l = 0.f, dvx_r = 0.f, duy_l = 0.f, duy_r = 0.f;
    float vm1 = 0.f, v0 = 0.f, vp1 = 0.f, vp2 = 0.f, vf_lo = 0.f;
    float p_l = 0.f, p_r = 0.f, ph_l = 0.f, ph_r = 0.f, dpn_lo = 0.f, rw_l = 0.f, rw_r = 0.f;
    if (acc) {
      const F2 msfvx = f2(m, WRFGPU_MSFVX), msfvy = f2(m, WRFGPU_MSFVY);
      const float msfvy_c = msfvy(i, j), msfvx_c = msfvx(i, j);
      mrdy = msfvy_c * rdy; mrdx = msfvy_c * rdx;
      ratio = msfvy_c / msfvx_c;
      pgA = ratio * .5f * rdy; pgB = ratio * rdy;
      if (FL & TF_PG) {
        muv_c = f2(m, WRFGPU_MUV)(i, j);
        mu_l = f2(m, WRFGPU_MU_2)(i, j - 1);
        mu_r = f2(m, WRFGPU_MU_2)(i, j);
      }
      if (FL & TF_COR) {
        const F2 f = f2(m, WRFGPU_F), e = f2(m, WRFGPU_E), sina = f2(m, WRFGPU_SINA);
        corA = ratio * 0.5f * (f(i, j) + f(i, j - 1)) * 0.25f;
        corB = ratio * 0.5f * (e(i, j) + e(i, j - 1)) * 0.5f * (sina(i, j) + sina(i, j - 1)) * 0.25f;
      }
      if (FL & TF_CURV) {
        const F2 msfuy = f2(m, WRFGPU_MSFUY);
        dvx_r = msfvx(i, j + 1) - msfvx(i, j);
        dvx_l = msfvx(i, j) - msfvx(i, j - 1);
        duy_r = msfuy(i + 1, j) - msfuy(i, j);
        duy_l = msfuy(i + 1, j - 1) - msfuy(i, j - 1);
      }
      vm1 = (k0 - 1 >= kts) ? v(i, k0 - 1, j) : 0.f; v0 = v(i, k0, j); vp1 = v(i, k0 + 1, j);
      vp2 = (k0 + 2 <= kme) ? v(i, k0 + 2, j) : 0.f;
      {
        const int kk = k0;
        if (kk == kts || kk == kte) vf_lo = 0.f;
        else if (kk == kts + 1 || kk == ktf)
          vf_lo = 0.5f * (rom(i, kk, j) + rom(i, kk, j - 1)) * (fzm(kk) * v0 + fzp(kk) * vm1);
        else {
          const float vel = 0.5f * (rom(i, kk, j) + rom(i, kk, j - 1));
          vf_lo = vel * flux3(v(i, kk - 2, j), vm1, v0, vp1, -vel);
        }
      }
      if (FL & TF_PG) {
        p_l = p(i, k0, j - 1); p_r = p(i, k0, j);
        ph_l = ph(i, k0, j - 1); ph_r = ph(i, k0, j);
        if (k0 == 1)
          dpn_lo = .5f * (m.cf1 * (p(i, 1, j - 1) + p(i, 1, j)) + m.cf2 * (p(i, 2, j - 1) + p(i, 2, j)) +
                          m.cf3 * (p(i, 3, j - 1) + p(i, 3, j)));
        else
          dpn_lo = .5f * (fzm(k0) * (p_l + p_r) + fzp(k0) * (p(i, k0 - 1, j - 1) + p(i, k0 - 1, j)));
      }
      if (FL & (TF_COR | TF_CURV)) { rw_l = rw(i, k0, j - 1); rw_r = rw(i, k0, j); }
    }
    const int o = (ty + TMA_HALO) * HALO_W + tx + TMA_HALO;
    auto load_in = [&](int k) {
      LevelIn q;
      q.t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
      q.f3 = (k + 3 <= kme) ? v(i, k + 3, j) : 0.f;
      const int kk = k + 1;
      q.romsum = (kk == kts || kk == kte) ? 0.f : rom(i, kk, j) + rom(i, kk, j - 1);
      q.rw_l1 = q.rw_r1 = 0.f;
      if (FL & (TF_COR | TF_CURV)) { q.rw_l1 = rw(i, k + 1, j - 1); q.rw_r1 = rw(i, k + 1, j); }
      q.p_l1 = q.p_r1 = q.ph_l1 = q.ph_r1 = q.altsum = q.alsum = q.pbd = q.phpd = q.cq = 0.f;
      if (FL & TF_PG) {
        if (kk != kde) { q.p_l1 = p(i, kk, j - 1); q.p_r1 = p(i, kk, j); }
        q.ph_l1 = ph(i, k + 1, j - 1); q.ph_r1 = ph(i, k + 1, j);
        q.altsum = alt(i, k, j) + alt(i, k, j - 1);
        q.alsum = al(i, k, j) + al(i, k, j - 1);
        q.pbd = pb(i, k, j) - pb(i, k, j - 1);
        q.phpd = php(i, k, j) - php(i, k, j - 1);
        q.cq = cqv(i, k, j);
      }
      q.cs_r = q.cs_l = 0.f;
      if (FL & TF_CURV) { q.cs_r = u(i, k, j) + u(i + 1, k, j); q.cs_l = u(i, k, j - 1) + u(i + 1, k, j - 1); }
      return q;
    };
    bool ok = true;
    for (int k = k0; k <= k1; ++k) {
      ok = ring.wait(k) && ok;
      const float* V = ring.plane(k, 0);
      const float* RU = ring.plane(k, 1);
      const float* RV = ring.plane(k, 2);
      float* FX = FXb + (k & 1) * FXN;
      float* FY = FYb + (k & 1) * FYN;
      tile_faces(V, FX, FY, [&](int q) { return 0.5f * (RU[q] + RU[q - HALO_W]); },
                 [&](int q) { return 0.5f * (RV[q] + RV[q - HALO_W]); }, tx, ty);
      __syncthreads();
      if (tid == 0 && k + TEND_RING - 1 <= k1) ring.issue(k + TEND_RING - 1, maps, x0, z0, m.kms);
      if (!acc) continue;
      if (k + 2 <= kme) {
        prefetch_l2(&rom(i, k + 2, j)); prefetch_l2(&p(i, k + 2, j)); prefetch_l2(&ph(i, k + 2, j));
        prefetch_l2(&alt(i, k + 2, j)); prefetch_l2(&al(i, k + 2, j)); prefetch_l2(&pb(i, k + 2, j));
        prefetch_l2(&php(i, k + 2, j)); prefetch_l2(&cqv(i, k + 2, j)); prefetch_l2(&rw(i, k + 2, j));
        prefetch_l2(&u(i, k + 2, j)); prefetch_l2(&tend(i, k + 2, j));
      }
      const LevelIn q = load_in(k);
      float t = q.t;
      t = t - mrdy * (FY[(ty + 1) * TX + tx] - FY[ty * TX + tx]);
      t = t - mrdx * (FX[ty * (TX + 1) + tx + 1] - FX[ty * (TX + 1) + tx]);
      {
        const int kk = k + 1;
        float vf_hi;
        if (kk == kts || kk == kte) vf_hi = 0.f;
        else if (kk == kts + 1 || kk == ktf)
          vf_hi = 0.5f * q.romsum * (fzm(kk) * vp1 + fzp(kk) * v0);
        else {
          const float vel = 0.5f * q.romsum;
          vf_hi = vel * flux3(vm1, v0, vp1, vp2, -vel);
        }
        t = t - ratio * rdzw(k) * (vf_hi - vf_lo);
        vf_lo = vf_hi;
      }
      if (FL & TF_PG) {
        const int kk = k + 1;
        float dpn_hi;
        if (kk == kde) {
          if (m.cf.top_lid)
            dpn_hi = .5f * (m.cfn * (p(i, kde - 1, j - 1) + p(i, kde - 1, j)) +
                            m.cfn1 * (p(i, kde - 2, j - 1) + p(i, kde - 2, j)));
          else dpn_hi = 0.f;
        } else {
          dpn_hi = .5f * (fzm(kk) * (q.p_l1 + q.p_r1) + fzp(kk) * (p_l + p_r));
        }
        float dpy = pgA * (c1h(k) * muv_c + c2h(k)) *
                    ((q.ph_r1 - q.ph_l1 + ph_r - ph_l) + q.altsum * (p_r - p_l) + q.alsum * q.pbd);
        dpy = dpy + pgB * q.phpd * (rdzw(k) * (dpn_hi - dpn_lo) - .5f * ((c1h(k) * mu_l) + (c1h(k) * mu_r)));
        t = t - q.cq * dpy;
        dpn_lo = dpn_hi;
        p_l = q.p_l1; p_r = q.p_r1; ph_l = q.ph_l1; ph_r = q.ph_r1;
      }
      if (FL & (TF_COR | TF_CURV)) {
        const float rusum = RU[o] + RU[o + 1] + RU[o - HALO_W] + RU[o - HALO_W + 1];
        const float rwsum = q.rw_l1 + rw_l + q.rw_r1 + rw_r;
        if (FL & TF_COR) t = t - corA * rusum + corB * rwsum;
        if (FL & TF_CURV) {
          const float vx_r = 0.5f * q.cs_r * dvx_r * rdy - 0.5f * (v0 + V[o + HALO_W]) * duy_r * rdx;
          const float vx_l = 0.5f * q.cs_l * dvx_l * rdy - 0.5f * (V[o - HALO_W] + v0) * duy_l * rdx;
          t = t - 0.5f * (vx_r + vx_l) * 0.25f * rusum - ratio * v0 * RERADIUS * 0.25f * rwsum;
        }
      }
      rw_l = q.rw_l1; rw_r = q.rw_r1;
      tend(i, k, j) = t;
      vm1 = v0; v0 = vp1; vp1 = vp2; vp2 = q.f3;
    }
    if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
  }
  if ((FL & TF_ZERO) && acc && blockIdx.y == gridDim.y - 1)
    for (int k = ktf + 1; k <= kte; ++k) tend(i, k, j) = 0.f;
}

// ---------------------------------------------------------------- rw_tend
// advect_w (module_advect_em.F:4364-6064), pg_buoy_w, coriolis and curvature
// (module_big_step_utilities_em.F) on the w levels.  pg_buoy_w overwrites
// cqw(k) with 1/(1+cqw(k)) after the k = kde point has read the original
// cqw(kde-1), so each column is walked in order by one thread (no level
// chunks).  The face velocities interpolate ru, rv between levels k and k-1
// (k-1 and k-2 at the top), so the ring keeps the two levels below the
// current one: after the barrier of level k the slot of level k-3 is free.
constexpr int W_RING = 6;
using HaloRingW = LevelRing<3, W_RING, HALO_W, HALO_H>;
constexpr size_t TENDW_SMEM = HaloRingW::SMEM + 2 * (FXN + FYN) * 4;

template <int FL, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_tend_w_col(TileLaunch L) {
  static_assert(FL & TF_ADV, "the staged form includes advection");
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i = tp.i0 + tx, j = tp.j0 + ty;
  const F3 tend = f3(m, WRFGPU_RW_TEND);
  const int kts = m.kts, kte = m.kte, kde = m.kde;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(kte, kde - 1);
  const bool inside = i <= m.ite && j <= m.jte;
  const bool acc = inside && i <= itf && j <= jtf;
  if ((FL & TF_ZERO) && inside && !acc)
    for (int k = kts; k <= kte; ++k) tend(i, k, j) = 0.f;
  if (!(tp.i0 <= itf && tp.j0 <= jtf)) return;  // block-uniform
  // next to an open boundary rw_tend has been formed by the edge-strip
  // kernel (k_tend.cu) from the cqw this kernel overwrites: keep it
  const bool keep = !((m.cf.open_xs || m.cf.open_ys) && in_open_strip(m, i, j, STRIP_W_TEND));
  const F3 w = f3(m, WRFGPU_W_2), rom = f3(m, WRFGPU_WW), p = f3(m, WRFGPU_P), cqw = f3(m, WRFGPU_CQW);
  const F3 u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2);
  const F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzu = f1(m, WRFGPU_RDN), rdnw = f1(m, WRFGPU_RDNW),
           c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F);
  const float rdx = m.rdx, rdy = m.rdy;
  HaloRingW ring;
  ring.init(smem, kts);
  float* FXb = (float*)(smem + HaloRingW::SMEM);
  float* FYb = FXb + 2 * FXN;
  const CUtensorMap* maps[3] = {tmap_of(m, WRFGPU_W_2, BOX_HALO), tmap_of(m, WRFGPU_RU, BOX_HALO),
                                tmap_of(m, WRFGPU_RV, BOX_HALO)};
  const int x0 = tp.i0 - TMA_HALO - m.ims, z0 = tp.j0 - TMA_HALO - m.jms;
  if (tid == 0) {
    ring.init_barriers();
    mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int d = 0; d < W_RING - 3 && kts + d <= kte; ++d) ring.issue(kts + d, maps, x0, z0, m.kms);
  auto vf = [&](int kk) -> float {
    if (kk == kts + 1 || kk == ktf + 1) return 0.25f * (rom(i, kk, j) + rom(i, kk - 1, j)) * (w(i, kk, j) + w(i, kk - 1, j));
    float vel = 0.5f * (rom(i, kk, j) + rom(i, kk - 1, j));
    return vel * flux3(w(i, kk - 2, j), w(i, kk - 1, j), w(i, kk, j), w(i, kk + 1, j), -vel);
  };
  // column constants, formed in the order of the per-level expressions
  float mrdy = 0.f, mrdx = 0.f, rmg = 0.f, ratio = 0.f, e_c = 0.f, cosa05 = 0.f, rsina05 = 0.f, ratio05 = 0.f;
  float muf_c = 0.f, mub_c = 0.f, cqw_top = 0.f, vf_lo = 0.f, mut_w = 0.f;
  const bool wdamp = m.cf.w_damping == 1;
  if (acc) {
    if (wdamp) mut_w = f2(m, WRFGPU_MUT)(i, j);
    const F2 msftx = f2(m, WRFGPU_MSFTX), msfty = f2(m, WRFGPU_MSFTY);
    mrdy = msftx(i, j) * rdy; mrdx = msftx(i, j) * rdx;
    rmg = (1.f / msfty(i, j)) * G;
    ratio = msftx(i, j) / msfty(i, j);
    if (FL & TF_COR) {
      e_c = f2(m, WRFGPU_E)(i, j);
      cosa05 = f2(m, WRFGPU_COSA)(i, j) * 0.5f;
      rsina05 = ratio * f2(m, WRFGPU_SINA)(i, j) * 0.5f;
    }
    ratio05 = ratio * 0.5f;
    if (FL & TF_PG) { muf_c = f2(m, WRFGPU_MU_2)(i, j); mub_c = f2(m, WRFGPU_MUB)(i, j); }
    cqw_top = cqw(i, kde - 1, j);  // read before the k = kde-1 overwrite below
    // the vertical flux of face k+1 is the lower face of level k+1
    vf_lo = kts + 1 <= ktf + 1 ? vf(kts + 1) : 0.f;
  }
  // levels k-1 (and k-2) of the mass fluxes at the own point and its +i / +j
  // neighbours, and of u, v, p, carried down the column; w(k-1 .. k+1) and
  // omega(k) of the own column for the vertical flux of face k+1
  float ru0m = 0.f, ru1m = 0.f, rv0m = 0.f, rv1m = 0.f;
  float u0m = 0.f, u1m = 0.f, v0m = 0.f, v1m = 0.f, pkm = 0.f;
  float wkm1 = 0.f, wk0 = 0.f, wkp1 = 0.f, romk = 0.f;
  const int kme = m.kme;
  if (acc) {
    wk0 = w(i, kts, j);
    wkp1 = kts + 1 <= kme ? w(i, kts + 1, j) : 0.f;
    romk = rom(i, kts, j);
  }
  const int o = (ty + TMA_HALO) * HALO_W + tx + TMA_HALO;
  bool ok = true;
  for (int k = kts; k <= kte; ++k) {
    // the level's global inputs, loaded together before the face work and
    // the level barrier so that their latency overlaps them
    float u0 = 0.f, u1 = 0.f, v0 = 0.f, v1 = 0.f, pk = 0.f, cqk = 0.f, romk1 = 0.f, wk2 = 0.f, t = 0.f;
    if (acc) {
      if (FL & TF_CURV) { u0 = u(i, k, j); u1 = u(i + 1, k, j); v0 = v(i, k, j); v1 = v(i, k, j + 1); }
      if (FL & TF_PG) {
        pk = p(i, k, j);
        if (k != kde && k >= 2) cqk = cqw(i, k, j);
      }
      romk1 = k + 1 <= kme ? rom(i, k + 1, j) : 0.f;
      wk2 = k + 2 <= kme ? w(i, k + 2, j) : 0.f;
      t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
    }
    ok = ring.wait(k) && ok;
    const float* Wk = ring.plane(k, 0);
    const float* RUk = ring.plane(k, 1);
    const float* RVk = ring.plane(k, 2);
    float* FX = FXb + (k & 1) * FXN;
    float* FY = FYb + (k & 1) * FYN;
    const bool adv = k >= kts + 1 && k <= ktf + 1;  // block-uniform
    if (adv) {
      const float* RUm = ring.plane(k - 1, 1);
      const float* RVm = ring.plane(k - 1, 2);
      if (k <= ktf) {
        const float a = fzm(k), b = fzp(k);
        tile_faces(Wk, FX, FY, [&](int q) { return a * RUk[q] + b * RUm[q]; },
                   [&](int q) { return a * RVk[q] + b * RVm[q]; }, tx, ty);
      } else {
        const float* RUmm = ring.plane(k - 2, 1);
        const float* RVmm = ring.plane(k - 2, 2);
        const float a = fzm(k - 1), b = fzp(k - 1);
        tile_faces(Wk, FX, FY, [&](int q) { return (2.f - a) * RUm[q] - b * RUmm[q]; },
                   [&](int q) { return (2.f - a) * RVm[q] - b * RVmm[q]; }, tx, ty);
      }
    }
    __syncthreads();
    if (tid == 0 && k - 3 + W_RING <= kte) ring.issue(k - 3 + W_RING, maps, x0, z0, m.kms);
    if (!acc) continue;
    const float ru0 = RUk[o], ru1 = RUk[o + 1], rv0 = RVk[o], rv1 = RVk[o + HALO_W];
    if (adv) {
      t = t - mrdy * (FY[(ty + 1) * TX + tx] - FY[ty * TX + tx]);
      t = t - mrdx * (FX[ty * (TX + 1) + tx + 1] - FX[ty * (TX + 1) + tx]);
      if (k <= ktf) {
        // vf(k + 1) from the carried window (the same operands and order)
        float vf_hi;
        if (k + 1 == kts + 1 || k + 1 == ktf + 1) vf_hi = 0.25f * (romk1 + romk) * (wkp1 + wk0);
        else {
          const float vel = 0.5f * (romk1 + romk);
          vf_hi = vel * flux3(wkm1, wk0, wkp1, wk2, -vel);
        }
        t = t - rdzu(k) * (vf_hi - vf_lo);
        vf_lo = vf_hi;
      } else {
        t = t + 2.f * rdzu(k - 1) * (vf_lo);
      }
    }
    if (FL & TF_PG) {
      if (k == kde) {
        float cq1 = 1.f / (1.f + cqw_top);
        float cq2 = cqw_top * cq1;
        t = t + rmg * (cq1 * 2.f * rdnw(k - 1) * (-pkm) - (c1f(k) * muf_c) - cq2 * (c1f(k) * mub_c + c2f(k)));
      } else if (k >= 2) {
        float cq1 = 1.f / (1.f + cqk);
        float cq2 = cqk * cq1;
        cqw(i, k, j) = cq1;
        t = t + rmg * (cq1 * rdzu(k) * (pk - pkm) - (c1f(k) * muf_c) - cq2 * (c1f(k) * mub_c + c2f(k)));
      }
    }
    // w_damp with w_damping = 1 (module_big_step_utilities_em.F:2687-2691),
    // after pg_buoy_w and before coriolis as rk_tendency calls them
    // (module_em.F:729-745); activation at w_beta (zadvect_implicit = 0)
    if (FL == TF_ALL && wdamp && k >= 2 && k <= kde - 1) {
      const float vert_cfl = fabsf(romk / (c1f(k) * mut_w + c2f(k)) * rdnw(k) * m.dt);
      if (vert_cfl > W_BETA)
        t = t - sgn1(Wk[o]) * W_ALPHA * (vert_cfl - m.cf.w_crit_cfl) * (c1f(k) * mut_w + c2f(k));
    }
    if (k >= kts + 1 && k <= ktf) {
      if (FL & TF_COR) {
        t = t + e_c * (cosa05 * (fzm(k) * (ru0 + ru1) + fzp(k) * (ru0m + ru1m)) -
                       rsina05 * (fzm(k) * (rv0 + rv1) + fzp(k) * (rv0m + rv1m)));
      }
    }
    if (k >= max(2, kts) && k <= ktf) {
      if (FL & TF_CURV) {
        t = t + RERADIUS * (0.5f * (fzm(k) * (ru0 + ru1) + fzp(k) * (ru0m + ru1m)) *
                                0.5f * (fzm(k) * (u0 + u1) + fzp(k) * (u0m + u1m)) +
                            ratio05 * (fzm(k) * (rv0 + rv1) + fzp(k) * (rv0m + rv1m)) *
                                0.5f * (fzm(k) * (v0 + v1) + fzp(k) * (v0m + v1m)));
      }
    }
    if (keep) tend(i, k, j) = t;
    ru0m = ru0; ru1m = ru1; rv0m = rv0; rv1m = rv1;
    u0m = u0; u1m = u1; v0m = v0; v1m = v1;
    pkm = pk;
    wkm1 = wk0; wk0 = wkp1; wkp1 = wk2; romk = romk1;
  }
  if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
}

// ---------------------------------------------------------------- t_tend
// advect_scalar of theta (module_advect_em.F:3394-3650, :4306-4333) plus the
// zero_tend of the *_save arrays at the points small_step_prep leaves alone
// (module_em.F:395-428); the vertical flux and the own-column window of
// theta carry down the column.
template <int FL, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) k_tend_t_col(TileLaunch L) {
  static_assert(FL & TF_ADV, "the staged form includes advection");
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i = tp.i0 + tx, j = tp.j0 + ty;
  const F3 tend = f3(m, WRFGPU_T_TEND);
  const int kts = m.kts, kte = m.kte, kme = m.kme;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(kte, m.kde - 1);
  const bool inside = i <= m.ite && j <= m.jte;
  if ((FL & TF_ZERO) && inside) {
    const bool ie = i == m.ide, je = j == m.jde;
    const F3 us = f3(m, WRFGPU_U_SAVE), vs = f3(m, WRFGPU_V_SAVE), ts = f3(m, WRFGPU_T_SAVE),
             ws = f3(m, WRFGPU_W_SAVE), phs = f3(m, WRFGPU_PH_SAVE);
    for (int k = kts; k <= kte; ++k) {
      const bool kt = k == m.kde;
      if (kt || je) us(i, k, j) = 0.f;
      if (kt || ie) vs(i, k, j) = 0.f;
      if (kt || ie || je) ts(i, k, j) = 0.f;
      if (ie || je) { ws(i, k, j) = 0.f; phs(i, k, j) = 0.f; }
    }
    if (ie || je) f2(m, WRFGPU_MU_SAVE)(i, j) = 0.f;
  }
  const bool acc = inside && i <= itf && j <= jtf;
  if ((FL & TF_ZERO) && inside && !acc)
    for (int k = kts; k <= kte; ++k) tend(i, k, j) = 0.f;
  if (tp.i0 <= itf && tp.j0 <= jtf) {  // block-uniform
    const F3 fld = f3(m, WRFGPU_T_2), rom = f3(m, WRFGPU_WW);
    const F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzw = f1(m, WRFGPU_RDNW);
    HaloRing ring;
    ring.init(smem, kts);
    float* FXb = (float*)(smem + HaloRing::SMEM);
    float* FYb = FXb + 2 * FXN;
    const CUtensorMap* maps[3] = {tmap_of(m, WRFGPU_T_2, BOX_HALO), tmap_of(m, WRFGPU_RU, BOX_HALO),
                                  tmap_of(m, WRFGPU_RV, BOX_HALO)};
    const int x0 = tp.i0 - TMA_HALO - m.ims, z0 = tp.j0 - TMA_HALO - m.jms;
    if (tid == 0) {
      ring.init_barriers();
      mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int d = 0; d < TEND_RING - 1 && kts + d <= ktf; ++d) ring.issue(kts + d, maps, x0, z0, m.kms);
    float mrdy = 0.f, mrdx = 0.f, fm1 = 0.f, f0 = 0.f, fp1 = 0.f, fp2 = 0.f;
    if (acc) {
      const float msftx_c = f2(m, WRFGPU_MSFTX)(i, j);
      mrdy = msftx_c * m.rdy; mrdx = msftx_c * m.rdx;
      f0 = fld(i, kts, j); fp1 = fld(i, kts + 1, j); fp2 = (kts + 2 <= kme) ? fld(i, kts + 2, j) : 0.f;
    }
    float vf_lo = 0.f;  // vf(kts) = 0
    bool ok = true;
    for (int k = kts; k <= ktf; ++k) {
      // the level's own-column loads, issued before the face work and the
      // barrier so that their latency overlaps them
      float fp3 = 0.f, romk1 = 0.f;
      if (acc) {
        fp3 = (k + 3 <= kme) ? fld(i, k + 3, j) : 0.f;
        romk1 = (k + 1 == kts || k + 1 == kte) ? 0.f : rom(i, k + 1, j);
      }
      ok = ring.wait(k) && ok;
      const float* T = ring.plane(k, 0);
      const float* RU = ring.plane(k, 1);
      const float* RV = ring.plane(k, 2);
      float* FX = FXb + (k & 1) * FXN;
      float* FY = FYb + (k & 1) * FYN;
      tile_faces(T, FX, FY, [&](int q) { return RU[q]; }, [&](int q) { return RV[q]; }, tx, ty);
      __syncthreads();
      if (tid == 0 && k + TEND_RING - 1 <= ktf) ring.issue(k + TEND_RING - 1, maps, x0, z0, m.kms);
      if (!acc) continue;
      if (k + 2 <= kme) { prefetch_l2(&rom(i, k + 2, j)); prefetch_l2(&tend(i, k + 2, j)); }
      float t = (FL & TF_ZERO) ? 0.f : tend(i, k, j);
      t = t - mrdy * (FY[(ty + 1) * TX + tx] - FY[ty * TX + tx]);
      t = t - mrdx * (FX[ty * (TX + 1) + tx + 1] - FX[ty * (TX + 1) + tx]);
      const int kk = k + 1;
      float vf_hi;
      if (kk == kts || kk == kte) vf_hi = 0.f;
      else if (kk == kts + 1 || kk == ktf) vf_hi = romk1 * (fzm(kk) * fp1 + fzp(kk) * f0);
      else {
        const float vel = romk1;
        vf_hi = vel * flux3(fm1, f0, fp1, fp2, -vel);
      }
      t = t - rdzw(k) * (vf_hi - vf_lo);
      vf_lo = vf_hi;
      tend(i, k, j) = t;
      fm1 = f0; f0 = fp1; fp1 = fp2; fp2 = fp3;
    }
    if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
  }
  if ((FL & TF_ZERO) && acc)
    for (int k = ktf + 1; k <= kte; ++k) tend(i, k, j) = 0.f;
}

// ---------------------------------------------------------------- ph_tend
// rhs_ph (module_big_step_utilities_em.F:1365-2178, 5th/6th order branch):
// the vertical term's wdwn(k+1) is wdwn(k) one level up, u and v of levels
// k, k-1 carry down, the column's map factors and mass terms are read once.
constexpr int PH_RING = 4;
using PhRing = LevelRing<2, PH_RING, HALO_W, HALO_H>;  // ph, phb halo planes

template <int FL>
__global__ void __launch_bounds__(TX* TY, 4) k_tend_ph_col(TileLaunch L) {
  static_assert((FL & TF_ADV) && (FL & TF_ZERO), "the staged form starts from zero and advects");
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, false, true);
  const Mem& m = block_member(L.mem, tp.m);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i = tp.i0 + tx, j = tp.j0 + ty;
  const F3 tend = f3(m, WRFGPU_PH_TEND);
  const int kts = m.kts, kte = m.kte, kde = m.kde;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1);
  const bool inside = i <= m.ite && j <= m.jte;
  const bool acc = inside && i <= itf && j <= jtf;
  if (inside && !acc)
    for (int k = kts; k <= kte; ++k) tend(i, k, j) = 0.f;
  if (!(tp.i0 <= itf && tp.j0 <= jtf)) return;  // block-uniform
  if (acc)
    for (int k = kts; k <= min(kte, 1); ++k) tend(i, k, j) = 0.f;
  const int ks = max(kts, 2);
  if (ks > kte) return;
  const F3 u = f3(m, WRFGPU_U_2), v = f3(m, WRFGPU_V_2), ww = f3(m, WRFGPU_WW), ph = f3(m, WRFGPU_PH_2),
           phb = f3(m, WRFGPU_PHB), w = f3(m, WRFGPU_W_2);
  const F1 c1f = f1(m, WRFGPU_C1F), c2f = f1(m, WRFGPU_C2F), fnm = f1(m, WRFGPU_FNM), fnp = f1(m, WRFGPU_FNP),
           rdnw = f1(m, WRFGPU_RDNW);
  PhRing ring;
  ring.init(smem, ks);
  const CUtensorMap* maps[2] = {tmap_of(m, WRFGPU_PH_2, BOX_HALO), tmap_of(m, WRFGPU_PHB, BOX_HALO)};
  const int x0 = tp.i0 - TMA_HALO - m.ims, z0 = tp.j0 - TMA_HALO - m.jms;
  if (tid == 0) {
    ring.init_barriers();
    mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int d = 0; d < PH_RING - 1 && ks + d <= kte; ++d) ring.issue(ks + d, maps, x0, z0, m.kms);
  // column constants
  float mut_c = 0.f, msfty_c = 0.f, muv1 = 0.f, muv0 = 0.f, muu1 = 0.f, muu0 = 0.f, mvy1 = 0.f, mvy0 = 0.f;
  float mux1 = 0.f, mux0 = 0.f, cy4 = 0.f, cx4 = 0.f, cy2 = 0.f, cx2 = 0.f;
  const float cfn = m.cfn, cfn1 = m.cfn1;
  const bool adv2 = m.cf.phi_adv_z == 2;
  auto wdwn = [&](int kk) {
    if (adv2) return rdnw(kk - 1) * (ph(i, kk, j) - ph(i, kk - 1, j) + phb(i, kk, j) - phb(i, kk - 1, j));
    return .5f * (ww(i, kk, j) + ww(i, kk - 1, j)) * rdnw(kk - 1) * (ph(i, kk, j) - ph(i, kk - 1, j) + phb(i, kk, j) - phb(i, kk - 1, j));
  };
  // carried: wdwn(k), ph, phb and ww of level k, and u, v of levels k-1,
  // k-2 at (i, i+1) / (j, j+1)
  float u0m = 0.f, u1m = 0.f, v0m = 0.f, v1m = 0.f, u0mm = 0.f, u1mm = 0.f, v0mm = 0.f, v1mm = 0.f, wd_lo = 0.f;
  float ph_c = 0.f, phb_c = 0.f, ww_c = 0.f;
  if (acc) {
    mut_c = f2(m, WRFGPU_MUT)(i, j); msfty_c = f2(m, WRFGPU_MSFTY)(i, j);
    muv1 = f2(m, WRFGPU_MUV)(i, j + 1); muv0 = f2(m, WRFGPU_MUV)(i, j);
    muu1 = f2(m, WRFGPU_MUU)(i + 1, j); muu0 = f2(m, WRFGPU_MUU)(i, j);
    mvy1 = f2(m, WRFGPU_MSFVY)(i, j + 1); mvy0 = f2(m, WRFGPU_MSFVY)(i, j);
    mux1 = f2(m, WRFGPU_MSFUX)(i + 1, j); mux0 = f2(m, WRFGPU_MSFUX)(i, j);
    cy4 = 0.25f * m.rdy / msfty_c; cx4 = 0.25f * m.rdx / msfty_c;
    cy2 = 0.5f * m.rdy / msfty_c; cx2 = 0.5f * m.rdx / msfty_c;
    u0m = u(i, 1, j); u1m = u(i + 1, 1, j); v0m = v(i, 1, j); v1m = v(i, 1, j + 1);  // level k-1 = 1
    wd_lo = (2 <= kte - 1) ? wdwn(2) : 0.f;  // wdwn(k) at k = 2
    ph_c = ph(i, ks, j); phb_c = phb(i, ks, j); ww_c = ww(i, ks, j);
  }
  const int o = (ty + TMA_HALO) * HALO_W + tx + TMA_HALO;
  bool ok = true;
  for (int k = ks; k <= kte; ++k) {
    // the level's global inputs, loaded together before the barrier so that
    // their latency overlaps it
    float ph_n = 0.f, phb_n = 0.f, ww_n = 0.f, u0 = 0.f, u1 = 0.f, v0 = 0.f, v1 = 0.f, wk = 0.f;
    if (acc) {
      if (k <= kte - 1) {
        ph_n = ph(i, k + 1, j); phb_n = phb(i, k + 1, j); ww_n = ww(i, k + 1, j);
        u0 = u(i, k, j); u1 = u(i + 1, k, j); v0 = v(i, k, j); v1 = v(i, k, j + 1);
      }
      if (m.cf.non_hydrostatic) wk = w(i, k, j);
    }
    __syncthreads();  // every thread is done with level k-1's slot
    if (tid == 0 && k + PH_RING - 1 <= kte) ring.issue(k + PH_RING - 1, maps, x0, z0, m.kms);
    ok = ring.wait(k) && ok;
    if (!acc) continue;
    const float* PH = ring.plane(k, 0);
    const float* PHB = ring.plane(k, 1);
    if (k + 2 <= kte) {
      prefetch_l2(&ph(i, k + 2, j)); prefetch_l2(&phb(i, k + 2, j)); prefetch_l2(&u(i, k + 2, j));
      prefetch_l2(&v(i, k + 2, j)); prefetch_l2(&ww(i, k + 2, j)); prefetch_l2(&w(i, k + 2, j));
    }
    float t = 0.f;
    // vertical advection of ph (:1396-1428): wdwn(k + 1) from the carried
    // level-k values (the same operands and order)
    if (k <= kte - 1) {
      const float wd_hi = adv2 ? rdnw(k) * (ph_n - ph_c + phb_n - phb_c)
                               : .5f * (ww_n + ww_c) * rdnw(k) * (ph_n - ph_c + phb_n - phb_c);
      if (adv2) t = t - ww_c * (fnm(k) * wd_hi + fnp(k) * wd_lo);
      else t = t - (fnm(k) * wd_hi + fnp(k) * wd_lo);
      wd_lo = wd_hi;
    }
    // "gw" term (:1432-1446)
    if (m.cf.non_hydrostatic) {
      if (k == kde) t = 0.f;
      t = t + (c1f(k) * mut_c + c2f(k)) * G * wk / msfty_c;
    }
    auto S = [&](int d) {  // 6th-order centred difference of ph + phb, stride d in the halo plane
      return 45.f * (PH[o + d] - PH[o - d]) - 9.f * (PH[o + 2 * d] - PH[o - 2 * d]) + (PH[o + 3 * d] - PH[o - 3 * d]) +
             45.f * (PHB[o + d] - PHB[o - d]) - 9.f * (PHB[o + 2 * d] - PHB[o - 2 * d]) +
             (PHB[o + 3 * d] - PHB[o - 3 * d]);
    };
    if (k <= kte - 1) {
      t = t - cy4 * (((c1f(k) * muv1 + c2f(k)) * (v1 + v1m) * mvy1 + (c1f(k) * muv0 + c2f(k)) * (v0 + v0m) * mvy0) *
                     (1.f / 60.f) * S(HALO_W));
      t = t - cx4 * (((c1f(k) * muu1 + c2f(k)) * (u1 + u1m) * mux1 + (c1f(k) * muu0 + c2f(k)) * (u0 + u0m) * mux0) *
                     (1.f / 60.f) * S(1));
    } else {
      t = t - cy2 * (((c1f(k) * muv1 + c2f(k)) * (cfn * v1m + cfn1 * v1mm) * mvy1 +
                      (c1f(k) * muv0 + c2f(k)) * (cfn * v0m + cfn1 * v0mm) * mvy0) *
                     (1.f / 60.f) * S(HALO_W));
      t = t - cx2 * (((c1f(k) * muu1 + c2f(k)) * (cfn * u1m + cfn1 * u1mm) * mux1 +
                      (c1f(k) * muu0 + c2f(k)) * (cfn * u0m + cfn1 * u0mm) * mux0) *
                     (1.f / 60.f) * S(1));
    }
    tend(i, k, j) = t;
    u0mm = u0m; u1mm = u1m; v0mm = v0m; v1mm = v1m;
    u0m = u0; u1m = u1; v0m = v0; v1m = v1;
    ph_c = ph_n; phb_c = phb_n; ww_c = ww_n;
  }
  if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
}

// variant parameter: 10 x blocks per SM + level chunks
void launch_tend_u_col(const TileLaunch& L, int nb, int flags, cudaStream_t s, int var) {
  const int p = TUNE_PARAM[TU_TENDU][var];
  const dim3 grid(nb, p % 10);
  if (flags != TF_ALL) return;
  if (p / 10 == 4) k_tend_u_col<TF_ALL, 4><<<grid, dim3(TX, TY), TEND_SMEM, s>>>(L);
  else k_tend_u_col<TF_ALL, 3><<<grid, dim3(TX, TY), TEND_SMEM, s>>>(L);
}
void launch_tend_v_col(const TileLaunch& L, int nb, int flags, cudaStream_t s, int var) {
  const int p = TUNE_PARAM[TU_TENDV][var];
  const dim3 grid(nb, p % 10);
  if (flags != TF_ALL) return;
  if (p / 10 == 4) k_tend_v_col<TF_ALL, 4><<<grid, dim3(TX, TY), TEND_SMEM, s>>>(L);
  else k_tend_v_col<TF_ALL, 3><<<grid, dim3(TX, TY), TEND_SMEM, s>>>(L);
}
void launch_tend_w_col(const TileLaunch& L, int nb, int var, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_tend_w_col<TF_ALL, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TENDW_SMEM);
    cudaFuncSetAttribute(k_tend_w_col<TF_ALL, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TENDW_SMEM);
    cudaFuncSetAttribute(k_tend_w_col<TF_ALL, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TENDW_SMEM);
    attr = true;
  }
  const int minb = TUNE_PARAM[TU_TENDW][var];
  if (minb == 2) k_tend_w_col<TF_ALL, 2><<<nb, dim3(TX, TY), TENDW_SMEM, s>>>(L);
  else if (minb == 3) k_tend_w_col<TF_ALL, 3><<<nb, dim3(TX, TY), TENDW_SMEM, s>>>(L);
  else k_tend_w_col<TF_ALL, 4><<<nb, dim3(TX, TY), TENDW_SMEM, s>>>(L);
}
void launch_tend_t_col(const TileLaunch& L, int nb, int flags, cudaStream_t s) {
  if (flags == (TF_ZERO | TF_ADV)) k_tend_t_col<TF_ZERO | TF_ADV, 4><<<nb, dim3(TX, TY), TEND_SMEM, s>>>(L);
}
void launch_tend_ph_col(const TileLaunch& L, int nb, int flags, cudaStream_t s) {
  if (flags == (TF_ZERO | TF_ADV)) k_tend_ph_col<TF_ZERO | TF_ADV><<<nb, dim3(TX, TY), PhRing::SMEM, s>>>(L);
}

}  // namespace wrfgpu
