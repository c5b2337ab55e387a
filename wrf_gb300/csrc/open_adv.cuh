// Flux-form advection next to open lateral boundaries (open_xs/xe/ys/ye,
// the em_quarter_ss namelist) as point functions: the order of each
// horizontal face flux (the reference's degrade_xs/xe/ys/ye,
// dyn_em/module_advect_em.F:500-516), the radiation terms of the boundary
// rows, and the positive-definite limiter's open-boundary ranges.  With
// periodic or symmetric boundaries every face takes the full stencil and the
// functions reduce to the interior formulas, bit for bit.  Used by the
// routine-level kernels and by the edge-strip recomputation of the large
// step (k_tend.cu, k_scalar.cu).
#pragma once
#include "common.cuh"

namespace wrfgpu {

// Order of the flux at face f (5: the full stencil, 3: third order, 2:
// second order) for a direction whose start / end boundary is open (os /
// oe), lo = ids or jds, hi = ide or jde.
// Faces between mass points (advect_scalar, advect_w, advect_scalar_pd, the
// y faces of advect_u and the x faces of advect_v): second order at lo+1 and
// hi-1, third order at lo+2 and hi-2 (module_advect_em.F:3554-3632).
__device__ __forceinline__ int open_order_mass(int f, bool os, bool oe, int lo, int hi) {
  if (os) {
    if (f == lo + 1) return 2;
    if (f == lo + 2) return 3;
  }
  if (oe) {
    if (f == hi - 1) return 2;
    if (f == hi - 2) return 3;
  }
  return 5;
}
// Faces between staggered points (the x faces of advect_u, the y faces of
// advect_v): second order at lo+1 and hi, third order at lo+2 and hi-1
// (module_advect_em.F:663-730, :2038-2075).
__device__ __forceinline__ int open_order_stag(int f, bool os, bool oe, int lo, int hi) {
  if (os) {
    if (f == lo + 1) return 2;
    if (f == lo + 2) return 3;
  }
  if (oe) {
    if (f == hi) return 2;
    if (f == hi - 1) return 3;
  }
  return 5;
}

// Radiation terms of a mass-point scalar at the open boundary rows
// (module_advect_em.F:4104-4175 advect_scalar, :7254-7328 advect_scalar_pd;
// no map factors), in the reference's order xs, xe, ys, ye; f is the field,
// fo the field the upwind difference is taken of.
__device__ __forceinline__ float scalar_radiation(const Mem& m, const F3& f, const F3& fo, const F3& ru, const F3& rv,
                                                  float t, int i, int j, int k) {
  if (m.cf.open_xs && i == m.ids) {
    const float ub = fminf_f(0.5f * (ru(i, k, j) + ru(i + 1, k, j)), 0.f);
    t = t - m.rdx * (ub * (fo(i + 1, k, j) - fo(i, k, j)) + f(i, k, j) * (ru(i + 1, k, j) - ru(i, k, j)));
  }
  if (m.cf.open_xe && i == m.ide - 1) {
    const float ub = fmaxf_f(0.5f * (ru(i, k, j) + ru(i + 1, k, j)), 0.f);
    t = t - m.rdx * (ub * (fo(i, k, j) - fo(i - 1, k, j)) + f(i, k, j) * (ru(i + 1, k, j) - ru(i, k, j)));
  }
  if (m.cf.open_ys && j == m.jds) {
    const float vb = fminf_f(0.5f * (rv(i, k, j) + rv(i, k, j + 1)), 0.f);
    t = t - m.rdy * (vb * (fo(i, k, j + 1) - fo(i, k, j)) + f(i, k, j) * (rv(i, k, j + 1) - rv(i, k, j)));
  }
  if (m.cf.open_ye && j == m.jde - 1) {
    const float vb = fmaxf_f(0.5f * (rv(i, k, j) + rv(i, k, j + 1)), 0.f);
    t = t - m.rdy * (vb * (fo(i, k, j) - fo(i, k, j - 1)) + f(i, k, j) * (rv(i, k, j + 1) - rv(i, k, j)));
  }
  return t;
}

// advect_scalar (module_advect_em.F:3394-3650 5th-order horizontal, radiation
// :4104-4175, 3rd-order vertical :4306-4333) at mass point (i, k), k in
// kts..ktf: t minus the y, x, radiation and vertical terms in that order.
struct ScalarAdv {
  F3 f, fo, ru, rv, rom;
  F2 msftx;
  F1 fzm, fzp, rdzw;
};
__device__ __forceinline__ float adv_scalar_point(const Mem& m, const ScalarAdv& a, float t, int i, int j, int k) {
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const int ktf = min(m.kte, m.kde - 1);
  const F3& fld = a.f;
  auto fy = [&](int jj) -> float {
    const int o = open_order_mass(jj, oys, oye, m.jds, m.jde);
    const float vel = a.rv(i, k, jj);
    if (o == 5)
      return vel * flux5(fld(i, k, jj - 3), fld(i, k, jj - 2), fld(i, k, jj - 1), fld(i, k, jj), fld(i, k, jj + 1),
                         fld(i, k, jj + 2), vel);
    if (o == 2) return 0.5f * a.rv(i, k, jj) * (fld(i, k, jj) + fld(i, k, jj - 1));
    return vel * flux3(fld(i, k, jj - 2), fld(i, k, jj - 1), fld(i, k, jj), fld(i, k, jj + 1), vel);
  };
  if ((!oys || j >= m.jds + 1) && (!oye || j <= m.jde - 2)) t = t - a.msftx(i, j) * m.rdy * (fy(j + 1) - fy(j));
  auto fx = [&](int ii) -> float {
    const int o = open_order_mass(ii, oxs, oxe, m.ids, m.ide);
    const float vel = a.ru(ii, k, j);
    if (o == 5)
      return vel * flux5(fld(ii - 3, k, j), fld(ii - 2, k, j), fld(ii - 1, k, j), fld(ii, k, j), fld(ii + 1, k, j),
                         fld(ii + 2, k, j), vel);
    if (o == 2) return 0.5f * (a.ru(ii, k, j)) * (fld(ii, k, j) + fld(ii - 1, k, j));
    return vel * flux3(fld(ii - 2, k, j), fld(ii - 1, k, j), fld(ii, k, j), fld(ii + 1, k, j), vel);
  };
  if ((!oxs || i >= m.ids + 1) && (!oxe || i <= m.ide - 2)) t = t - a.msftx(i, j) * m.rdx * (fx(i + 1) - fx(i));
  t = scalar_radiation(m, fld, a.fo, a.ru, a.rv, t, i, j, k);
  auto vf = [&](int kk) -> float {
    if (kk == m.kts || kk == m.kte) return 0.f;
    if (kk == m.kts + 1 || kk == ktf) return a.rom(i, kk, j) * (a.fzm(kk) * fld(i, kk, j) + a.fzp(kk) * fld(i, kk - 1, j));
    const float vel = a.rom(i, kk, j);
    return vel * flux3(fld(i, kk - 2, j), fld(i, kk - 1, j), fld(i, kk, j), fld(i, kk + 1, j), -vel);
  };
  t = t - a.rdzw(k) * (vf(k + 1) - vf(k));
  return t;
}

// ------------------------------------------------------------ edge strips
// The points of a member with open boundaries whose large-step results the
// open branches change: within two points of an open edge for the
// tendencies and the 5th/3rd-order transport (STRIP_W_TEND), within three
// for the positive-definite transport, whose limiter factors couple
// neighbouring cells (STRIP_W_PD), and the limiter factors themselves one
// further, halo row / column included where the other direction is
// periodic (STRIP_W_PD + 1, h = 1).  A strip of width w: the x strips
// i in ids..ids+w-1 and ide-w..ide over rows jds-h..jde, then the y strips
// j in jds..jds+w-1 and jde-w..jde over the columns outside the x strips
// (ids-h..ide without open x); ids = jds = 1.
constexpr int STRIP_W_TEND = 3, STRIP_W_PD = 4;
__host__ __device__ inline int strip_cols(int ide, int jde, bool ox, bool oy, int w, int h) {
  const int nw = 2 * w + 1;
  int n = ox ? nw * (jde + h) : 0;
  if (oy) n += nw * (ox ? ide - nw : ide + h);
  return n;
}
__device__ __forceinline__ void strip_col(const Mem& m, int c, int w, int h, int* i, int* j) {
  const int nw = 2 * w + 1;
  const bool ox = m.cf.open_xs;
  if (ox) {
    const int nx = nw * (m.jde + h);
    if (c < nx) {
      const int a = c % nw;
      *j = 1 - h + c / nw;
      *i = a < w ? 1 + a : m.ide - w + (a - w);
      return;
    }
    c -= nx;
  }
  const int i0 = ox ? 1 + w : 1 - h, ni = ox ? m.ide - nw : m.ide + h;
  const int r = c / ni;
  *i = i0 + c % ni;
  *j = r < w ? 1 + r : m.jde - w + (r - w);
}
__device__ __forceinline__ bool in_open_strip(const Mem& m, int i, int j, int w) {
  return (m.cf.open_xs && (i <= m.ids + w - 1 || i >= m.ide - w)) ||
         (m.cf.open_ys && (j <= m.jds + w - 1 || j >= m.jde - w));
}
// Position of a thread of a strip launch: blocks of STRIP_THREADS over each
// member's strip columns x levels kms..kme.
struct StripPos {
  int m, i, j, k;
  bool valid;
};
__device__ __forceinline__ StripPos strip_pos(const StripLaunch& L) {
  StripPos sp;
  const int b = blockIdx.x;
  sp.m = find_member(L.block_start, L.nmem, b);
  const Mem& m = L.mem[sp.m];
  const int p = (b - __ldg(L.block_start + sp.m)) * STRIP_THREADS + (int)threadIdx.x;
  const int nc = strip_cols(m.ide, m.jde, m.cf.open_xs, m.cf.open_ys, L.w, L.h);
  const int nk = m.kme - m.kms + 1;
  sp.valid = nc > 0 && p < nc * nk;
  sp.i = sp.j = 0;
  sp.k = 0;
  if (sp.valid) {
    sp.k = m.kms + p / nc;
    strip_col(m, p % nc, L.w, L.h, &sp.i, &sp.j);
  }
  return sp;
}

// ------------------------------------------------------------ advect_scalar_pd
struct PDCtx {
  F3 f, fo, ru, rv, rom;
  F2 mut, mub, mu_old, msftx, msfty;
  F1 c1, c2, fzm, fzp, rdzw;
  float rdx, rdy, dt;
  int kts, ktf, kde;
  // the faces' Courant numbers and low-order flux factors formed once per
  // step by k_pd_courant (the same expressions, so the same bits), when set
  bool pre;
  F3 crx, cry, crz, lfx, lfy, lfz;
};
__device__ __forceinline__ PDCtx pd_ctx(const Mem& m, int species, float dt, bool pre = false) {
  PDCtx c{f3p(m, m.q[species]), f3p(m, m.qo[species]), f3(m, WRFGPU_RU_M), f3(m, WRFGPU_RV_M), f3(m, WRFGPU_WW_M),
          f2(m, WRFGPU_MUTS), f2(m, WRFGPU_MUB), f2(m, WRFGPU_MU_1), f2(m, WRFGPU_MSFTX), f2(m, WRFGPU_MSFTY),
          f1(m, WRFGPU_C1H), f1(m, WRFGPU_C2H), f1(m, WRFGPU_FNM), f1(m, WRFGPU_FNP), f1(m, WRFGPU_RDNW),
          m.rdx, m.rdy, dt, m.kts, min(m.kte, m.kde - 1), m.kde, false};
  if (pre && m.pdc[0]) {
    c.pre = true;
    c.crx = f3p(m, m.pdc[0]); c.cry = f3p(m, m.pdc[1]); c.crz = f3p(m, m.pdc[2]);
    c.lfx = f3p(m, m.pdc[3]); c.lfy = f3p(m, m.pdc[4]); c.lfz = f3p(m, m.pdc[5]);
  }
  return c;
}
// Face fluxes (module_advect_em.F:6505-6779): *hi = high-order minus upwind,
// *lo = upwind.  Next to an open start boundary in x the second-order face
// forms its Courant number as (ru / mu) dt / dx (:6681-6685); the other
// faces as ru dt / dx / mu.
__device__ __forceinline__ void pd_fx(const Mem& m, const PDCtx& c, int i, int k, int j, float* hi, float* lo) {
  const int o = open_order_mass(i, m.cf.open_xs, m.cf.open_xe, m.ids, m.ide);
  const bool quirk = o == 2 && m.cf.open_xs && i == m.ids + 1;
  float vel, cr, lf;
  if (c.pre && !quirk) {
    vel = c.ru(i, k, j);
    cr = c.crx(i, k, j);
    lf = c.lfx(i, k, j);
  } else {
    const float dx = 2.f / (c.msfty(i, j) + c.msfty(i - 1, j)) / c.rdx;
    const float mu = 0.5f * ((c.c1(k) * c.mut(i, j) + c.c2(k)) + (c.c1(k) * c.mut(i - 1, j) + c.c2(k)));
    if (quirk) {
      vel = c.ru(i, k, j) / mu;
      cr = vel * c.dt / dx;
    } else {
      vel = c.ru(i, k, j);
      cr = vel * c.dt / dx / mu;
    }
    lf = mu * (dx / c.dt);
  }
  const float l = lf * flux_upwind(c.fo(i - 1, k, j), c.fo(i, k, j), cr);
  float h;
  if (o == 5)
    h = vel * pflux5(c.f(i - 3, k, j), c.f(i - 2, k, j), c.f(i - 1, k, j), c.f(i, k, j), c.f(i + 1, k, j), c.f(i + 2, k, j), vel);
  else if (o == 3)
    h = vel * pflux3(c.f(i - 2, k, j), c.f(i - 1, k, j), c.f(i, k, j), c.f(i + 1, k, j), vel);
  else
    h = 0.5f * (c.ru(i, k, j)) * (c.f(i, k, j) + c.f(i - 1, k, j));
  *lo = l; *hi = h - l;
}
__device__ __forceinline__ void pd_fy(const Mem& m, const PDCtx& c, int i, int k, int j, float* hi, float* lo) {
  const int o = open_order_mass(j, m.cf.open_ys, m.cf.open_ye, m.jds, m.jde);
  const float vel = c.rv(i, k, j);
  float cr, lf;
  if (c.pre) {
    cr = c.cry(i, k, j);
    lf = c.lfy(i, k, j);
  } else {
    const float dy = 2.f / (c.msftx(i, j) + c.msftx(i, j - 1)) / c.rdy;
    const float mu = 0.5f * ((c.c1(k) * c.mut(i, j) + c.c2(k)) + (c.c1(k) * c.mut(i, j - 1) + c.c2(k)));
    cr = vel * c.dt / dy / mu;
    lf = mu * (dy / c.dt);
  }
  const float l = lf * flux_upwind(c.fo(i, k, j - 1), c.fo(i, k, j), cr);
  float h;
  if (o == 5)
    h = vel * pflux5(c.f(i, k, j - 3), c.f(i, k, j - 2), c.f(i, k, j - 1), c.f(i, k, j), c.f(i, k, j + 1), c.f(i, k, j + 2), vel);
  else if (o == 3)
    h = vel * pflux3(c.f(i, k, j - 2), c.f(i, k, j - 1), c.f(i, k, j), c.f(i, k, j + 1), vel);
  else
    h = 0.5f * c.rv(i, k, j) * (c.f(i, k, j) + c.f(i, k, j - 1));
  *lo = l; *hi = h - l;
}
__device__ __forceinline__ void pd_fz(const PDCtx& c, int i, int k, int j, float* hi, float* lo) {
  if (k == 1 || k == c.kde) { *hi = 0.f; *lo = 0.f; return; }
  const float vel = c.rom(i, k, j);
  float cr, lf;
  if (c.pre) {
    cr = c.crz(i, k, j);
    lf = c.lfz(i, k, j);
  } else {
    const float dz = 2.f / (c.rdzw(k) + c.rdzw(k - 1));
    const float mu = 0.5f * ((c.c1(k) * c.mut(i, j) + c.c2(k)) + (c.c1(k) * c.mut(i, j) + c.c2(k)));
    cr = vel * c.dt / dz / mu;
    lf = mu * (dz / c.dt);
  }
  const float l = lf * flux_upwind(c.fo(i, k - 1, j), c.fo(i, k, j), cr);
  float h;
  if (k == c.kts + 1 || k == c.ktf) h = c.rom(i, k, j) * (c.fzm(k) * c.f(i, k, j) + c.fzp(k) * c.f(i, k - 1, j));
  else h = vel * pflux3(c.f(i, k - 2, j), c.f(i, k - 1, j), c.f(i, k, j), c.f(i, k + 1, j), -vel);
  *lo = l; *hi = h - l;
}
// Cells the limiter acts on (module_advect_em.F:7681-7708): next to an open
// boundary not the boundary row itself.
__device__ __forceinline__ bool pd_limited(const Mem& m, int i, int j) {
  return (!m.cf.open_xs || i >= m.ids + 1) && (!m.cf.open_xe || i <= m.ide - 2) && (!m.cf.open_ys || j >= m.jds + 1) &&
         (!m.cf.open_ye || j <= m.jde - 2);
}
// Cells that take the x (y) flux divergence (:7822-7823, :7851-7852).
__device__ __forceinline__ bool pd_xdiv(const Mem& m, int i) {
  return (!m.cf.open_xs || i >= m.ids + 1) && (!m.cf.open_xe || i <= m.ide - 2);
}
__device__ __forceinline__ bool pd_ydiv(const Mem& m, int j) {
  return (!m.cf.open_ys || j >= m.jds + 1) && (!m.cf.open_ye || j <= m.jde - 2);
}
// Limiter factor of cell (i, k, j), or -1 where the cell is not limited.
__device__ __forceinline__ float pd_scale_cell(const Mem& m, const PDCtx& c, int i, int k, int j) {
  if (!pd_limited(m, i, j)) return -1.f;
  float hx0, lx0, hx1, lx1, hy0, ly0, hy1, ly1, hz0, lz0, hz1, lz1;
  pd_fx(m, c, i, k, j, &hx0, &lx0); pd_fx(m, c, i + 1, k, j, &hx1, &lx1);
  pd_fy(m, c, i, k, j, &hy0, &ly0); pd_fy(m, c, i, k, j + 1, &hy1, &ly1);
  pd_fz(c, i, k, j, &hz0, &lz0); pd_fz(c, i, k + 1, j, &hz1, &lz1);
  const float mx = c.msftx(i, j), my = c.msfty(i, j), dt = c.dt;
  const float ph_low = ((c.c1(k) * c.mub(i, j) + c.c2(k)) + (c.c1(k) * c.mu_old(i, j))) * c.fo(i, k, j) -
                       dt * (mx * my * (c.rdx * (lx1 - lx0) + c.rdy * (ly1 - ly0)) + my * c.rdzw(k) * (lz1 - lz0));
  const float flux_out = dt * ((mx * my) * (c.rdx * (fmaxf_f(0.f, hx1) - fminf_f(0.f, hx0)) +
                                            c.rdy * (fmaxf_f(0.f, hy1) - fminf_f(0.f, hy0))) +
                               my * c.rdzw(k) * (fminf_f(0.f, hz1) - fmaxf_f(0.f, hz0)));
  float s = -1.f;
  if (flux_out > ph_low) s = fmaxf_f(0.f, ph_low / (flux_out + 1.e-20f));
  return s;
}
// advect_scalar_pd's tendency at mass point (i, k, j): t minus the radiation
// terms, then the divergence of the limited fluxes (z, then x, then y), each
// face scaled by its upwind cell's factor scale(ci, ck, cj) (a face is only
// ever modified by its upwind cell, so the result does not depend on the
// reference's loop order).
template <class SC>
__device__ __forceinline__ float pd_tend_cell(const Mem& m, const PDCtx& c, int i, int k, int j, float t, SC scale) {
  auto lim = [&](float v, int ci, int ck, int cj) {
    const float s = scale(ci, ck, cj);
    return s >= 0.f ? s * v : v;
  };
  t = scalar_radiation(m, c.f, c.fo, c.ru, c.rv, t, i, j, k);
  float hz0, lz0, hz1, lz1;
  pd_fz(c, i, k, j, &hz0, &lz0); pd_fz(c, i, k + 1, j, &hz1, &lz1);
  // vertical face k: the cell below (k-1) owns negative flux, the cell above (k) positive flux
  if (k > 1) { if (hz0 < 0.f) hz0 = lim(hz0, i, k - 1, j); else if (hz0 > 0.f) hz0 = lim(hz0, i, k, j); }
  if (k + 1 < c.kde) { if (hz1 < 0.f) hz1 = lim(hz1, i, k, j); else if (hz1 > 0.f) hz1 = lim(hz1, i, k + 1, j); }
  t = t - c.rdzw(k) * (hz1 - hz0 + lz1 - lz0);
  const float mx = c.msftx(i, j);
  if (pd_xdiv(m, i)) {
    float hx0, lx0, hx1, lx1;
    pd_fx(m, c, i, k, j, &hx0, &lx0); pd_fx(m, c, i + 1, k, j, &hx1, &lx1);
    // face (i): left cell i-1 owns positive flux, cell i owns negative flux
    if (hx0 > 0.f) hx0 = lim(hx0, i - 1, k, j); else if (hx0 < 0.f) hx0 = lim(hx0, i, k, j);
    if (hx1 > 0.f) hx1 = lim(hx1, i, k, j); else if (hx1 < 0.f) hx1 = lim(hx1, i + 1, k, j);
    t = t - mx * (c.rdx * (hx1 - hx0 + lx1 - lx0));
  }
  if (pd_ydiv(m, j)) {
    float hy0, ly0, hy1, ly1;
    pd_fy(m, c, i, k, j, &hy0, &ly0); pd_fy(m, c, i, k, j + 1, &hy1, &ly1);
    if (hy0 > 0.f) hy0 = lim(hy0, i, k, j - 1); else if (hy0 < 0.f) hy0 = lim(hy0, i, k, j);
    if (hy1 > 0.f) hy1 = lim(hy1, i, k, j); else if (hy1 < 0.f) hy1 = lim(hy1, i, k, j + 1);
    t = t - mx * (c.rdy * (hy1 - hy0 + ly1 - ly0));
  }
  return t;
}

}  // namespace wrfgpu
