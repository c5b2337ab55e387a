// Fused scalar transport of the large step: advection and rk_update_scalar
// in one column-marching pass per species, writing the new scalar into the
// member's spare buffer (swapped with the current one afterwards).
//
//   k_scalar_adv_update  advect_scalar (module_advect_em.F:3394-3650 5th-order
//                        horizontal, :4306-4333 3rd-order vertical) followed by
//                        rk_update_scalar (module_em.F:1587-1799), every species
//                        whose scheme is not the positive-definite one at this stage
//   k_scalar_pd_update   advect_scalar_pd (module_advect_em.F:6505-6779 fluxes,
//                        :7595-7645 vertical, limiter :7681-7781, divergence
//                        :7783-7883) followed by rk_update_scalar, at the last stage
//
// Layout: one block per (TX x TY tile of mass columns, pair of species):
// two species in the lanes of packed FP32 arithmetic (pair.cuh) share the
// staged mass fluxes, Courant numbers and column constants; the block
// marches k from kts to ktf.  The 3-D inputs of each level (the scalar,
// the old scalar, ru_m, rv_m) are staged in shared memory as TMA tile loads
// of the tile plus a 4-point halo, several levels ahead in a ring of slots
// that complete on mbarriers; every x- and y-face flux is computed once per
// level into shared memory, vertical stencils live in per-column register
// windows, and the new value is written once.  The arithmetic of each flux,
// limiter factor, divergence and update is the reference's, term for term
// and in its order, so the results are bit-identical to the separate routine
// kernels of k_scalar.cu.
//
// HBM traffic per species and stage (algorithmic): read q, q_old, write the
// new q (+ q_old at stage 1); the mass fluxes ru_m, rv_m, ww_m are read by
// the species blocks of a tile back to back and come from L2 after the first.
#include "common.cuh"
#include "kernels.h"
#include "pair.cuh"

namespace wrfgpu {

__device__ __forceinline__ bool pd_scheme(const Mem& m, int species, int rk_step) {
  int adv = species < m.n_moist ? m.cf.moist_adv_opt : m.cf.scalar_adv_opt;
  return rk_step == m.cf.rk_ord && adv == 1;
}

// Staged plane: the tile plus a 4-point halo, origin (i0 - 4, j0 - 4).
constexpr int HW = TX + 2 * TMA_HALO, HH = TY + 2 * TMA_HALO, HPLANE = HW * HH;
constexpr unsigned HPLANE_BYTES = HPLANE * 4;

// A ring of level slots; each slot holds NPL halo planes and completes on its
// own mbarrier.  Only thread 0 issues; everyone waits.
template <int NPL, int NSLOT>
struct PlaneRing {
  float* buf;      // [NSLOT][NPL][HH][HW]
  uint64_t* bar;   // [NSLOT]
  int kts;
  __device__ float* plane(int slot, int p) const { return buf + (slot * NPL + p) * HPLANE; }
  __device__ int slot_of(int k) const { return (k - kts) % NSLOT; }
  // thread 0: load level k of the NPL fields into its slot
  __device__ void issue(int k, const CUtensorMap* const* maps, int x0, int z0, int kms) const {
    const int sl = slot_of(k);
    fence_proxy_async_smem();
    mbar_expect_tx(&bar[sl], NPL * HPLANE_BYTES);
    for (int p = 0; p < NPL; ++p) tma_load_3d(plane(sl, p), maps[p], x0, k - kms, z0, &bar[sl]);
  }
  __device__ bool wait(int k) const { return mbar_wait(&bar[slot_of(k)], ((k - kts) / NSLOT) & 1); }
};

// ------------------------------------------------------------------ non-PD
constexpr int ADV_RING = 4;  // levels k .. k+3 in flight
constexpr int ADV_NPL = 4;   // q of both species of the pair, ru_m, rv_m
// face planes (float2: both species), two levels
constexpr size_t ADV_SMEM = (size_t)ADV_RING * ADV_NPL * HPLANE_BYTES + 2 * (TY * (TX + 1) + (TY + 1) * TX) * 8 +
                            ADV_RING * 8;

// Species pair (2 p, 2 p + 1) of block (tile, p) that take the 5th/3rd-order
// scheme at this stage; where only one of them does, both lanes carry it and
// it is written once.  False when neither does.
struct SpeciesPair {
  int s0, s1;
  bool store1;
};
__device__ __forceinline__ bool adv_pair(const Mem& m, int p, int rk_step, SpeciesPair* sp) {
  const int sa = 2 * p, sb = 2 * p + 1;
  const bool va = sa < m.nsp && !pd_scheme(m, sa, rk_step), vb = sb < m.nsp && !pd_scheme(m, sb, rk_step);
  if (!va && !vb) return false;
  sp->s0 = va ? sa : sb;
  sp->s1 = vb ? sb : sp->s0;
  sp->store1 = va && vb;
  return true;
}

// SCT: some member stores sc_tend (the species' sixth-order diffusion); the
// variant without it keeps the common case free of its load and test.
// pairs: bit p set = pair p of every member is transported by this launch.
template <int MINB, bool SCT>
__global__ void __launch_bounds__(TX* TY, MINB) k_scalar_adv_update(TileLaunch L, int rk_step, unsigned pairs) {
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, TILE_PER_PAIR);
  if (!((pairs >> tp.sub) & 1u)) return;  // block-uniform
  const Mem& m = block_member(L.mem, tp.m);
  SpeciesPair sp;
  if (!adv_pair(m, tp.sub, rk_step, &sp)) return;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = tp.i0, j0 = tp.j0;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(m.kte, m.kde - 1);
  const int kts = m.kts, kte = m.kte, kme = m.kme;

  PlaneRing<ADV_NPL, ADV_RING> ring;
  ring.buf = (float*)smem;
  float2* fx_base = reinterpret_cast<float2*>(ring.buf + ADV_RING * ADV_NPL * HPLANE);  // [2][TY][TX+1]
  float2* fy_base = fx_base + 2 * TY * (TX + 1);                                      // [2][TY+1][TX]
  ring.bar = reinterpret_cast<uint64_t*>(fy_base + 2 * (TY + 1) * TX);
  ring.kts = kts;
  const CUtensorMap* maps[ADV_NPL] = {tmap_of(m, m.qmap[sp.s0], BOX_HALO), tmap_of(m, m.qmap[sp.s1], BOX_HALO),
                                      tmap_of(m, WRFGPU_RU_M, BOX_HALO), tmap_of(m, WRFGPU_RV_M, BOX_HALO)};
  const int x0 = i0 - TMA_HALO - m.ims, z0 = j0 - TMA_HALO - m.jms;
  if (tid == 0) {
    for (int q = 0; q < ADV_RING; ++q) mbar_init(&ring.bar[q], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int d = 0; d < ADV_RING - 1 && kts + d <= ktf; ++d) ring.issue(kts + d, maps, x0, z0, m.kms);

  const int i = i0 + tx, j = j0 + ty;
  const bool own = i <= itf && j <= jtf;
  const Stage st = stage_of(m, rk_step);
  const F3 fa = f3p(m, m.q[sp.s0]), fb = f3p(m, m.q[sp.s1]), olda = f3p(m, m.qo[sp.s0]), oldb = f3p(m, m.qo[sp.s1]);
  const F3 outa = f3p(m, m.qa[sp.s0]), outb = f3p(m, m.qa[sp.s1]), rom = f3(m, WRFGPU_WW_M);
  F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP), rdzw = f1(m, WRFGPU_RDNW);
  F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H);
  // sc_tend of each species (null unless it is diffused); at the last stage a
  // positive-definite species' sc_tend was spent (and zeroed) by the PD pre-update
  const F3 scta = f3p(m, (!SCT || pd_scheme(m, sp.s0, rk_step)) ? nullptr : sc_tend_of(m, sp.s0));
  const F3 sctb = f3p(m, (!SCT || pd_scheme(m, sp.s1, rk_step)) ? nullptr : sc_tend_of(m, sp.s1));
  auto ld2 = [](const F3& a, const F3& b, int ii, int k, int jj) { return make_float2(a(ii, k, jj), b(ii, k, jj)); };
  float msftx = 0.f, msfty = 0.f, muold = 0.f, munew = 0.f;
  // own-column registers: scalar window fld(k-1 .. k+2), next values of old and rom
  float2 wm1 = bc2(0.f), w0 = bc2(0.f), wp1 = bc2(0.f), wp2 = bc2(0.f), old_k = bc2(0.f);
  float rom_k1 = 0.f;
  if (own) {
    msftx = f2(m, WRFGPU_MSFTX)(i, j);
    msfty = f2(m, WRFGPU_MSFTY)(i, j);
    muold = f2(m, WRFGPU_MU_1)(i, j) + f2(m, WRFGPU_MUB)(i, j);
    munew = f2(m, WRFGPU_MU_2)(i, j) + f2(m, WRFGPU_MUB)(i, j);
    w0 = ld2(fa, fb, i, kts, j);
    wp1 = ld2(fa, fb, i, kts + 1, j);
    wp2 = (kts + 2 <= kme) ? ld2(fa, fb, i, kts + 2, j) : bc2(0.f);
    old_k = rk_step == 1 ? bc2(0.f) : ld2(olda, oldb, i, kts, j);
    rom_k1 = rom(i, kts + 1, j);
  }
  const float rdx = m.rdx, rdy = m.rdy;
  float2 vf_lo = bc2(0.f);  // vf(kts) = 0
  bool ok = true;
  for (int k = kts; k <= ktf; ++k) {
    if (tid == 0 && k + ADV_RING - 1 <= ktf) ring.issue(k + ADV_RING - 1, maps, x0, z0, m.kms);
    ok = ring.wait(k) && ok;
    const int sl = ring.slot_of(k);
    const float* QA = ring.plane(sl, 0);
    const float* QB = ring.plane(sl, 1);
    const float* U = ring.plane(sl, 2);
    const float* V = ring.plane(sl, 3);
    auto q2 = [&](int o) { return make_float2(QA[o], QB[o]); };
    float2* FX = fx_base + (k & 1) * TY * (TX + 1);
    float2* FY = fy_base + (k & 1) * (TY + 1) * TX;
    // x faces i0 .. i0+TX of rows j0 .. j0+TY-1 and y faces j0 .. j0+TY of
    // columns i0 .. i0+TX-1: every thread its cell's left and bottom faces;
    // the TY right faces of the last column go to warp TY-1 and the TX top
    // faces of the last row to warp TY-2, so no warp computes more than three
    auto xface = [&](int r, int c) {  // face (i0 + c, j0 + r)
      const int o = (r + TMA_HALO) * HW + c + TMA_HALO;
      const float vel = U[o];
      FX[r * (TX + 1) + c] = muls(vel, flux5_2(q2(o - 3), q2(o - 2), q2(o - 1), q2(o), q2(o + 1), q2(o + 2), vel));
    };
    auto yface = [&](int r, int c) {
      const int o = (r + TMA_HALO) * HW + c + TMA_HALO;
      const float vel = V[o];
      FY[r * TX + c] = muls(vel, flux5_2(q2(o - 3 * HW), q2(o - 2 * HW), q2(o - HW), q2(o), q2(o + HW),
                                         q2(o + 2 * HW), vel));
    };
    xface(ty, tx);
    yface(ty, tx);
    if (ty == TY - 1 && tx < TY) xface(tx, TX);
    if (ty == TY - 2) yface(TY, tx);
    __syncthreads();
    if (own) {
      // prefetch the next level's own-column values
      const float2 wp3 = (k + 3 <= kme) ? ld2(fa, fb, i, k + 3, j) : bc2(0.f);
      const float2 old_n = (rk_step != 1 && k + 1 <= ktf) ? ld2(olda, oldb, i, k + 1, j) : bc2(0.f);
      const float rom_n = (k + 2 <= kme) ? rom(i, k + 2, j) : 0.f;
      // vertical flux of the upper face k+1 (lower face kept from the previous level)
      float2 vf_hi;
      const int kk = k + 1;
      if (kk == kts || kk == kte) vf_hi = bc2(0.f);
      else if (kk == kts + 1 || kk == ktf) vf_hi = muls(rom_k1, add2(muls(fzm(kk), wp1), muls(fzp(kk), w0)));
      else vf_hi = muls(rom_k1, flux3_2(wm1, w0, wp1, wp2, -rom_k1));
      float2 t = bc2(0.f);
      t = sub2(t, muls(msftx * rdy, sub2(FY[(ty + 1) * TX + tx], FY[ty * TX + tx])));
      t = sub2(t, muls(msftx * rdx, sub2(FX[ty * (TX + 1) + tx + 1], FX[ty * (TX + 1) + tx])));
      t = sub2(t, muls(rdzw(k), sub2(vf_hi, vf_lo)));
      vf_lo = vf_hi;
      // rk_update_scalar (+ sc_tend: the species' stage-1 sixth-order diffusion)
      float2 tendency = muls(msfty, t);
      if (SCT && scta.p) tendency.x = tendency.x + scta(i, k, j);
      if (SCT && sctb.p) tendency.y = tendency.y + sctb(i, k, j);
      float2 q1;
      if (rk_step == 1) {
        q1 = w0;
        olda(i, k, j) = q1.x;
        if (sp.store1) oldb(i, k, j) = q1.y;
      } else {
        q1 = old_k;
      }
      const float2 num = add2(muls(c1(k) * muold + c2(k), q1), muls(st.dt_rk, tendency));
      const float den = c1(k) * munew + c2(k);
      outa(i, k, j) = num.x / den;
      if (sp.store1) outb(i, k, j) = num.y / den;
      // slide
      wm1 = w0; w0 = wp1; wp1 = wp2; wp2 = wp3;
      old_k = old_n; rom_k1 = rom_n;
    }
  }
  if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
}

// ------------------------------------------------------------------ PD Courant numbers
// The Courant numbers of advect_scalar_pd's low-order fluxes
// (module_advect_em.F:6505-6779, :7595-7645) depend on the mass fluxes and
// column masses only, not on the species: formed once per step here, for the
// x face between columns i-1 and i (pdc[0]), the y face between rows j-1 and
// j (pdc[1]) and the z face k of column (i, j) (pdc[2]), over the faces the
// PD kernel's limiter region reads (columns its-1 .. itf+2, rows
// jts-1 .. jtf+2), with the PD kernel's expressions (the same bits).
// Column layout: one thread per (i, j) of the memory extent, levels in
// chunks of four with their loads issued first.
__global__ void __launch_bounds__(BX* BY) k_pd_courant(Launch L, int rk_step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid || !m.pdc[0]) return;
  const int i = bp.i, j = bp.j;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(m.kte, m.kde - 1);
  if (i < m.its - 1 || i > itf + 2 || j < m.jts - 1 || j > jtf + 2) return;
  const Stage st = stage_of(m, rk_step);
  const float dt = st.dt_rk, rdx = m.rdx, rdy = m.rdy;
  const F2 mut = f2(m, WRFGPU_MUTS), msx = f2(m, WRFGPU_MSFTX), msy = f2(m, WRFGPU_MSFTY);
  const F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H), rdzw = f1(m, WRFGPU_RDNW);
  const F3 ru = f3(m, WRFGPU_RU_M), rv = f3(m, WRFGPU_RV_M), rw = f3(m, WRFGPU_WW_M);
  const F3 crx = f3p(m, m.pdc[0]), cry = f3p(m, m.pdc[1]), crz = f3p(m, m.pdc[2]);
  const F3 lfx = f3p(m, m.pdc[3]), lfy = f3p(m, m.pdc[4]), lfz = f3p(m, m.pdc[5]);
  const float mt = mut(i, j), mtx = mut(i - 1, j), mty = mut(i, j - 1);
  const float xdx = 2.f / (msy(i, j) + msy(i - 1, j)) / rdx;
  const float ydy = 2.f / (msx(i, j) + msx(i, j - 1)) / rdy;
  const float xdxt = xdx / dt, ydyt = ydy / dt;
  const int klast = max(ktf, m.kde - 1);
  struct V { float u, v, w; };
  chunked_levels<4, V>(
      m.kts, klast,
      [&](int k, V& d) {
        d.u = k <= ktf ? ru.ro(i, k, j) : 0.f;
        d.v = k <= ktf ? rv.ro(i, k, j) : 0.f;
        d.w = rw.ro(i, k, j);
      },
      [&](int k, const V& d) {
        if (k <= ktf) {
          const float c1k = c1(k), c2k = c2(k);
          const float mux = 0.5f * ((c1k * mt + c2k) + (c1k * mtx + c2k));
          crx(i, k, j) = d.u * dt / xdx / mux;
          lfx(i, k, j) = mux * xdxt;
          const float muy = 0.5f * ((c1k * mt + c2k) + (c1k * mty + c2k));
          cry(i, k, j) = d.v * dt / ydy / muy;
          lfy(i, k, j) = muy * ydyt;
        }
        if (k > 1 && k < m.kde && k - 1 >= m.kms) {  // z face k
          const float dz = 2.f / (rdzw(k) + rdzw(k - 1));
          const float muz = 0.5f * ((c1(k) * mt + c2(k)) + (c1(k) * mt + c2(k)));
          crz(i, k, j) = d.w * dt / dz / muz;
          lfz(i, k, j) = muz * (dz / dt);
        }
      });
}

// ------------------------------------------------------------------ PD
struct PDPlanes {
  static constexpr int SW = TX + 2, SH = TY + 2;  // limiter factors, halo 1
  static constexpr int XW = TX + 3, XH = TY + 2;  // x faces i0-1 .. i0+TX+1, rows j0-1 .. j0+TY
  static constexpr int YW = TX + 2, YH = TY + 3;  // y faces j0-1 .. j0+TY+1, columns i0-1 .. i0+TX
  static constexpr int XN = XW * XH, YN = YW * YH, SN = SW * SH;
};
constexpr int PD_RING = 2;   // levels L, L+1 in flight
// q and q_old of both species of the pair, ru_m, rv_m, and the x and y faces'
// Courant numbers and low-order flux factors (k_pd_courant)
constexpr int PD_NPL = 10;
constexpr int PD_FSLOT = 3;  // face planes kept for three levels
// face planes (float2: both species), limiter factors (float2), mbarriers
constexpr size_t PD_SMEM = (size_t)PD_RING * PD_NPL * HPLANE_BYTES +
                           8 * (PD_FSLOT * 2 * (PDPlanes::XN + PDPlanes::YN) + 2 * PDPlanes::SN) + PD_RING * 8;
// One thread per limiter cell of the 34 x 10 region (tile + 1), plus one
// thread per face the cells' left / bottom faces leave out (the 10 x faces of
// column i0 + 33 and the 34 y faces of row j0 + 9): every thread computes at
// most one x face and one y face per level, with no loop.
constexpr int PD_THREADS = PDPlanes::SN + PDPlanes::XH + PDPlanes::YW;  // 384

// One cell of the limiter region (tile + 1): its column's vertical window,
// both species of the pair in the lanes.
struct ZCell {
  int i, j;
  bool valid;
  float mut, mub, mu_old, mx, my;
  float2 fm1, f0, fp1, fp2;  // scalar at L-1 .. L+2
  float2 fo0, fop1;          // old scalar at L, L+1
  float2 hz0, lz0;           // z face L (lower face of level L)
  float2 hz1, lz1;           // z face L+1
  float2 hzm, lzm;           // z face L-1
  float2 fom1;               // old scalar at L-1
  float romp1;               // ww_m at face L+1
};

// Column constants of level k, staged in shared memory once per block:
// a = {c1h, c2h, rdnw, 0}, b = {0, fnm, fnp, 0}.
struct LevelConst { float4 a, b; };

// z face kk = L+1 of a limiter cell (advect_scalar_pd's fqz, fqzl).
__device__ __forceinline__ void zface(const ZCell& c, int kk, const LevelConst& t, float cr, float lf, int kts, int kde,
                                      int ktf, float2* hi, float2* lo) {
  if (kk == 1 || kk == kde) { *hi = bc2(0.f); *lo = bc2(0.f); return; }
  const float vel = c.romp1;
  const float2 l = muls(lf, flux_upwind_2(c.fo0, c.fop1, upwind_weights(cr)));
  float2 h;
  if (kk == kts + 1 || kk == ktf) h = muls(vel, add2(muls(t.b.y, c.fp1), muls(t.b.z, c.f0)));
  else h = muls(vel, pflux3_2(c.fm1, c.f0, c.fp1, c.fp2, -vel));
  *lo = l; *hi = sub2(h, l);
}

// advect_scalar_pd's flux limiting of one face by its upwind cell's factor
// (sc < 0: the cell is not limited), one lane.
__device__ __forceinline__ float lim1(float v, float sc) { return sc >= 0.f ? sc * v : v; }

// Positive-definite transport of a pair of species (the lanes of packed
// FP32 arithmetic, pair.cuh): species 2 p and 2 p + 1 of block (tile, p).
// Where only one species of the pair uses the positive-definite scheme at
// this stage, both lanes carry it and it is written once.
template <int MINB>
__global__ void __launch_bounds__(PD_THREADS, MINB) k_scalar_pd_update(TileLaunch L, int rk_step) {
  using P = PDPlanes;
  extern __shared__ __align__(128) unsigned char smem[];
  const TilePos tp = tile_pos(L, TILE_PER_PAIR);
  const Mem& m = block_member(L.mem, tp.m);
  const int sa = 2 * tp.sub, sb = 2 * tp.sub + 1;
  const bool va = sa < m.nsp && pd_scheme(m, sa, rk_step), vb = sb < m.nsp && pd_scheme(m, sb, rk_step);
  if (!va && !vb) return;
  const int s0 = va ? sa : sb, s1 = vb ? sb : s0;
  const bool store1 = va && vb;
  const int tid = threadIdx.x;
  const int i0 = tp.i0, j0 = tp.j0;
  const int itf = min(m.ite, m.ide - 1), jtf = min(m.jte, m.jde - 1), ktf = min(m.kte, m.kde - 1);
  const int kts = m.kts, kme = m.kme;
  const Stage st = stage_of(m, rk_step);
  const float dt = st.dt_rk, rdx = m.rdx, rdy = m.rdy;

  PlaneRing<PD_NPL, PD_RING> ring;
  ring.buf = (float*)smem;
  float2* p = reinterpret_cast<float2*>(ring.buf + PD_RING * PD_NPL * HPLANE);
  float2* sXH = p; p += PD_FSLOT * P::XN;
  float2* sXL = p; p += PD_FSLOT * P::XN;
  float2* sYH = p; p += PD_FSLOT * P::YN;
  float2* sYL = p; p += PD_FSLOT * P::YN;
  float2* sSC = p; p += 2 * P::SN;
  const int nlev = m.kme - m.kms + 1;
  LevelConst* sLV = reinterpret_cast<LevelConst*>(p);  // [k - kms]
  ring.bar = reinterpret_cast<uint64_t*>(sLV + nlev);
  ring.kts = kts;
  const CUtensorMap* maps[PD_NPL] = {tmap_of(m, m.qmap[s0], BOX_HALO), tmap_of(m, m.qmap[s1], BOX_HALO),
                                     tmap_of(m, WRFGPU_N3D + 3 * s0 + 1, BOX_HALO),
                                     tmap_of(m, WRFGPU_N3D + 3 * s1 + 1, BOX_HALO),
                                     tmap_of(m, WRFGPU_RU_M, BOX_HALO), tmap_of(m, WRFGPU_RV_M, BOX_HALO),
                                     tmap_of(m, PDC_SLOT + 0, BOX_HALO), tmap_of(m, PDC_SLOT + 3, BOX_HALO),
                                     tmap_of(m, PDC_SLOT + 1, BOX_HALO), tmap_of(m, PDC_SLOT + 4, BOX_HALO)};
  const int x0 = i0 - TMA_HALO - m.ims, z0 = j0 - TMA_HALO - m.jms;
  if (tid == 0) {
    for (int q = 0; q < PD_RING; ++q) mbar_init(&ring.bar[q], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int d = 0; d < PD_RING - 1 && kts + d <= ktf; ++d) ring.issue(kts + d, maps, x0, z0, m.kms);

  const F3 fa = f3p(m, m.q[s0]), fb = f3p(m, m.q[s1]), foa = f3p(m, m.qo[s0]), fob = f3p(m, m.qo[s1]);
  const F3 outa = f3p(m, m.qa[s0]), outb = f3p(m, m.qa[s1]), rom = f3(m, WRFGPU_WW_M);
  const F3 crza = f3p(m, m.pdc[2]), lfza = f3p(m, m.pdc[5]);
  F2 mut2 = f2(m, WRFGPU_MUTS), msx2 = f2(m, WRFGPU_MSFTX), msy2 = f2(m, WRFGPU_MSFTY);
  F2 mub2 = f2(m, WRFGPU_MUB), mu1 = f2(m, WRFGPU_MU_1), mu2 = f2(m, WRFGPU_MU_2);
  {
    F1 c1 = f1(m, WRFGPU_C1H), c2 = f1(m, WRFGPU_C2H), rdzw = f1(m, WRFGPU_RDNW);
    F1 fzm = f1(m, WRFGPU_FNM), fzp = f1(m, WRFGPU_FNP);
    for (int q = tid; q < nlev; q += PD_THREADS) {
      const int k = m.kms + q;
      sLV[q].a = make_float4(c1(k), c2(k), rdzw(k), 0.f);
      sLV[q].b = make_float4(0.f, fzm(k), fzp(k), 0.f);
    }
  }
  __syncthreads();  // the level table is complete
  auto ld2 = [](const F3& a, const F3& b, int i, int k, int j) { return make_float2(a(i, k, j), b(i, k, j)); };

  // this thread's limiter cell (sx, sy) of the region, and its faces
  // cells 0..31 of each row on one warp (contiguous shared-memory rows, no
  // bank conflicts), the rows' last two cells on the next 20 threads
  static_assert(P::SW == 34 && 32 * P::SH < P::SN, "thread map assumes 32-wide tiles");
  const bool has_cell = tid < P::SN;
  int sx = 0, sy = 0;
  if (has_cell) {
    if (tid < 32 * P::SH) { sy = tid >> 5; sx = tid & 31; }
    else { const int q = tid - 32 * P::SH; sy = q >> 1; sx = 32 + (q & 1); }
  }
  int xq = -1, yq = -1;  // x / y face this thread computes (index in the face planes)
  if (has_cell) {
    xq = sy * P::XW + sx;  // left face of the cell
    yq = sy * P::YW + sx;  // bottom face of the cell
  } else {
    const int q = tid - P::SN;
    if (q < P::XH) xq = q * P::XW + (P::XW - 1);     // column i0 + TX + 1
    else yq = (P::YH - 1) * P::YW + (q - P::XH);     // row j0 + TY + 1
  }
  // level-independent data of the faces: the face's point and its offset in
  // the halo plane
  bool xok = false, yok = false;
  int xo = 0, yo = 0;
  if (xq >= 0) {
    const int r = xq / P::XW, c = xq - r * P::XW;
    const int ii = i0 - 1 + c, jj = j0 - 1 + r;
    xok = ii >= m.its - 1 && ii <= itf + 2 && jj >= m.jts - 1 && jj <= jtf + 1;
    xo = (r + TMA_HALO - 1) * HW + (c + TMA_HALO - 1);  // (i0-1+c, j0-1+r) in the halo plane
  }
  if (yq >= 0) {
    const int r = yq / P::YW, c = yq - r * P::YW;
    const int ii = i0 - 1 + c, jj = j0 - 1 + r;
    yok = ii >= m.its - 1 && ii <= itf + 1 && jj >= m.jts - 1 && jj <= jtf + 2;
    yo = (r + TMA_HALO - 1) * HW + (c + TMA_HALO - 1);
  }

  // the limiter cell's vertical window
  ZCell c;
  c.i = i0 - 1 + sx; c.j = j0 - 1 + sy;
  c.valid = has_cell && c.i >= m.its - 1 && c.i <= itf + 1 && c.j >= m.jts - 1 && c.j <= jtf + 1;
  c.mut = c.mub = c.mu_old = 0.f; c.mx = c.my = 1.f;
  c.fm1 = c.f0 = c.fp1 = c.fp2 = c.fo0 = c.fop1 = c.fom1 = bc2(0.f);
  c.hz0 = c.lz0 = c.hz1 = c.lz1 = c.hzm = c.lzm = bc2(0.f);
  c.romp1 = 0.f;
  if (c.valid) {
    c.mut = mut2(c.i, c.j); c.mub = mub2(c.i, c.j); c.mu_old = mu1(c.i, c.j);
    c.mx = msx2(c.i, c.j); c.my = msy2(c.i, c.j);
    // window for L = kts (f(L-1) unused: face kts+1 is second order); z face kts = 0
    c.f0 = ld2(fa, fb, c.i, kts, c.j);
    c.fp1 = ld2(fa, fb, c.i, kts + 1, c.j);
    c.fp2 = (kts + 2 <= kme) ? ld2(fa, fb, c.i, kts + 2, c.j) : bc2(0.f);
    c.fo0 = ld2(foa, fob, c.i, kts, c.j);
    c.fop1 = ld2(foa, fob, c.i, kts + 1, c.j);
    c.romp1 = rom(c.i, kts + 1, c.j);
  }
  // interior cells of the region are the tile's cells: they also update
  const int i = c.i, j = c.j;
  const bool own = has_cell && sx >= 1 && sx <= TX && sy >= 1 && sy <= TY && i <= itf && j <= jtf;
  float muold_u = 0.f, munew_u = 0.f, msfty_o = 1.f, msftx_o = 1.f;
  if (own) {
    muold_u = mu1(i, j) + mub2(i, j);
    munew_u = mu2(i, j) + mub2(i, j);
    msfty_o = msy2(i, j);
    msftx_o = msx2(i, j);
  }
  float2 sc_m1 = bc2(-1.f), sc_0 = bc2(-1.f), sc_p1 = bc2(-1.f);  // own column factors at levels L-2, L-1, L
  const int so = sy * P::SW + sx;                // own cell in the factor planes
  const int xoc = sy * P::XW + sx, yoc = sy * P::YW + sx;  // own cell's left / bottom faces
  bool ok = true;
  // the own cell's z face Courant number and low-order factor of the next
  // level, loaded one iteration ahead
  auto zcourant = [&](int lv, float* cr, float* lf) {
    const bool zin = c.valid && lv <= ktf && lv + 1 > 1 && lv + 1 < m.kde;
    *cr = zin ? crza.ro(c.i, lv + 1, c.j) : 0.f;
    *lf = zin ? lfza.ro(c.i, lv + 1, c.j) : 0.f;
  };
  float crz_n, lfz_n;
  zcourant(kts, &crz_n, &lfz_n);

  // One barrier per level.  Iteration Lv: faces of level Lv (face slot Lv % 3)
  // and the z face Lv+1 of the own cell; barrier; limiter factor of level Lv
  // (factor slot Lv & 1); divergence of level Lv-1, which reads face slot
  // (Lv-1) % 3, the neighbours' factors of level Lv-1 (written before this
  // barrier) and its own factor of level Lv (this thread's).  A slot is
  // rewritten only after a later barrier that every reader of its previous
  // level has passed: face slot (Lv+1) % 3 held level Lv-2, last read before
  // this barrier; factor slot (Lv+1) & 1 holds level Lv-1, read before the
  // next one; the ring slot of level Lv+3 (issued after this barrier) held
  // level Lv, read before it.
  for (int Lv = kts; Lv <= ktf + 1; ++Lv) {
    const int slot = Lv & 1;
    float c1k = 0.f, c2k = 0.f, rdzwk = 0.f;
    if (Lv <= ktf) {
      const float crz = crz_n, lfz = lfz_n;
      if (tid == 0 && Lv + PD_RING - 1 <= ktf) ring.issue(Lv + PD_RING - 1, maps, x0, z0, m.kms);
      const float4 tl = sLV[Lv - m.kms].a;
      c1k = tl.x; c2k = tl.y; rdzwk = tl.z;
      ok = ring.wait(Lv) && ok;
      const int rs = ring.slot_of(Lv);
      const float* FA = ring.plane(rs, 0);
      const float* FB = ring.plane(rs, 1);
      const float* FOA = ring.plane(rs, 2);
      const float* FOB = ring.plane(rs, 3);
      const float* RU = ring.plane(rs, 4);
      const float* RV = ring.plane(rs, 5);
      const float* CRX = ring.plane(rs, 6);
      const float* LFX = ring.plane(rs, 7);
      const float* CRY = ring.plane(rs, 8);
      const float* LFY = ring.plane(rs, 9);
      auto q2 = [&](int o) { return make_float2(FA[o], FB[o]); };
      auto qo2 = [&](int o) { return make_float2(FOA[o], FOB[o]); };
      const int fs = Lv % PD_FSLOT;
      float2* XH = sXH + fs * P::XN; float2* XL = sXL + fs * P::XN;
      float2* YH = sYH + fs * P::YN; float2* YL = sYL + fs * P::YN;
      // ---- this thread's x and y faces of level Lv
      if (xq >= 0) {
        float2 hi = bc2(0.f), lo = bc2(0.f);
        if (xok) {
          const int o = xo;
          const float vel = RU[o];
          lo = muls(LFX[o], flux_upwind_2(qo2(o - 1), qo2(o), upwind_weights(CRX[o])));
          const float2 h = muls(vel, pflux5_2(q2(o - 3), q2(o - 2), q2(o - 1), q2(o), q2(o + 1), q2(o + 2), vel));
          hi = sub2(h, lo);
        }
        XH[xq] = hi; XL[xq] = lo;
      }
      if (yq >= 0) {
        float2 hi = bc2(0.f), lo = bc2(0.f);
        if (yok) {
          const int o = yo;
          const float vel = RV[o];
          lo = muls(LFY[o], flux_upwind_2(qo2(o - HW), qo2(o), upwind_weights(CRY[o])));
          const float2 h =
              muls(vel, pflux5_2(q2(o - 3 * HW), q2(o - 2 * HW), q2(o - HW), q2(o), q2(o + HW), q2(o + 2 * HW), vel));
          hi = sub2(h, lo);
        }
        YH[yq] = hi; YL[yq] = lo;
      }
      // ---- vertical face Lv+1 of this thread's limiter cell
      if (c.valid) zface(c, Lv + 1, sLV[Lv + 1 - m.kms], crz, lfz, kts, m.kde, ktf, &c.hz1, &c.lz1);
    }
    __syncthreads();
    if (Lv <= ktf) {
      const int fs = Lv % PD_FSLOT;
      const float2* XH = sXH + fs * P::XN; const float2* XL = sXL + fs * P::XN;
      const float2* YH = sYH + fs * P::YN; const float2* YL = sYL + fs * P::YN;
      // ---- limiter factor of level Lv (advect_scalar_pd ph_low / flux_out)
      if (c.valid) {
        const float2 hx0 = XH[xoc], hx1 = XH[xoc + 1], lx0 = XL[xoc], lx1 = XL[xoc + 1];
        const float2 hy0 = YH[yoc], hy1 = YH[yoc + P::YW], ly0 = YL[yoc], ly1 = YL[yoc + P::YW];
        const float mx = c.mx, my = c.my;
        const float2 ph_low =
            sub2(muls((c1k * c.mub + c2k) + (c1k * c.mu_old), c.fo0),
                 muls(dt, add2(muls(mx * my, add2(muls(rdx, sub2(lx1, lx0)), muls(rdy, sub2(ly1, ly0)))),
                               muls(my * rdzwk, sub2(c.lz1, c.lz0)))));
        const float2 flux_out =
            muls(dt, add2(muls(mx * my, add2(muls(rdx, sub2(max0_2(hx1), min0_2(hx0))),
                                             muls(rdy, sub2(max0_2(hy1), min0_2(hy0))))),
                          muls(my * rdzwk, sub2(min0_2(c.hz1), max0_2(c.hz0)))));
        float2 sc = bc2(-1.f);
        if (flux_out.x > ph_low.x) sc.x = fmaxf_f(0.f, ph_low.x / (flux_out.x + 1.e-20f));
        if (flux_out.y > ph_low.y) sc.y = fmaxf_f(0.f, ph_low.y / (flux_out.y + 1.e-20f));
        sSC[slot * P::SN + so] = sc;
        sc_p1 = sc;
      }
    }
    // ---- divergence + update of level k = Lv - 1
    const int k = Lv - 1;
    if (k >= kts && own) {
      const int fs = k % PD_FSLOT;
      const float2* XH = sXH + fs * P::XN; const float2* XL = sXL + fs * P::XN;
      const float2* YH = sYH + fs * P::YN; const float2* YL = sYL + fs * P::YN;
      const float2* SC = sSC + (k & 1) * P::SN;
      float2 hx0 = XH[xoc], hx1 = XH[xoc + 1];
      const float2 lx0 = XL[xoc], lx1 = XL[xoc + 1];
      float2 hy0 = YH[yoc], hy1 = YH[yoc + P::YW];
      const float2 ly0 = YL[yoc], ly1 = YL[yoc + P::YW];
      // z faces k (hzm) and k+1 (hz0) of the own column, as of this iteration
      float2 hz0 = c.hzm, hz1 = c.hz0;
      const float2 lz0 = c.lzm, lz1 = c.lz0;
      const float2 s_own = sc_0;
      const float2 sxm = SC[so - 1], sxp = SC[so + 1], sym = SC[so - P::SW], syp = SC[so + P::SW];
      // lane by lane, each face takes its upwind cell's factor: through a
      // horizontal face a positive flux comes from the cell on the low side;
      // through z face k a negative flux comes from the cell below (level
      // k-1), a positive one from the cell above (module_advect_em.F:7762-7779)
      auto limit = [](float2& h, float2 s_from_low, float2 s_from_high) {
        if (h.x > 0.f) h.x = lim1(h.x, s_from_low.x); else if (h.x < 0.f) h.x = lim1(h.x, s_from_high.x);
        if (h.y > 0.f) h.y = lim1(h.y, s_from_low.y); else if (h.y < 0.f) h.y = lim1(h.y, s_from_high.y);
      };
      limit(hx0, sxm, s_own);
      limit(hx1, s_own, sxp);
      limit(hy0, sym, s_own);
      limit(hy1, s_own, syp);
      if (k > 1) {
        if (hz0.x < 0.f) hz0.x = lim1(hz0.x, sc_m1.x); else if (hz0.x > 0.f) hz0.x = lim1(hz0.x, s_own.x);
        if (hz0.y < 0.f) hz0.y = lim1(hz0.y, sc_m1.y); else if (hz0.y > 0.f) hz0.y = lim1(hz0.y, s_own.y);
      }
      if (k + 1 < m.kde) {
        if (hz1.x < 0.f) hz1.x = lim1(hz1.x, s_own.x); else if (hz1.x > 0.f) hz1.x = lim1(hz1.x, sc_p1.x);
        if (hz1.y < 0.f) hz1.y = lim1(hz1.y, s_own.y); else if (hz1.y > 0.f) hz1.y = lim1(hz1.y, sc_p1.y);
      }
      const float mx = msftx_o;
      const float4 tk = sLV[k - m.kms].a;  // c1h, c2h, rdnw of level k
      float2 t = bc2(0.f);
      t = sub2(t, muls(tk.z, sub2(add2(sub2(hz1, hz0), lz1), lz0)));
      t = sub2(t, muls(mx, muls(rdx, sub2(add2(sub2(hx1, hx0), lx1), lx0))));
      t = sub2(t, muls(mx, muls(rdy, sub2(add2(sub2(hy1, hy0), ly1), ly0))));
      // rk_update_scalar (last stage: q1 = q_old)
      const float2 tendency = muls(msfty_o, t);
      const float2 num = add2(muls(tk.x * muold_u + tk.y, c.fom1), muls(dt, tendency));
      const float den = tk.x * munew_u + tk.y;
      outa(i, k, j) = num.x / den;
      if (store1) outb(i, k, j) = num.y / den;
    }
    // ---- slide the windows to level Lv+1 (loads for the next level issued now)
    sc_m1 = sc_0; sc_0 = sc_p1;
    zcourant(Lv + 1, &crz_n, &lfz_n);
    if (c.valid) {
      c.hzm = c.hz0; c.lzm = c.lz0;
      c.hz0 = c.hz1; c.lz0 = c.lz1;
      c.fom1 = c.fo0;
      c.fm1 = c.f0; c.f0 = c.fp1; c.fp1 = c.fp2;
      c.fp2 = (Lv + 3 <= kme) ? ld2(fa, fb, c.i, Lv + 3, c.j) : bc2(0.f);
      c.fo0 = c.fop1;
      c.fop1 = (Lv + 2 <= kme) ? ld2(foa, fob, c.i, Lv + 2, c.j) : bc2(0.f);
      c.romp1 = (Lv + 2 <= kme) ? rom(c.i, Lv + 2, c.j) : 0.f;
    }
  }
  if (!ok && tid == 0) raise_err(m, ERR_TIMEOUT);
}

// ------------------------------------------------------------------ swap
// After a fused update: the spare buffer holds the new scalar; exchange it
// with the current one (pointers and tensor-map slots) in every member's table.
__global__ void k_swap_species(Mem* mems, int nmem) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem) return;
  Mem& M = mems[m];
  for (int s = 0; s < M.nsp; ++s) {
    float* t = M.q[s];
    M.q[s] = M.qa[s];
    M.qa[s] = t;
    const int tm = M.qmap[s];
    M.qmap[s] = M.qamap[s];
    M.qamap[s] = tm;
  }
}

template <typename K>
static void set_smem(K kernel, size_t bytes) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
void launch_scalar_adv_update(const TileLaunch& L, int nblocks, int rk_step, cudaStream_t s, int var, bool sct,
                              unsigned pairs) {
  static bool attr = false;
  if (!attr) {
    set_smem(k_scalar_adv_update<2, false>, ADV_SMEM);
    set_smem(k_scalar_adv_update<3, false>, ADV_SMEM);
    set_smem(k_scalar_adv_update<4, false>, ADV_SMEM);
    set_smem(k_scalar_adv_update<3, true>, ADV_SMEM);
    attr = true;
  }
  const int minb = TUNE_PARAM[TU_ADV][var];
  if (sct) k_scalar_adv_update<3, true><<<nblocks, dim3(TX, TY), ADV_SMEM, s>>>(L, rk_step, pairs);
  else if (minb == 2) k_scalar_adv_update<2, false><<<nblocks, dim3(TX, TY), ADV_SMEM, s>>>(L, rk_step, pairs);
  else if (minb == 3) k_scalar_adv_update<3, false><<<nblocks, dim3(TX, TY), ADV_SMEM, s>>>(L, rk_step, pairs);
  else k_scalar_adv_update<4, false><<<nblocks, dim3(TX, TY), ADV_SMEM, s>>>(L, rk_step, pairs);
}
void launch_scalar_pd_update(const TileLaunch& L, int nblocks, int nlev_max, int rk_step, cudaStream_t s, int var) {
  static size_t attr = 0;
  const size_t bytes = PD_SMEM + sizeof(LevelConst) * (size_t)nlev_max;
  if (bytes > attr) {
    set_smem(k_scalar_pd_update<1>, bytes);
    set_smem(k_scalar_pd_update<2>, bytes);
    attr = bytes;
  }
  if (TUNE_PARAM[TU_PD][var] == 1) k_scalar_pd_update<1><<<nblocks, PD_THREADS, bytes, s>>>(L, rk_step);
  else k_scalar_pd_update<2><<<nblocks, PD_THREADS, bytes, s>>>(L, rk_step);
}
void launch_pd_courant(const Launch& L2, int nblocks, int rk_step, cudaStream_t s) {
  k_pd_courant<<<nblocks, dim3(BX, BY), 0, s>>>(L2, rk_step);
}
void launch_swap_species(Mem* d_mems, int nmem, cudaStream_t s) {
  k_swap_species<<<(nmem + 63) / 64, 64, 0, s>>>(d_mems, nmem);
}

}  // namespace wrfgpu
