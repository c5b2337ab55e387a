// The forward-in-time tendencies of the first RK stage: explicit diffusion
// with constant coefficients (diff_opt = 1, km_opt = 1: horizontal_diffusion,
// horizontal_diffusion_3dmp and the vertical_diffusion family,
// dyn_em/module_big_step_utilities_em.F:2715-3581, called from rk_tendency's
// forward step, dyn_em/module_em.F:801-877, and from rk_scalar_tend,
// :1378-1419), sixth-order numerical diffusion (sixth_order_diffusion,
// :6220-6636, module_em.F:879-932 and 1421-1435) and the Rayleigh damping
// toward the base state (damp_opt = 2); and the addition of those
// tendencies to the large-step tendencies at every stage (rk_addtend_dry,
// dyn_em/module_em.F:959-1092).
//
// The diffusions are point kernels over (i, j) x level blocks: every point
// forms its explicit and sixth-order terms in the reference's order and
// writes its stored tendency once (a vertical flux divergence reads the two
// fluxes around the level, each formed from its own two levels).  They run
// once per large step on inputs that L2 holds for their stencils; the
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

// ---- explicit diffusion (diff_opt = 1) with constant coefficients (km_opt = 1:
// isotropic_km, module_diffusion_em.F:1717-1775, sets xkmh = khdif and
// xkhh = khdif / prandtl everywhere, so each coefficient array access below is
// that one value xk).

constexpr float PRANDTL = 1.f / 3.0f;  // module_model_constants.F:86

// horizontal_diffusion (module_big_step_utilities_em.F:2715-2950) of variable
// kind V at (i, k, j) with mass mu, level coefficients c1, c2 and coefficient
// xk; with `base`, horizontal_diffusion_3dmp (:2953-3060), the field minus
// its 3-D base state.  Returns the term the reference adds to the tendency.
template <int V>
__device__ float hdiff_point(const Mem& m, const F3& f, const F3* base, const F2& mu, float c1, float c2, int i, int k,
                             int j, float xk) {
  const F2 msfux = f2(m, WRFGPU_MSFUX), msfuy = f2(m, WRFGPU_MSFUY), msfvx = f2(m, WRFGPU_MSFVX),
           msfvx_inv = f2(m, WRFGPU_MSFVX_INV), msfvy = f2(m, WRFGPU_MSFVY), msftx = f2(m, WRFGPU_MSFTX),
           msfty = f2(m, WRFGPU_MSFTY);
  const float rdx = m.rdx, rdy = m.rdy;
  auto M = [&](int ii, int jj) { return c1 * mu.ro(ii, jj) + c2; };
  float mkrdxm, mkrdxp, mrdx, mkrdym, mkrdyp, mrdy;
  if (V == DV_U) {  // :2801-2814
    mkrdxm = (msftx.ro(i - 1, j) / msfty.ro(i - 1, j)) * M(i - 1, j) * xk * rdx;
    mkrdxp = (msftx.ro(i, j) / msfty.ro(i, j)) * M(i, j) * xk * rdx;
    mrdx = msfux.ro(i, j) * msfuy.ro(i, j) * rdx;
    mkrdym = ((msfuy.ro(i, j) + msfuy.ro(i, j - 1)) / (msfux.ro(i, j) + msfux.ro(i, j - 1))) * 0.25f *
             (M(i, j) + M(i, j - 1) + M(i - 1, j - 1) + M(i - 1, j)) * 0.25f * (xk + xk + xk + xk) * rdy;
    mkrdyp = ((msfuy.ro(i, j) + msfuy.ro(i, j + 1)) / (msfux.ro(i, j) + msfux.ro(i, j + 1))) * 0.25f *
             (M(i, j) + M(i, j + 1) + M(i - 1, j + 1) + M(i - 1, j)) * 0.25f * (xk + xk + xk + xk) * rdy;
    mrdy = msfux.ro(i, j) * msfuy.ro(i, j) * rdy;
  } else if (V == DV_V) {  // :2847-2856 (the y coefficients carry no mass there)
    mkrdxm = ((msfvx.ro(i, j) + msfvx.ro(i - 1, j)) / (msfvy.ro(i, j) + msfvy.ro(i - 1, j))) * 0.25f *
             (M(i, j) + M(i, j - 1) + M(i - 1, j - 1) + M(i - 1, j)) * 0.25f * (xk + xk + xk + xk) * rdx;
    mkrdxp = ((msfvx.ro(i, j) + msfvx.ro(i + 1, j)) / (msfvy.ro(i, j) + msfvy.ro(i + 1, j))) * 0.25f *
             (M(i, j) + M(i, j - 1) + M(i + 1, j - 1) + M(i + 1, j)) * 0.25f * (xk + xk + xk + xk) * rdx;
    mrdx = msfvx.ro(i, j) * msfvy.ro(i, j) * rdx;
    mkrdym = (msfty.ro(i, j - 1) / msftx.ro(i, j - 1)) * xk * rdy;
    mkrdyp = (msfty.ro(i, j) / msftx.ro(i, j)) * xk * rdy;
    mrdy = msfvx.ro(i, j) * msfvy.ro(i, j) * rdy;
  } else if (V == DV_W) {  // :2885-2900
    mkrdxm = (msfux.ro(i, j) / msfuy.ro(i, j)) * 0.25f * (M(i, j) + M(i - 1, j) + M(i, j) + M(i - 1, j)) * 0.25f *
             (xk + xk + xk + xk) * rdx;
    mkrdxp = (msfux.ro(i + 1, j) / msfuy.ro(i + 1, j)) * 0.25f * (M(i + 1, j) + M(i, j) + M(i + 1, j) + M(i, j)) *
             0.25f * (xk + xk + xk + xk) * rdx;
    mrdx = msftx.ro(i, j) * msfty.ro(i, j) * rdx;
    mkrdym = (msfvy.ro(i, j) * msfvx_inv.ro(i, j)) * 0.25f * (M(i, j) + M(i, j - 1) + M(i, j) + M(i, j - 1)) *
             0.25f * (xk + xk + xk + xk) * rdy;
    mkrdyp = (msfvy.ro(i, j + 1) * msfvx_inv.ro(i, j + 1)) * 0.25f *
             (M(i, j + 1) + M(i, j) + M(i, j + 1) + M(i, j)) * 0.25f * (xk + xk + xk + xk) * rdy;
    mrdy = msftx.ro(i, j) * msfty.ro(i, j) * rdy;
  } else {  // mass points: :2930-2937, :3030-3037
    mkrdxm = (msfux.ro(i, j) / msfuy.ro(i, j)) * 0.5f * (xk + xk) * 0.5f * (M(i, j) + M(i - 1, j)) * rdx;
    mkrdxp = (msfux.ro(i + 1, j) / msfuy.ro(i + 1, j)) * 0.5f * (xk + xk) * 0.5f * (M(i + 1, j) + M(i, j)) * rdx;
    mrdx = msftx.ro(i, j) * msfty.ro(i, j) * rdx;
    mkrdym = (msfvy.ro(i, j) * msfvx_inv.ro(i, j)) * 0.5f * (xk + xk) * 0.5f * (M(i, j) + M(i, j - 1)) * rdy;
    mkrdyp = (msfvy.ro(i, j + 1) * msfvx_inv.ro(i, j + 1)) * 0.5f * (xk + xk) * 0.5f * (M(i, j + 1) + M(i, j)) * rdy;
    mrdy = msftx.ro(i, j) * msfty.ro(i, j) * rdy;
  }
  const float q0 = f.ro(i, k, j);
  float dxp = f.ro(i + 1, k, j) - q0, dxm = q0 - f.ro(i - 1, k, j);
  float dyp = f.ro(i, k, j + 1) - q0, dym = q0 - f.ro(i, k, j - 1);
  if (base) {  // field(+1) - field(0) - base(+1) + base(0), and so on
    const F3& b = *base;
    const float b0 = b.ro(i, k, j);
    dxp = dxp - b.ro(i + 1, k, j) + b0;
    dxm = dxm - b0 + b.ro(i - 1, k, j);
    dyp = dyp - b.ro(i, k, j + 1) + b0;
    dym = dym - b0 + b.ro(i, k, j - 1);
  }
  return mrdx * (mkrdxp * dxp - mkrdxm * dxm) + mrdy * (mkrdyp * dyp - mkrdym * dym);
}

// Vertical diffusion kinds: vertical_diffusion_u / _v (the wind minus its 1-D
// base profile; module_big_step_utilities_em.F:3382-3581), vertical_diffusion
// 'w' and 'm' (:3064-3187), vertical_diffusion_mp (a 1-D base profile, qv;
// :3192-3281) and vertical_diffusion_3dmp (a 3-D base state, theta;
// :3286-3376).
enum { VD_U = 0, VD_V = 1, VD_W = 2, VD_M = 3, VD_MP = 4, VD_3DMP = 5 };

// The vertical flux vflux(i, kk) (levels kts..ktf-1) of kind V.
template <int V>
__device__ __forceinline__ float vflux_at(const Mem& m, const F3& f, const F1& b1, const F3* b3, const F3& alt, int i,
                                          int kk, int j, float kvdif) {
  const F1 rdn = f1(m, WRFGPU_RDN);
  const float df = f.ro(i, kk + 1, j) - f.ro(i, kk, j);
  if (V == VD_W) return (kvdif / alt.ro(i, kk, j)) * f1(m, WRFGPU_RDNW)(kk) * df;
  if (V == VD_U)
    return kvdif * rdn(kk + 1) /
           (0.25f * (alt.ro(i, kk, j) + alt.ro(i - 1, kk, j) + alt.ro(i, kk + 1, j) + alt.ro(i - 1, kk + 1, j))) *
           (df - b1(kk + 1) + b1(kk));
  if (V == VD_V)
    return kvdif * rdn(kk + 1) /
           (0.25f * (alt.ro(i, kk, j) + alt.ro(i, kk, j - 1) + alt.ro(i, kk + 1, j) + alt.ro(i, kk + 1, j - 1))) *
           (df - b1(kk + 1) + b1(kk));
  const float a = kvdif * rdn(kk + 1) / (0.5f * (alt.ro(i, kk, j) + alt.ro(i, kk + 1, j)));
  if (V == VD_M) return a * df;
  if (V == VD_MP) return a * (df - b1(kk + 1) + b1(kk));
  return a * (df - b3->ro(i, kk + 1, j) + b3->ro(i, kk, j));
}

// The term vertical diffusion of kind V adds to the tendency at level k,
// with the column mass c1 mass + c2 of that level: the divergence of the
// fluxes vflux(k) - vflux(k-1), vflux(kts-1) = vflux(kts), vflux(ktf) = 0.
template <int V>
__device__ float vdiff_point(const Mem& m, const F3& f, const F1& b1, const F3* b3, float mass, float c1, float c2,
                             int i, int k, int j, float kvdif) {
  const F3 alt = f3(m, WRFGPU_ALT);
  const int kts = m.kts, ktf = min(m.kte, m.kde - 1);
  auto vf = [&](int kk) { return kk >= ktf ? 0.f : vflux_at<V>(m, f, b1, b3, alt, i, max(kk, kts), j, kvdif); };
  const float dv = vf(k) - vf(k - 1);
  const float g2 = G * G;
  if (V == VD_U) return g2 * f1(m, WRFGPU_RDNW)(k) / (c1 * mass + c2) / (0.5f * (alt.ro(i - 1, k, j) + alt.ro(i, k, j))) * dv;
  if (V == VD_V) return g2 * f1(m, WRFGPU_RDNW)(k) / (c1 * mass + c2) / (0.5f * (alt.ro(i, k, j - 1) + alt.ro(i, k, j))) * dv;
  if (V == VD_W)
    return f1(m, WRFGPU_RDN)(k) * G * G / (c1 * mass + c2) / (0.5f * (alt.ro(i, k, j) + alt.ro(i, k - 1, j))) * dv;
  return g2 / (c1 * mass + c2) / alt.ro(i, k, j) * f1(m, WRFGPU_RDNW)(k) * dv;
}

// Point ranges of the diffusion terms next to open boundaries (a periodic x
// keeps its ranges): horizontal_diffusion (module_big_step_utilities_em.F:
// 2786-2790 u, :2834-2839 v, :2874-2879 w, :2919-2924 and :3026-3031 mass
// points), vertical_diffusion_u / _v (:3443-3446, :3545-3546; the other
// kinds have none) and sixth_order_diffusion (:6336-6443).
__device__ __forceinline__ bool hdiff_open_in(const Mem& m, int V, int i, int j) {
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const bool x = m.cf.periodic_x || ((!oxs || i >= m.ids + 1) && (!oxe || i <= (V == DV_U ? m.ide - 1 : m.ide - 2)));
  return x && (!oys || j >= m.jds + 1) && (!oye || j <= (V == DV_V ? m.jde - 1 : m.jde - 2));
}
__device__ __forceinline__ bool vdiff_open_in(const Mem& m, int V, int i, int j) {
  if (V == VD_U) return m.cf.periodic_x || ((!m.cf.open_xs || i >= m.ids + 1) && (!m.cf.open_xe || i <= m.ide - 1));
  if (V == VD_V) return (!m.cf.open_ys || j >= m.jds + 1) && (!m.cf.open_ye || j <= m.jde - 1);
  return true;
}
__device__ __forceinline__ bool diff6_open_in(const Mem& m, int V, int i, int j) {
  const bool oxs = m.cf.open_xs, oxe = m.cf.open_xe, oys = m.cf.open_ys, oye = m.cf.open_ye;
  const int ids = m.ids, ide = m.ide, jds = m.jds, jde = m.jde;
  if (V == DV_V && oxs)  // :6383-6388: all four limits on open_xs
    return i >= ids + 3 && i <= ide - 4 && j >= jds + 3 && j <= jde - 3;
  const int xe = V == DV_U ? ide - 3 : ide - 4, ye = V == DV_V ? jde - 3 : jde - 4;
  return (!oxs || i >= ids + 3) && (!oxe || i <= xe) && (!oys || j >= jds + 3) && (!oye || j <= ye);
}

// Stage 1, mode 0 (rk_tendency): the forward-in-time tendencies ru_tendf,
// rv_tendf, rw_tendf and t_tendf of u_2, v_2, w_2 and t_2: the explicit
// diffusion (diff_opt = 1; mut, khdif, kvdif), then the sixth-order diffusion
// (mut, the large step dt).  Mode 1 (rk_scalar_tend, after the acoustic
// steps): each diffused species' sc_tend, with muts, khdif / prandtl,
// kvdif / prandtl and the stage's dt (dt / 3); qv (species 0) diffuses
// vertically against its base profile qv_base.  Loop limits of :2760-2790,
// :3100-3130, :6330-6443 (open boundaries: each term its own, above);
// points outside them get no term.  Mode 2 is mode 0 added
// onto the stored tendencies' values (the routine-level rk_tendency, whose
// *_tendf arrays arrive holding the physics tendencies).
__global__ void __launch_bounds__(BX* BY) k_forward_diff(Launch L, int mode) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  const bool d1 = m.cf.diff_opt == 1, d6 = m.cf.diff_6th_opt != 0;
  if (!bp.valid || m.tendf[0] == nullptr || !(d1 || d6)) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  const int ktf = min(m.kte, m.kde - 1);
  if (i < m.its || j < m.jts || k < m.kts || k > ktf) return;
  const int i_end = min(m.ide - 1, m.ite), j_end = min(m.jde - 1, m.jte);
  const F1 c1h = f1(m, WRFGPU_C1H), c2h = f1(m, WRFGPU_C2H);
  const float c1 = c1h(k), c2 = c2h(k);
  if (mode == 1) {
    if (i > i_end || j > j_end) return;
    const float coef = m.cf.diff_6th_factor * 0.015625f / (2.0f * stage_of(m, 1).dt_rk);
    const float khdq = m.cf.khdif / PRANDTL, kvdq = m.cf.kvdif / PRANDTL;
    const F2 muts = f2(m, WRFGPU_MUTS);
    const F1 qvb = f1(m, WRFGPU_QV_BASE);
    for (int s = 0; s < m.nsp; ++s) {
      float* sc = sc_tend_of(m, s);
      if (!sc) continue;
      const F3 q = f3p(m, m.q[s]);
      float t = 0.f;
      if (mix2_on(m, s)) {
        if (hdiff_open_in(m, DV_M, i, j)) t = t + hdiff_point<DV_M>(m, q, nullptr, muts, c1, c2, i, k, j, khdq);
        const float mu = muts.ro(i, j);
        t = t + (s == 0 ? vdiff_point<VD_MP>(m, q, qvb, nullptr, mu, c1, c2, i, k, j, kvdq)
                        : vdiff_point<VD_M>(m, q, qvb, nullptr, mu, c1, c2, i, k, j, kvdq));
      }
      if (mix6_on(m, s) && diff6_open_in(m, DV_M, i, j)) t = diff6_point<DV_M>(m, q, muts, i, k, j, c1, c2, coef, t);
      f3p(m, sc)(i, k, j) = t;
    }
    return;
  }
  const float coef = m.cf.diff_6th_factor * 0.015625f / (2.0f * m.dt);
  const float xkmh = m.cf.khdif, xkhh = m.cf.khdif / PRANDTL, kvdif = m.cf.kvdif;
  const F2 mut = f2(m, WRFGPU_MUT);
  const bool acc = mode == 2;  // onto the stored values (the routine-level form: physics tendencies)
  if (i <= m.ite && j <= j_end) {
    const F3 u = f3(m, WRFGPU_U_2);
    float t = acc ? f3p(m, m.tendf[0])(i, k, j) : 0.f;
    if (d1) {
      if (hdiff_open_in(m, DV_U, i, j)) t = t + hdiff_point<DV_U>(m, u, nullptr, mut, c1, c2, i, k, j, xkmh);
      if (k <= ktf - 1 && vdiff_open_in(m, VD_U, i, j))
        t = t + vdiff_point<VD_U>(m, u, f1(m, WRFGPU_U_BASE), nullptr, f2(m, WRFGPU_MUU).ro(i, j), c1, c2, i, k, j,
                                  kvdif);
    }
    if (d6 && diff6_open_in(m, DV_U, i, j)) t = diff6_point<DV_U>(m, u, mut, i, k, j, c1, c2, coef, t);
    f3p(m, m.tendf[0])(i, k, j) = t;
  }
  if (i <= i_end && j <= m.jte) {
    const F3 v = f3(m, WRFGPU_V_2);
    float t = acc ? f3p(m, m.tendf[1])(i, k, j) : 0.f;
    if (d1) {
      if (hdiff_open_in(m, DV_V, i, j)) t = t + hdiff_point<DV_V>(m, v, nullptr, mut, c1, c2, i, k, j, xkmh);
      if (k <= ktf - 1 && j <= j_end && vdiff_open_in(m, VD_V, i, j))
        t = t + vdiff_point<VD_V>(m, v, f1(m, WRFGPU_V_BASE), nullptr, f2(m, WRFGPU_MUV).ro(i, j), c1, c2, i, k, j,
                                  kvdif);
    }
    if (d6 && diff6_open_in(m, DV_V, i, j)) t = diff6_point<DV_V>(m, v, mut, i, k, j, c1, c2, coef, t);
    f3p(m, m.tendf[1])(i, k, j) = t;
  }
  if (i <= i_end && j <= j_end) {
    const float mt = mut.ro(i, j);
    if (k >= m.kts + 1) {
      const F3 w = f3(m, WRFGPU_W_2);
      const float c1w = f1(m, WRFGPU_C1F)(k), c2w = f1(m, WRFGPU_C2F)(k);
      float t = acc ? f3p(m, m.tendf[2])(i, k, j) : 0.f;
      if (d1) {
        if (hdiff_open_in(m, DV_W, i, j)) t = t + hdiff_point<DV_W>(m, w, nullptr, mut, c1w, c2w, i, k, j, xkmh);
        t = t + vdiff_point<VD_W>(m, w, c1h, nullptr, mt, c1w, c2w, i, k, j, kvdif);
      }
      if (d6 && diff6_open_in(m, DV_W, i, j)) t = diff6_point<DV_W>(m, w, mut, i, k, j, c1w, c2w, coef, t);
      f3p(m, m.tendf[2])(i, k, j) = t;
    }
    const F3 th = f3(m, WRFGPU_T_2), tb = f3(m, WRFGPU_T_INIT);
    float t = acc ? f3p(m, m.tendf[3])(i, k, j) : 0.f;
    if (d1) {
      if (hdiff_open_in(m, DV_M, i, j)) t = t + hdiff_point<DV_M>(m, th, &tb, mut, c1, c2, i, k, j, xkhh);
      t = t + vdiff_point<VD_3DMP>(m, th, c1h, &tb, mt, c1, c2, i, k, j, 3.f * kvdif);
    }
    if (d6 && diff6_open_in(m, DV_M, i, j)) t = diff6_point<DV_M>(m, th, mut, i, k, j, c1, c2, coef, t);
    f3p(m, m.tendf[3])(i, k, j) = t;
  }
}

// The routine-level form of rk_scalar_tend's stage-1 diffusion of one species
// (module_em.F:1378-1435): species 0 of a scratch domain, its explicit
// diffusion (diff_opt = 1 and mix2 on; qv: vertical_diffusion_mp against
// qv_base) and then its sixth-order diffusion (diff_6th_opt != 0 and mix6 on)
// accumulated into the caller's scalar_tends, carried in the H_DIABATIC
// buffer, with mut (MUTS) and the caller's dt_step.
__global__ void __launch_bounds__(BX* BY) k_species_diff_routine(Launch L, int qv) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  const int ktf = min(m.kte, m.kde - 1);
  if (i < m.its || j < m.jts || k < m.kts || k > ktf) return;
  if (i > min(m.ide - 1, m.ite) || j > min(m.jde - 1, m.jte)) return;
  const float c1 = f1(m, WRFGPU_C1H)(k), c2 = f1(m, WRFGPU_C2H)(k);
  const F2 muts = f2(m, WRFGPU_MUTS);
  const F3 q = f3p(m, m.q[0]);
  F3 out = f3(m, WRFGPU_H_DIABATIC);
  float t = out(i, k, j);
  if (mix2_on(m, 0)) {
    const float kvdq = m.cf.kvdif / PRANDTL;
    if (hdiff_open_in(m, DV_M, i, j)) t = t + hdiff_point<DV_M>(m, q, nullptr, muts, c1, c2, i, k, j, m.cf.khdif / PRANDTL);
    const F1 qvb = f1(m, WRFGPU_QV_BASE);
    t = t + (qv ? vdiff_point<VD_MP>(m, q, qvb, nullptr, muts.ro(i, j), c1, c2, i, k, j, kvdq)
                : vdiff_point<VD_M>(m, q, qvb, nullptr, muts.ro(i, j), c1, c2, i, k, j, kvdq));
  }
  if (mix6_on(m, 0) && diff6_open_in(m, DV_M, i, j)) {
    const float coef = m.cf.diff_6th_factor * 0.015625f / (2.0f * stage_of(m, 1).dt_rk);
    t = diff6_point<DV_M>(m, q, muts, i, k, j, c1, c2, coef, t);
  }
  out(i, k, j) = t;
}

// Stage 1, damp_opt = 2: rk_rayleigh_damp (module_big_step_utilities_em.F:
// 5836-6110), relaxation of u, v, w and theta toward the base-state
// profiles in the top zdamp metres, into ru_tendf .. t_tendf.  One thread per
// column (i, j) of the memory extent, handling u, v, w and theta of that
// column; the top layer's level heights are formed again where they are
// used (the same expressions, so the same bits) instead of being stored.
// A member that also stores the explicit or sixth-order diffusion
// accumulates onto it (written earlier in the same stage), as does the
// routine-level form (acc_all: onto the caller's tendencies); otherwise every level of the loop
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
__global__ void __launch_bounds__(BX* BY) k_rayleigh_damp(Launch L, bool acc_all) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid || m.cf.damp_opt != 2 || m.tendf[0] == nullptr) return;
  const int i = bp.i, j = bp.j;
  if (i < m.its || j < m.jts) return;
  const int kts = m.kts, ktf = min(m.kte, m.kde - 1), kde = m.kde;
  const bool acc = acc_all || m.cf.diff_6th_opt != 0 || m.cf.diff_opt == 1;
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

// The routine-level form of rk_addtend_dry (module_em.F:959-1092), every
// term of the reference: at stage 1 the saved tendencies join the forward
// ones (ru_tendf += u_save msfuy, ..., ph_tendf += ph_save, t_tendf +=
// t_save), and every stage adds them to the large-step tendencies with
// theta's h_diabatic term; mu_tend += mu_tendf.  ph_tendf is carried in the
// ADVECT_TEND buffer and mu_tendf in MUDF.
__global__ void __launch_bounds__(BX* BY) k_addtend_dry_routine(Launch L, int rk_step) {
  BlockPos bp = block_pos(L);
  const Mem& m = block_member(L.mem, bp.m);
  if (!bp.valid || m.tendf[0] == nullptr) return;
  const int i = bp.i, j = bp.j, k = bp.k;
  if (i < m.its || j < m.jts || k < m.kts || k > m.kte) return;
  const int i_end = min(m.ite, m.ide - 1), j_end = min(m.jte, m.jde - 1);
  const bool s1 = rk_step == 1;
  const F2 msfuy = f2(m, WRFGPU_MSFUY), msfvx = f2(m, WRFGPU_MSFVX), msfvx_inv = f2(m, WRFGPU_MSFVX_INV),
           msfty = f2(m, WRFGPU_MSFTY);
  if (k <= m.kte - 1 && i <= m.ite && j <= j_end) {
    F3 f = f3p(m, m.tendf[0]), t = f3(m, WRFGPU_RU_TEND);
    if (s1) f(i, k, j) = f(i, k, j) + f3(m, WRFGPU_U_SAVE)(i, k, j) * msfuy(i, j);
    t(i, k, j) = t(i, k, j) + f(i, k, j) / msfuy(i, j);
  }
  if (k <= m.kte - 1 && i <= i_end && j <= m.jte) {
    F3 f = f3p(m, m.tendf[1]), t = f3(m, WRFGPU_RV_TEND);
    if (s1) f(i, k, j) = f(i, k, j) + f3(m, WRFGPU_V_SAVE)(i, k, j) * msfvx(i, j);
    t(i, k, j) = t(i, k, j) + f(i, k, j) * msfvx_inv(i, j);
  }
  if (i <= i_end && j <= j_end) {
    F3 f = f3p(m, m.tendf[2]), t = f3(m, WRFGPU_RW_TEND);
    if (s1) f(i, k, j) = f(i, k, j) + f3(m, WRFGPU_W_SAVE)(i, k, j) * msfty(i, j);
    t(i, k, j) = t(i, k, j) + f(i, k, j) / msfty(i, j);
    F3 pf = f3(m, WRFGPU_ADVECT_TEND), pt = f3(m, WRFGPU_PH_TEND);
    if (s1) pf(i, k, j) = pf(i, k, j) + f3(m, WRFGPU_PH_SAVE)(i, k, j);
    pt(i, k, j) = pt(i, k, j) + pf(i, k, j) / msfty(i, j);
    if (k <= m.kte - 1) {
      F3 tf = f3p(m, m.tendf[3]), tt = f3(m, WRFGPU_T_TEND);
      if (s1) tf(i, k, j) = tf(i, k, j) + f3(m, WRFGPU_T_SAVE)(i, k, j);
      const float mass = f1(m, WRFGPU_C1H)(k) * f2(m, WRFGPU_MUT)(i, j) + f1(m, WRFGPU_C2H)(k);
      tt(i, k, j) = tt(i, k, j) + tf(i, k, j) / msfty(i, j) + mass * f3(m, WRFGPU_H_DIABATIC)(i, k, j) / msfty(i, j);
    }
    if (k == m.kts) {
      F2 mt = f2(m, WRFGPU_MU_TEND);
      mt(i, j) = mt(i, j) + f2(m, WRFGPU_MUDF)(i, j);
    }
  }
}

}  // namespace

void launch_addtend_dry_routine(const Launch& L, int nblocks, int rk_step, cudaStream_t s) {
  k_addtend_dry_routine<<<nblocks, dim3(BX, BY), 0, s>>>(L, rk_step);
}

void launch_forward_diff(const Launch& L, int nblocks, int mode, cudaStream_t s) {
  k_forward_diff<<<nblocks, dim3(BX, BY), 0, s>>>(L, mode);
}

void launch_species_diff_routine(const Launch& L, int nblocks, int qv, cudaStream_t s) {
  k_species_diff_routine<<<nblocks, dim3(BX, BY), 0, s>>>(L, qv);
}

void launch_rayleigh_damp(const Launch& L2, int nblocks, cudaStream_t s, bool acc_all) {
  k_rayleigh_damp<<<nblocks, dim3(BX, BY), 0, s>>>(L2, acc_all);
}

void launch_addtend_dry(const Launch& L, int nblocks, cudaStream_t s) {
  k_addtend_dry<<<nblocks, dim3(BX, BY), 0, s>>>(L);
}

}  // namespace wrfgpu
