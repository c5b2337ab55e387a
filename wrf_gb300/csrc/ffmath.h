// Correctly rounded single-precision log and pow for the equation of state.
//
// Fast path: float-float ("double-float") arithmetic on FP32 units, built on
// Dekker's error-free transformations (TwoSum, and TwoProduct with a fused
// multiply-add), with table-driven reductions in the manner of Tang
// ("Table-driven implementation of the logarithm / exponential function",
// ACM TOMS 1989/1990):
//   log x = E log 2 + T_j + log1p(r),  r = m rc_j - 1 exactly, |r| < 2^-8,
//           T_j = -log(rc_j) (128 entries), log1p to r^6;
//   exp z = 2^k 2^(j/64) exp(r),  r = z - (64k + j) log2/64, |r| < 2^-7,
//           exp(r) to r^5;
// the tables are in ffmath_tables.h (gen_ffmath_tables.py, 50-digit decimal
// arithmetic).  Relative error below 1e-13 for log and pow (measured by
// tests/native/ffmath_check.cpp against long double).
// Rounding test (Ziv's strategy): the float-float result hi + lo rounds to hi
// unless |lo| sits within 1e-12 |hi| of half an ulp of hi; only then is the
// value recomputed in FP64 with the CUDA / libm double functions and rounded
// once (~1e-5 of the inputs).
//
// They replace the libm calls of calc_p_rho_phi (the reference's LOG and
// x**cpovcv through vspow, frame/libmassv.F:383), so that the GPU rounds
// like a correctly rounded libm.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#ifdef __CUDACC__
#define FFM_HD __host__ __device__ __forceinline__
#else
#define FFM_HD inline
#endif
#include "ffmath_tables.h"

namespace wrfgpu_ff {

struct ff { float hi, lo; };

FFM_HD float fmaf_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
FFM_HD float frexpf_(float x, int* e) {
#ifdef __CUDA_ARCH__
  return frexpf(x, e);
#else
  return std::frexp(x, e);
#endif
}
FFM_HD float ldexpf_(float x, int e) {
#ifdef __CUDA_ARCH__
  return ldexpf(x, e);
#else
  return std::ldexp(x, e);
#endif
}
FFM_HD float rintf_(float x) {
#ifdef __CUDA_ARCH__
  return rintf(x);
#else
  return std::nearbyint(x);
#endif
}

FFM_HD ff two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
FFM_HD ff fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = a + b;
  return {s, b - (s - a)};
}
FFM_HD ff two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf_(a, b, -p)};
}
FFM_HD ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  ff t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
FFM_HD ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  float e = p.lo + (a.hi * b.lo + a.lo * b.hi);
  return fast_two_sum(p.hi, e);
}
FFM_HD ff ff_mulf(ff a, float b) {
  ff p = two_prod(a.hi, b);
  float e = p.lo + a.lo * b;
  return fast_two_sum(p.hi, e);
}

// tables: global memory on the device (read through the non-coherent cache),
// ordinary arrays on the host
#ifdef __CUDACC__
static __device__ __align__(16) const float LOG_TAB_DEV[128][4] = WRFGPU_FF_LOG_TAB;
static __device__ __align__(8) const float EXP_TAB_DEV[64][2] = WRFGPU_FF_EXP_TAB;
#endif
static const float LOG_TAB_HOST[128][4] = WRFGPU_FF_LOG_TAB;
static const float EXP_TAB_HOST[64][2] = WRFGPU_FF_EXP_TAB;

FFM_HD uint32_t f2u(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u; std::memcpy(&u, &x, 4); return u;
#endif
}
FFM_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x; std::memcpy(&x, &u, 4); return x;
#endif
}
// hi + lo with |lo| small: add one float
FFM_HD ff ff_addf(ff a, float b) {
  ff s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}

// log x for a positive normal float, as a float pair
FFM_HD ff ff_log_t(float x) {
  const uint32_t b = f2u(x);
  int e = (int)(b >> 23) - 127;
  const int j = (int)((b >> 16) & 127u);
  const float m = u2f((b & 0x007FFFFFu) | 0x3F800000u);  // [1, 2)
#ifdef __CUDA_ARCH__
  const float4 t = __ldg(reinterpret_cast<const float4*>(LOG_TAB_DEV[j]));
  const float rc = t.x, th = t.y, tl = t.z;
#else
  const float rc = LOG_TAB_HOST[j][0], th = LOG_TAB_HOST[j][1], tl = LOG_TAB_HOST[j][2];
#endif
  if (j >= 64) e += 1;  // m in [1.5, 2) counts as m/2 (the table holds -log(rc) - log 2)
  // r = m rc - 1 exactly: m rc = p.hi + p.lo, p.hi - 1 exact (p.hi near 1)
  const ff p = two_prod(m, rc);
  const ff r = two_sum(p.hi - 1.f, p.lo);
  // log1p(r) = r - r^2/2 + r^3/3 + r^4 (-1/4 + r/5 - r^2/6) + O(r^7): the
  // terms through r^3 in float-float (r^3/3 is ~r^2/3 of the result, so its
  // float rounding alone would cost up to 1e-12), the rest in float
  const float rh = r.hi;
  ff r2 = two_prod(rh, rh);
  r2.lo += 2.f * rh * r.lo;
  ff r3 = ff_mulf(r2, rh);
  r3.lo += rh * (rh * r.lo);
  const ff t3 = ff_mul(r3, ff{THIRD_HI, THIRD_LO});
  const float r4 = r2.hi * r2.hi;
  const float d4 = r4 * (-0.25f + rh * (0.2f - rh * (1.f / 6.f)));
  ff l = ff_add(r, ff{-0.5f * r2.hi, -0.5f * r2.lo});
  l = ff_add(l, t3);
  l = ff_addf(l, d4);
  l = ff_add(ff{th, tl}, l);
  if (e != 0) {
    const float ef = (float)e;
    const float h = ef * LN2F_HI;
    const ff el = fast_two_sum(h, fmaf_(ef, LN2F_HI, -h) + ef * LN2F_LO);
    l = ff_add(el, l);
  }
  return l;
}

// exp z for |z| < ~80, as 2^k times a float pair in [0.7, 1.5)
FFM_HD ff ff_exp_t(ff z, int* k) {
  const float nf = rintf_(z.hi * INV_LN2_64);
  const int n = (int)nf;
  // r = z - n log2/64: n * LN2_64_HI is exact (13-bit constant, |n| < 2^11)
  // and so is z.hi minus it (the two are within a factor of two)
  const float a = z.hi - nf * LN2_64_HI;
  const ff bm = two_prod(nf, LN2_64_MID);
  ff r = two_sum(a, -bm.hi);
  r.lo += (z.lo - bm.lo) - nf * LN2_64_LO;
  r = fast_two_sum(r.hi, r.lo);
  // exp(r) - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120) + O(r^6)
  const float rh = r.hi;
  ff r2 = two_prod(rh, rh);
  r2.lo += 2.f * rh * r.lo;
  const float c3 = rh * r2.hi * (1.f / 6.f + rh * (1.f / 24.f + rh * (1.f / 120.f)));
  ff q = ff_add(r, ff{0.5f * r2.hi, 0.5f * r2.lo});
  q = ff_addf(q, c3);
  const ff e1 = ff_add(ff{1.f, 0.f}, q);
  const int j = n & 63;
  *k = n >> 6;  // floor(n / 64)
#ifdef __CUDA_ARCH__
  const float2 t = __ldg(reinterpret_cast<const float2*>(EXP_TAB_DEV[j]));
  return ff_mul(e1, ff{t.x, t.y});
#else
  return ff_mul(e1, ff{EXP_TAB_HOST[j][0], EXP_TAB_HOST[j][1]});
#endif
}

// Ziv's rounding test for a normalised float-float v = hi + lo (|lo| <= ulp(hi)/2)
// known to relative accuracy 1e-13 or better: hi is the correctly rounded value unless
// |lo| lies within 1e-12 |hi| of half an ulp of hi, or hi is a power of two.
FFM_HD bool rounds_safely(ff v) {
  int e;
  const float m = frexpf_(fabsf(v.hi), &e);
  if (m == 0.5f) return false;
  const float half_ulp = ldexpf_(1.f, e - 25);
  return fabsf(fabsf(v.lo) - half_ulp) > 1e-12f * fabsf(v.hi);
}

FFM_HD bool normal_positive(float x) {
  const uint32_t b = f2u(x);
  return b >= 0x00800000u && b < 0x7F800000u;  // positive, normal, finite
}

// log(x) for x > 0, correctly rounded to float.
FFM_HD float logf_cr(float x) {
  if (normal_positive(x)) {
    ff l = ff_log_t(x);
    l = fast_two_sum(l.hi, l.lo);
    if (l.hi != 0.f && rounds_safely(l)) return l.hi;
  }
  return (float)::log((double)x);
}

// x^y for x > 0 (finite, normal result), correctly rounded to float.
FFM_HD float powf_cr(float x, float y) {
  if (normal_positive(x)) {
    const ff z = ff_mulf(ff_log_t(x), y);
    if (fabsf(z.hi) < 80.f) {
      int k = 0;
      ff v = ff_exp_t(z, &k);
      v = fast_two_sum(v.hi, v.lo);
      if (k > -120 && k < 120 && rounds_safely(v)) return ldexpf_(v.hi, k);
    }
  }
  return (float)::pow((double)x, (double)y);
}

// ---------------------------------------------------------------- sin
// Double-double helpers (Dekker / Knuth error-free transformations in FP64).
struct dd { double hi, lo; };
FFM_HD double fma_d(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
FFM_HD dd dd_fast_two_sum(double a, double b) { const double s = a + b; return {s, b - (s - a)}; }
FFM_HD dd dd_add(dd a, dd b) {
  const double s = a.hi + b.hi, bb = s - a.hi, e = (a.hi - (s - bb)) + (b.hi - bb);
  return dd_fast_two_sum(s, e + a.lo + b.lo);
}
FFM_HD dd dd_mul(dd a, dd b) {
  const double p = a.hi * b.hi, e = fma_d(a.hi, b.hi, -p);
  return dd_fast_two_sum(p, e + (a.hi * b.lo + a.lo * b.hi));
}
FFM_HD dd dd_div_d(dd a, double b) {  // a / b, b an exact small integer here
  const double q1 = a.hi / b;
  const double p = q1 * b, pe = fma_d(q1, b, -p);
  const double r = ((a.hi - p) - pe) + a.lo;
  return dd_fast_two_sum(q1, r / b);
}

// sin x for a float |x| <= 2 as a double-double (relative error below
// 2^-95): the Taylor series x - x^3/3! + x^5/5! - ... summed to x^33/33!
// (below 2^-100 of the sum for |x| <= 2).
FFM_HD dd sin_dd_small(double x) {
  const dd x2 = {x * x, 0.0};  // exact: x has 24 significant bits
  dd term = {x, 0.0}, sum = {x, 0.0};
  for (int n = 1; n <= 16; ++n) {
    term = dd_div_d(dd_mul(term, x2), (double)(2 * n) * (double)(2 * n + 1));
    term.hi = -term.hi;
    term.lo = -term.lo;
    sum = dd_add(sum, term);
  }
  return sum;
}

// sin(x) for |x| <= 2, correctly rounded to float.  Fast path: the FP64 sine
// (libm on the host, CUDA's double sin on the device; both within 2 ulp of
// FP64) rounded once, accepted when it lies farther than 2^-45 of its value
// from a float rounding boundary; otherwise the double-double series decides
// (the same code on host and device).  Used by the w Rayleigh damping of
// advance_w (damp_opt = 3), whose argument lies in [0, pi/2].
FFM_HD float sinf_cr(float x) {
  const double d = (double)x;
  const double s = ::sin(d);
  const float f = (float)s;
  const double e = s - (double)f;          // exact
  int ex;
  const float mant = frexpf_(fabsf(f), &ex);
  const double half_ulp = (double)ldexpf_(1.f, ex - 25);
  if (f != 0.f && mant != 0.5f && fabs(fabs(e) - half_ulp) > 0x1p-45 * fabs(s)) return f;
  if (x == 0.f) return x;
  const dd v = sin_dd_small(d);
  // round hi + lo to float: hi's rounding, moved one float step when lo
  // carries the sum past the midpoint with a neighbour (the midpoints of
  // adjacent floats are exact doubles, and hi - midpoint is exact)
  float r = (float)v.hi;
  const double up = 0.5 * ((double)r + (double)nextafterf(r, INFINITY));
  const double dn = 0.5 * ((double)r + (double)nextafterf(r, -INFINITY));
  if ((v.hi - up) + v.lo > 0.0) r = nextafterf(r, INFINITY);
  else if ((v.hi - dn) + v.lo < 0.0) r = nextafterf(r, -INFINITY);
  return r;
}

}  // namespace wrfgpu_ff
