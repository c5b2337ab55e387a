// Correctly rounded single-precision log and pow for the equation of state.
//
// Fast path: float-float ("double-float") arithmetic on FP32 units, built on
// Dekker's error-free transformations (TwoSum, and TwoProduct with a fused
// multiply-add), with truncated Taylor series of atanh (log) and exp after
// the usual reduction exp(z) = 2^n exp(z - n ln2).  Its relative error is a
// few 1e-15, far below half an FP32 ulp (6e-8).
// Rounding test (Ziv's strategy): the float-float result hi + lo rounds to hi
// unless |lo| sits within the error bound of half an ulp of hi; only then is
// the value recomputed in FP64 with the CUDA / libm double functions and
// rounded once.  That happens for ~1e-5 of the inputs.
//
// They replace the libm calls of calc_p_rho_phi (the reference's LOG and
// x**cpovcv through vspow, frame/libmassv.F:383), so that the GPU rounds
// like a correctly rounded libm.
#pragma once
#include <cmath>
#ifdef __CUDACC__
#define FFM_HD __host__ __device__ __forceinline__
#else
#define FFM_HD inline
#endif

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
FFM_HD ff ff_div(ff a, ff b) {  // a / b with two correction steps
  float q1 = a.hi / b.hi;
  ff r = ff_add(a, ff_mulf(ff{-b.hi, -b.lo}, q1));
  float q2 = r.hi / b.hi;
  r = ff_add(r, ff_mulf(ff{-b.hi, -b.lo}, q2));
  float q3 = r.hi / b.hi;
  ff q = fast_two_sum(q1, q2);
  return ff_add(q, ff{q3, 0.f});
}

// ln 2 and 1/n as (nearest float, float remainder) pairs.
constexpr float LN2_HI = 0.6931471824645996f;
constexpr float LN2_LO = -1.9046542121259336e-09f;
constexpr float INV_LN2 = 1.4426950408889634f;
#define WRFGPU_FF(h, l) ff { h##f, l##f }

// natural log of x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(t) = 2t (1 + t^2/3 + t^4/5 + ...), t = (m-1)/(m+1), |t| <= 0.172.
// Terms from t^8 on are summed in float (their float error is < 1e-14 of the
// result); the series is cut after t^18 (truncation < 1e-15).
FFM_HD ff ff_log(float x) {
  int e = 0;
  float m = frexpf_(x, &e);
  if (m < 0.70710678f) { m = m * 2.f; e -= 1; }
  ff num = {m - 1.f, 0.f};  // exact (Sterbenz)
  ff den = two_sum(m, 1.f);
  ff t = ff_div(num, den);
  ff t2 = ff_mul(t, t);
  const float s = t2.hi;
  const float f8 = 1.f / 9.f + s * (1.f / 11.f + s * (1.f / 13.f + s * (1.f / 15.f + s * (1.f / 17.f + s * (1.f / 19.f)))));
  ff a = ff_add(WRFGPU_FF(0.1428571492433548, -6.38621200366174e-09), ff_mulf(t2, f8));  // 1/7 + ...
  a = ff_add(WRFGPU_FF(0.20000000298023224, -2.9802322831784522e-09), ff_mul(t2, a));     // 1/5 + ...
  a = ff_add(WRFGPU_FF(0.3333333432674408, -9.934107758624577e-09), ff_mul(t2, a));      // 1/3 + ...
  a = ff_add(ff{1.f, 0.f}, ff_mul(t2, a));
  ff lm = ff_mul(ff{2.f * t.hi, 2.f * t.lo}, a);
  const float ef = (float)e;
  ff el = ff_add(two_prod(ef, LN2_HI), ff{ef * LN2_LO, 0.f});
  return ff_add(el, lm);
}

// exp(r) for |r| <= ~0.35: Horner in float-float down to the r^6/720 term,
// the r^7.. r^13 terms in float (their float error is < 2e-14 of the
// result; truncation < 2e-16).
FFM_HD ff ff_exp_reduced(ff r) {
  const float s = r.hi;
  const float g = 1.f / 5040.f + s * (1.f / 40320.f + s * (1.f / 362880.f + s * (1.f / 3628800.f +
                  s * (1.f / 39916800.f + s * (1.f / 479001600.f + s * (1.f / 6227020800.f))))));
  ff a = ff_add(WRFGPU_FF(0.0013888889225199819, -3.3631094437103215e-11), ff_mulf(r, g));  // 1/720
  a = ff_add(WRFGPU_FF(0.008333333767950535, -4.34617203337595e-10), ff_mul(r, a));         // 1/120
  a = ff_add(WRFGPU_FF(0.0416666679084301, -1.2417634698280722e-09), ff_mul(r, a));         // 1/24
  a = ff_add(WRFGPU_FF(0.1666666716337204, -4.967053879312289e-09), ff_mul(r, a));          // 1/6
  a = ff_add(ff{0.5f, 0.f}, ff_mul(r, a));
  a = ff_add(ff{1.f, 0.f}, ff_mul(r, a));
  return ff_add(ff{1.f, 0.f}, ff_mul(r, a));
}
#undef WRFGPU_FF

// Ziv's rounding test for a normalised float-float v = hi + lo (|lo| <= ulp(hi)/2)
// known to relative accuracy ~1e-14: hi is the correctly rounded value unless
// |lo| lies within 1e-12 |hi| of half an ulp of hi, or hi is a power of two.
FFM_HD bool rounds_safely(ff v) {
  int e;
  const float m = frexpf_(fabsf(v.hi), &e);
  if (m == 0.5f) return false;
  const float half_ulp = ldexpf_(1.f, e - 25);
  return fabsf(fabsf(v.lo) - half_ulp) > 1e-12f * fabsf(v.hi);
}

// log(x) for x > 0, correctly rounded to float.
FFM_HD float logf_cr(float x) {
  ff l = ff_log(x);
  l = fast_two_sum(l.hi, l.lo);
  if (rounds_safely(l)) return l.hi;
  return (float)::log((double)x);
}

// x^y for x > 0 (finite, normal result), correctly rounded to float.
FFM_HD float powf_cr(float x, float y) {
  ff z = ff_mulf(ff_log(x), y);
  const float n = rintf_(z.hi * INV_LN2);
  const ff nl = two_prod(n, LN2_HI);  // n ln2_hi exactly
  ff r = ff_add(z, ff{-nl.hi, -nl.lo});
  r = ff_add(r, ff{-n * LN2_LO, 0.f});
  ff v = ff_exp_reduced(r);
  v = fast_two_sum(v.hi, v.lo);
  if (rounds_safely(v)) return ldexpf_(v.hi, (int)n);
  return (float)::pow((double)x, (double)y);
}

}  // namespace wrfgpu_ff
