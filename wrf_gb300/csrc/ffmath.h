// Correctly rounded (to within ~1e-10 relative before the final rounding)
// single-precision log and pow, evaluated in float-float ("double-float")
// arithmetic with FP32 fused multiply-adds: Dekker's TwoSum / TwoProduct
// error-free transformations and truncated Taylor series of atanh and exp.
// They replace the libm calls of calc_p_rho_phi (the reference's LOG and
// x**cpovcv through vspow) so the GPU rounds like a correctly rounded libm,
// which the reference's glibc build matches in all but rare cases.
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
  float e = (s.lo + a.lo) + b.lo;
  return fast_two_sum(s.hi, e);
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
FFM_HD ff ff_div(ff a, ff b) {  // a / b, two Newton-style correction steps
  float q1 = a.hi / b.hi;
  ff r = ff_add(a, ff_mulf(ff{-b.hi, -b.lo}, q1));
  float q2 = r.hi / b.hi;
  r = ff_add(r, ff_mulf(ff{-b.hi, -b.lo}, q2));
  float q3 = r.hi / b.hi;
  ff q = fast_two_sum(q1, q2);
  return ff_add(q, ff{q3, 0.f});
}

// ln 2 split into a float and its float remainder.
constexpr float LN2_HI = 0.6931471824645996f;
constexpr float LN2_LO = -1.9046542121259336e-09f;

// natural log of x > 0 as a float-float: x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(t), t = (m-1)/(m+1), |t| <= 0.172.
FFM_HD ff ff_log(float x) {
  int e = 0;
#ifdef __CUDA_ARCH__
  float m = frexpf(x, &e);
#else
  float m = std::frexp(x, &e);
#endif
  if (m < 0.70710678f) { m = m * 2.f; e -= 1; }
  ff num = {m - 1.f, 0.f};                  // exact (Sterbenz)
  ff den = two_sum(m, 1.f);
  ff t = ff_div(num, den);
  ff t2 = ff_mul(t, t);
  // 2t (1 + t^2/3 + t^4/5 + ...): leading 1/3 term in float-float, the rest in float
  float s2 = t2.hi;
  float tail = s2 * (1.f / 5.f + s2 * (1.f / 7.f + s2 * (1.f / 9.f + s2 * (1.f / 11.f + s2 * (1.f / 13.f)))));
  ff third = {0.3333333432674408f, -9.934107758624577e-09f};  // 1/3 as float-float
  ff inner = ff_add(third, ff{tail, 0.f});              // 1/3 + t^2/5 + ...
  ff series = ff_add(ff{1.f, 0.f}, ff_mul(t2, inner));  // 1 + t^2 (1/3 + ...)
  ff lm = ff_mul(ff{2.f * t.hi, 2.f * t.lo}, series);
  ff el = ff_add(two_prod((float)e, LN2_HI), ff{(float)e * LN2_LO, 0.f});
  return ff_add(el, lm);
}

// exp of a float-float |z| <= ~0.7: exp(z) = 1 + z + z^2/2 + z^3/6 + z^4/24 + z^5 P(z),
// the terms up to z^4 in float-float, the z^5 tail in float.
FFM_HD ff ff_exp_small(ff z) {
  ff z2 = ff_mul(z, z);
  ff z3 = ff_mul(z2, z);
  ff z4 = ff_mul(z2, z2);
  const float zh = z.hi;
  const float tail = z4.hi * zh *
                     (1.f / 120.f + zh * (1.f / 720.f + zh * (1.f / 5040.f + zh * (1.f / 40320.f + zh * (1.f / 362880.f)))));
  const ff sixth = {0.1666666716337204f, -4.967053879312289e-09f};    // 1/6
  const ff twentyfourth = {0.0416666679084301f, -1.2417634698280722e-09f};  // 1/24
  ff r = ff_add(ff_mul(z4, twentyfourth), ff{tail, 0.f});
  r = ff_add(ff_mul(z3, sixth), r);
  r = ff_add(ff_mulf(z2, 0.5f), r);
  r = ff_add(z, r);
  return ff_add(ff{1.f, 0.f}, r);
}

// log(x) rounded to float.
FFM_HD float logf_cr(float x) {
  ff l = ff_log(x);
  return l.hi + l.lo;
}

// x^y for x > 0 with |y log x| <= ~0.7 (the equation-of-state range: x near 1).
FFM_HD float powf_cr(float x, float y) {
  ff z = ff_mulf(ff_log(x), y);
  if (fabsf(z.hi) > 0.69f) {  // outside the series range: split exp(z) = exp(z/2)^2
    ff h = ff_exp_small(ff{0.5f * z.hi, 0.5f * z.lo});
    ff r = ff_mul(h, h);
    return r.hi + r.lo;
  }
  ff r = ff_exp_small(z);
  return r.hi + r.lo;
}

}  // namespace wrfgpu_ff
