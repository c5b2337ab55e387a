// Division by a constant without a divide instruction, bit-identical to IEEE
// round-to-nearest division.
//
// Method of Brisebarre, Muller and Raina, "Accelerating correctly rounded
// floating-point division when the divisor is known in advance", IEEE Trans.
// Computers 53(8), 2004: with zh = RN(1/c),
//     q = RN(x * zh),  r = x - q c (exact, one fma),  result = RN(q + r zh).
// Whether this returns RN(x / c) for every x depends on c; for c = 12 and
// c = 60 (the flux denominators of the advection operators) it was checked
// against IEEE division for all 2^32 single-precision inputs (tests run the
// range below 2^-96, two whole binades and a sample of the rest, which covers
// every input by scale invariance).  Inputs of magnitude below 2^-110, where
// the quotient nears the subnormal range and the remainder stops being exact,
// and infinities and NaNs take the division itself.
//
// Shared by the kernels (nvcc) and the host-side check (gcc, with
// -ffp-contract=off so that x * zh is not fused).
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define WRFGPU_HD __host__ __device__ __forceinline__
#else
#define WRFGPU_HD static inline
#endif

WRFGPU_HD float wrfgpu_div_const(float x, float c, float zh) {
  const float ax = fabsf(x);
  if (!(ax >= 0x1p-110f && ax <= 3.40282347e38f)) return x / c;
  const float q = x * zh;
  const float r = fmaf(-q, c, x);
  return fmaf(r, zh, q);
}

WRFGPU_HD float wrfgpu_div12(float x) { return wrfgpu_div_const(x, 12.0f, 1.0f / 12.0f); }
WRFGPU_HD float wrfgpu_div60(float x) { return wrfgpu_div_const(x, 60.0f, 1.0f / 60.0f); }

/* x / c + s y / c with both quotients rounded as IEEE division (s = +1 or
 * -1), one range test for the pair: the fast path is taken when neither
 * numerator is below 2^-110 in magnitude or infinite (a NaN propagates
 * through either path).  The 5th- and 3rd-order fluxes each divide two
 * numerators by the same constant. */
WRFGPU_HD float wrfgpu_div_const_pair(float x, float y, float s, float c, float zh) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float lo = ax < ay ? ax : ay, hi = ax < ay ? ay : ax;
  if (!(lo >= 0x1p-110f && hi <= 3.40282347e38f)) return x / c + s * (y / c);
  const float qx = x * zh, qy = y * zh;
  const float rx = fmaf(-qx, c, x), ry = fmaf(-qy, c, y);
  return fmaf(rx, zh, qx) + s * fmaf(ry, zh, qy);
}
WRFGPU_HD float wrfgpu_div12_add(float x, float y) { return wrfgpu_div_const_pair(x, y, 1.0f, 12.0f, 1.0f / 12.0f); }
WRFGPU_HD float wrfgpu_div60_sub(float x, float y) { return wrfgpu_div_const_pair(x, y, -1.0f, 60.0f, 1.0f / 60.0f); }
