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
