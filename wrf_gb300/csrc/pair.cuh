// Two species in the two lanes of a packed FP32 pair.
//
// Blackwell executes add / sub / fma on float2 operands as one instruction
// (add.rn.f32x2 etc.) with each lane rounded exactly as the scalar
// instruction rounds it (IEEE round-to-nearest-even per component).  The
// scalar transport kernels carry two species per thread in such pairs: every
// flux, limiter and update expression keeps the reference's scalar operation
// order, lane by lane, so each lane's bits are those of the scalar code; the
// species-independent factors (mass fluxes, Courant numbers, column
// constants) are shared by both lanes, and the additions, which dominate the
// flux and limiter arithmetic, take one instruction per pair.  Comparisons,
// min / max and divisions stay per lane.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace wrfgpu {

__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }
// Explicit round-to-nearest packed instructions (PTX add / sub / fma
// .rn.f32x2).  Products are formed lane by lane with the scalar multiply:
// measured on GB300, a packed multiply whose result feeds a chain of packed
// additions can come out rounded as if fused with them, while a scalar
// product feeding packed additions always rounds where the scalar code does
// (bit-for-bit checks of every helper below against its scalar twin on
// 2^20 random, tiny, zero and subnormal pairs: tests/native/pair_check.cu).
__device__ __forceinline__ unsigned long long u64_of(float2 a) { return *reinterpret_cast<unsigned long long*>(&a); }
__device__ __forceinline__ float2 f2_of(unsigned long long r) { return *reinterpret_cast<float2*>(&r); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(u64_of(a)), "l"(u64_of(b)));
  return f2_of(r);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(u64_of(a)), "l"(u64_of(b)));
  return f2_of(r);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(u64_of(a)), "l"(u64_of(b)), "l"(u64_of(c)));
  return f2_of(r);
}
// s * x with a scalar s: (s * x.x, s * x.y)
__device__ __forceinline__ float2 muls(float s, float2 x) { return make_float2(s * x.x, s * x.y); }

// pflux5 (common.cuh) of both lanes: velocity ua is species-independent.
__device__ __forceinline__ float2 pflux5_2(float2 qm3, float2 qm2, float2 qm1, float2 q, float2 qp1, float2 qp2,
                                           float ua) {
  const float2 p6 = add2(sub2(muls(37.f / 60.f, add2(q, qm1)), muls(2.f / 15.f, add2(qp1, qm2))),
                         muls(1.f / 60.f, add2(qp2, qm3)));
  const float2 d = add2(sub2(sub2(qp2, qm3), muls(5.f, sub2(qp1, qm2))), muls(10.f, sub2(q, qm1)));
  return sub2(p6, muls(1.f * sgn1(ua) * (1.f / 60.f), d));
}
// pflux3 (common.cuh) of both lanes
__device__ __forceinline__ float2 pflux3_2(float2 qm2, float2 qm1, float2 q, float2 qp1, float ua) {
  const float2 p4 = sub2(muls(7.f / 12.f, add2(q, qm1)), muls(1.f / 12.f, add2(qp1, qm2)));
  return add2(p4, muls(1.f * sgn1(ua) * (1.f / 12.f), sub2(sub2(qp1, qm2), muls(3.f, sub2(q, qm1)))));
}
// flux_upwind (common.cuh): the two Courant weights are species-independent
struct Upw {
  float a, b;
};
__device__ __forceinline__ Upw upwind_weights(float cr) {
  return Upw{0.5f * fminf_f(1.0f, (cr + fabsf(cr))), 0.5f * fmaxf_f(-1.0f, (cr - fabsf(cr)))};
}
__device__ __forceinline__ float2 flux_upwind_2(float2 qm1, float2 q, Upw w) {
  return add2(muls(w.a, qm1), muls(w.b, q));
}

// wrfgpu_div_const_pair (cdiv.h) of both lanes: x / c + s y / c with each
// quotient rounded as IEEE division.  When every numerator of both lanes is
// in the method's range the two lanes go through the packed fused
// multiply-adds together (each lane the scalar method's operations);
// otherwise each lane takes the scalar function.
__device__ __forceinline__ bool div_range_ok(float x, float y) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float lo = ax < ay ? ax : ay, hi = ax < ay ? ay : ax;
  return lo >= 0x1p-110f && hi <= 3.40282347e38f;
}
__device__ __forceinline__ float2 div_const_pair2(float2 x, float2 y, float s, float c, float zh) {
  if (div_range_ok(x.x, y.x) && div_range_ok(x.y, y.y)) {
    const float2 z2 = bc2(zh), nc2 = bc2(-c);
    const float2 qx = mul2(x, z2), qy = mul2(y, z2);
    const float2 rx = fma2(qx, nc2, x), ry = fma2(qy, nc2, y);
    const float2 a = fma2(rx, z2, qx), b = fma2(ry, z2, qy);
    return s > 0.f ? add2(a, b) : sub2(a, b);
  }
  return make_float2(wrfgpu_div_const_pair(x.x, y.x, s, c, zh), wrfgpu_div_const_pair(x.y, y.y, s, c, zh));
}
// flux5 / flux3 (common.cuh) of both lanes
__device__ __forceinline__ float2 flux5_2(float2 qm3, float2 qm2, float2 qm1, float2 q, float2 qp1, float2 qp2,
                                          float ua) {
  const float2 x = add2(sub2(muls(37.f, add2(q, qm1)), muls(8.f, add2(qp1, qm2))), add2(qp2, qm3));
  const float2 y = muls(1.f * sgn1(ua), add2(sub2(sub2(qp2, qm3), muls(5.f, sub2(qp1, qm2))), muls(10.f, sub2(q, qm1))));
  return div_const_pair2(x, y, -1.0f, 60.0f, 1.0f / 60.0f);
}
__device__ __forceinline__ float2 flux3_2(float2 qm2, float2 qm1, float2 q, float2 qp1, float ua) {
  const float2 x = sub2(muls(7.f, add2(q, qm1)), add2(qp1, qm2));
  const float2 y = muls(1.f * sgn1(ua), sub2(sub2(qp1, qm2), muls(3.f, sub2(q, qm1))));
  return div_const_pair2(x, y, 1.0f, 12.0f, 1.0f / 12.0f);
}

__device__ __forceinline__ float2 max0_2(float2 x) { return make_float2(fmaxf_f(0.f, x.x), fmaxf_f(0.f, x.y)); }
__device__ __forceinline__ float2 min0_2(float2 x) { return make_float2(fminf_f(0.f, x.x), fminf_f(0.f, x.y)); }

}  // namespace wrfgpu
