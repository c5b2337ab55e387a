// Bit-for-bit check of the paired flux helpers (wrf_gb300/csrc/pair.cuh)
// against their scalar twins (common.cuh): 2^20 pairs of inputs drawn from
// zeros, subnormals, repeated values, small values and the whole exponent
// range; every helper must give each lane the scalar helper's bits.  Prints
// one line per helper with its mismatch count and exits non-zero on a CUDA
// error.  Each thread reads 8 inputs of its own slot and 8 of slot
// (7 t + 3) mod N, both inside the 8 N-float input.
#include <cstdio>
#include <cstring>
#include <cstdint>
#include "../../wrf_gb300/csrc/pair.cuh"
using namespace wrfgpu;
constexpr int N = 1 << 20;
constexpr int NH = 8;  // helpers checked

__global__ void k_check(const float* in, unsigned* bad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N) return;
  const float* a = in + 8 * (size_t)t;
  const float* b = in + 8 * (size_t)((t * 7 + 3) % N);
  float2 v[6];
  for (int q = 0; q < 6; ++q) v[q] = make_float2(a[q], b[q]);
  const float ua = a[7] - 0.5f;
  float2 r[NH];
  r[0] = flux5_2(v[0], v[1], v[2], v[3], v[4], v[5], ua);
  r[1] = flux3_2(v[0], v[1], v[2], v[3], ua);
  r[2] = pflux5_2(v[0], v[1], v[2], v[3], v[4], v[5], ua);
  r[3] = pflux3_2(v[0], v[1], v[2], v[3], ua);
  r[4] = flux_upwind_2(v[0], v[1], upwind_weights(ua));
  r[5] = add2(v[0], v[1]);
  r[6] = sub2(v[0], v[1]);
  r[7] = mul2(v[0], v[1]);
  for (int l = 0; l < 2; ++l) {
    const float* w = l ? b : a;
    float s[NH];
    s[0] = flux5(w[0], w[1], w[2], w[3], w[4], w[5], ua);
    s[1] = flux3(w[0], w[1], w[2], w[3], ua);
    s[2] = pflux5(w[0], w[1], w[2], w[3], w[4], w[5], ua);
    s[3] = pflux3(w[0], w[1], w[2], w[3], ua);
    s[4] = flux_upwind(w[0], w[1], ua);
    s[5] = __fadd_rn(w[0], w[1]);
    s[6] = __fsub_rn(w[0], w[1]);
    s[7] = __fmul_rn(w[0], w[1]);
    for (int q = 0; q < NH; ++q) {
      const float p = l ? r[q].y : r[q].x;
      if (__float_as_uint(p) != __float_as_uint(s[q])) atomicAdd(&bad[q], 1u);
    }
  }
}

int main() {
  float* h = new float[8 * (size_t)N];
  uint32_t st = 12345;
  auto rnd = [&]() { st = st * 1664525u + 1013904223u; return st; };
  for (size_t q = 0; q < 8 * (size_t)N; ++q) {
    const uint32_t r = rnd();
    float x;
    switch (r % 8) {
      case 0: x = 0.f; break;                                                   // zeros
      case 1: { uint32_t u = rnd() & 0x807fffffu; memcpy(&x, &u, 4); break; }  // subnormals
      case 2: x = (float)(rnd() % 1000) * 1e-3f; break;                         // repeated values
      case 3: x = 1e-6f * (float)(rnd() % 100); break;                          // small values
      default: { uint32_t u = (rnd() & 0x3fffffffu) | ((rnd() & 1u) << 31); memcpy(&x, &u, 4); }
    }
    h[q] = x;
  }
  float* d = nullptr;
  unsigned* bad = nullptr;
  if (cudaMalloc(&d, 8 * (size_t)N * 4) != cudaSuccess || cudaMalloc(&bad, NH * 4) != cudaSuccess) return 2;
  cudaMemcpy(d, h, 8 * (size_t)N * 4, cudaMemcpyHostToDevice);
  cudaMemset(bad, 0, NH * 4);
  k_check<<<N / 256, 256>>>(d, bad);
  unsigned hb[NH];
  cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
  const char* nm[NH] = {"flux5", "flux3", "pflux5", "pflux3", "upwind", "add", "sub", "mul"};
  for (int q = 0; q < NH; ++q) printf("%-7s mismatches %u\n", nm[q], hb[q]);
  const cudaError_t e = cudaGetLastError();
  printf("status %s\n", cudaGetErrorString(e));
  cudaFree(d);
  cudaFree(bad);
  delete[] h;
  return e == cudaSuccess ? 0 : 1;
}
