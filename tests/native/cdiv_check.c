/* Host check of wrfgpu_div12 / wrfgpu_div60 (wrf_gb300/csrc/cdiv.h) against
 * IEEE division.  Covers every input of magnitude below 2^-96 (where the
 * guard and the subnormal quotients sit), every input in [1, 4) (two whole
 * binades: away from the subnormal range the method is invariant under
 * scaling by powers of two), both signs, and a strided sample over all bit
 * patterns.  The paired forms (x / 60 - y / 60, x / 12 + y / 12 under one
 * range test) are checked on pairs drawn from the same inputs and from the
 * special values.  Prints the number of mismatches; exit status 1 on any. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include "../../wrf_gb300/csrc/cdiv.h"

static float from_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static unsigned long long bad = 0, checked = 0;

static int same(float a, float b) { return to_bits(a) == to_bits(b) || (a != a && b != b); }

static void check_pair(float x, float y) {
  const float a = x / 60.0f - y / 60.0f, b = wrfgpu_div60_sub(x, y);
  const float c = x / 12.0f + y / 12.0f, d = wrfgpu_div12_add(x, y);
  ++checked;
  if (!same(a, b)) ++bad;
  if (!same(c, d)) ++bad;
}

static void check(uint32_t u) {
  float x = from_bits(u);
  float a = x / 12.0f, b = wrfgpu_div12(x);
  float c = x / 60.0f, d = wrfgpu_div60(x);
  ++checked;
  if (to_bits(a) != to_bits(b) && !(a != a && b != b)) ++bad;
  if (to_bits(c) != to_bits(d) && !(c != c && d != d)) ++bad;
}

int main(void) {
  const uint32_t small_end = to_bits(0x1p-96f);
  const uint32_t one = to_bits(1.0f), four = to_bits(4.0f);
  for (uint32_t s = 0; s < 2; ++s) {
    const uint32_t sign = s << 31;
    for (uint32_t u = 0; u < small_end; ++u) check(sign | u);
    for (uint32_t u = one; u < four; ++u) check(sign | u);
  }
  for (uint64_t u = 0; u < (1ull << 32); u += 4099) check((uint32_t)u);
  check(to_bits(1.0f / 0.0f));
  check(to_bits(-1.0f / 0.0f));
  {
    const float special[] = {0.0f, -0.0f, 0x1p-126f, -0x1p-149f, 0x1p-111f, 0x1p-110f, -0x1p-109f, 1.0f, -3.0f,
                             5.0e-7f, 3.40282347e38f, -3.40282347e38f, 1.0f / 0.0f, -1.0f / 0.0f};
    const int ns = (int)(sizeof(special) / sizeof(special[0]));
    for (int a = 0; a < ns; ++a)
      for (int b = 0; b < ns; ++b) check_pair(special[a], special[b]);
    uint32_t h = 12345u;
    for (uint64_t u = 0; u < (1ull << 32); u += 65537) {
      h = h * 1664525u + 1013904223u;
      check_pair(from_bits((uint32_t)u), from_bits(h));
      check_pair(from_bits((uint32_t)u), from_bits((uint32_t)u ^ 0x00400001u));  /* close in value */
      check_pair(from_bits(one + (h & 0x7fffffu)), from_bits(one + ((uint32_t)u & 0x7fffffu)));
    }
  }
  printf("checked %llu inputs, %llu mismatches\n", checked, bad);
  return bad != 0;
}
