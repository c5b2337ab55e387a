// Host check of the correctly rounded logf_cr / powf_cr of
// wrf_gb300/csrc/ffmath.h (the same float-float code the kernels run; built
// with -ffp-contract=off, fma only where the code asks for it).
//  * every float in [1/4, 4) and a strided sample of [2^-40, 2^40]:
//    logf_cr(x) == (float)log((double)x);
//  * a strided sample of x in [1e-3, 4]: powf_cr(x, 1.4) == (float)pow(x, 1.4);
//  * the float-float approximations' relative error against long double,
//    which must stay below the rounding test's 1e-12 bound;
//  * sinf_cr on every 32nd float of [0, pi/2] against long double sin rounded
//    to float, and its double-double series alone on a sparser sample.
// Prints the counts; exit status 1 on any mismatch or error above 5e-13.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include "../../wrf_gb300/csrc/ffmath.h"

using namespace wrfgpu_ff;

static float from_bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t to_bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

int main() {
  long long nlog = 0, badlog = 0, npow = 0, badpow = 0;
  double maxe_log = 0.0, maxe_pow = 0.0;
  auto check_log = [&](float x) {
    ++nlog;
    const float a = logf_cr(x), b = (float)std::log((double)x);
    if (to_bits(a) != to_bits(b)) ++badlog;
    const ff l = ff_log_t(x);
    const long double ex = logl((long double)x);
    if (ex != 0.0L) {
      const double e = (double)fabsl(((long double)l.hi + (long double)l.lo - ex) / ex);
      if (e > maxe_log) maxe_log = e;
    }
  };
  for (uint32_t u = to_bits(0.25f); u < to_bits(4.0f); ++u) check_log(from_bits(u));
  for (uint32_t u = to_bits(0x1p-40f); u < to_bits(0x1p40f); u += 997) check_log(from_bits(u));
  const float y = 1.4f;
  for (uint32_t u = to_bits(1e-3f); u < to_bits(4.0f); u += 13) {
    const float x = from_bits(u);
    ++npow;
    const float a = powf_cr(x, y), b = (float)std::pow((double)x, (double)y);
    if (to_bits(a) != to_bits(b)) ++badpow;
    const ff z = ff_mulf(ff_log_t(x), y);
    int k = 0;
    const ff v = ff_exp_t(z, &k);
    const long double ex = powl((long double)x, (long double)y);
    const double e = (double)fabsl((ldexpl((long double)v.hi + (long double)v.lo, k) - ex) / ex);
    if (e > maxe_pow) maxe_pow = e;
  }
  long long nsin = 0, badsin = 0, nser = 0, badser = 0;
  for (uint32_t u = 0; u <= to_bits(1.5707964f); u += 32) {
    const float x = from_bits(u);
    ++nsin;
    if (to_bits(sinf_cr(x)) != to_bits((float)sinl((long double)x))) ++badsin;
  }
  for (uint32_t u = to_bits(1e-6f); u <= to_bits(1.5707964f); u += 1021) {
    const float x = from_bits(u);
    ++nser;
    const dd v = sin_dd_small((double)x);
    const long double ex = sinl((long double)x);
    const long double e = fabsl(((long double)v.hi + (long double)v.lo - ex) / ex);
    if (e > 1e-18L) ++badser;
  }
  std::printf("log: %lld inputs, %lld mismatches, max rel error %.3e\n", nlog, badlog, maxe_log);
  std::printf("pow: %lld inputs, %lld mismatches, max rel error %.3e\n", npow, badpow, maxe_pow);
  std::printf("sin: %lld inputs, %lld mismatches; series: %lld inputs, %lld above 1e-18\n", nsin, badsin, nser, badser);
  return (badlog || badpow || badsin || badser || maxe_log > 5e-13 || maxe_pow > 5e-13) ? 1 : 0;
}
