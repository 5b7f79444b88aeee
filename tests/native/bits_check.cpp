// Host check of the integer float <-> double conversions of rg_bits.h
// against the host's own IEEE conversions (round to nearest even).
// Prints the number of mismatches and of values checked.
#include <math.h>
#include <stdio.h>
#include <stdint.h>

#include "../../openradioss_gb300/csrc/rg_bits.h"

static uint64_t s = 0x9e3779b97f4a7c15ull;
static uint64_t rnd() {
  s ^= s << 13;
  s ^= s >> 7;
  s ^= s << 17;
  return s;
}

static long bad = 0, n = 0;
static void check_narrow(double d) {
  const float a = rg::narrow_f64(d), b = (float)d;
  n++;
  if (isnan(b) ? !isnan(a) : rg::bits_f32(a) != rg::bits_f32(b)) {
    if (bad < 10) printf("narrow %.17g: %a vs %a\n", d, a, b);
    bad++;
  }
}
static void check_widen(float f) {
  const double a = rg::widen_f32(f), b = (double)f;
  n++;
  if (isnan(b) ? !isnan(a) : rg::bits_f64(a) != rg::bits_f64(b)) {
    if (bad < 10) printf("widen %a: %a vs %a\n", f, a, b);
    bad++;
  }
}

int main() {
  // every float whose low 6 fraction bits are a pattern of the stride: all
  // exponents, signs, zeros, subnormals, infinities and NaNs included
  for (uint64_t u = 0; u < (1ull << 32); u += 61) check_widen(rg::f32_bits((uint32_t)u));
  const uint32_t edge[] = {0u, 0x80000000u, 1u, 0x7fffffu, 0x800000u, 0x7f7fffffu, 0x7f800000u,
                           0xff800000u, 0x7fc00000u, 0x80800000u, 0x3f800000u};
  for (uint32_t u : edge) check_widen(rg::f32_bits(u));
  // doubles: random bits over the whole exponent range, and around the
  // float range with the dropped 29 bits at and next to one half
  for (int i = 0; i < 20000000; i++) check_narrow(rg::f64_bits(rnd()));
  for (uint32_t e = 860; e <= 1190; e++)
    for (int i = 0; i < 20000; i++) {
      const uint64_t sign = (rnd() & 1) << 63;
      const uint64_t hi = (rnd() & 0x7fffffull) << 29;
      const uint64_t lows[] = {0ull, 1ull, 0xfffffffull, 0x10000000ull, 0x10000001ull,
                               0x1fffffffull, rnd() & 0x1fffffffull};
      for (uint64_t lo : lows) check_narrow(rg::f64_bits(sign | ((uint64_t)e << 52) | hi | lo));
    }
  const double dedge[] = {0.0, -0.0, 3.4028234663852886e38, 3.4028235677973366e38,
                          3.4028235677973362e38, 1.1754943508222875e-38, 1.401298464324817e-45,
                          7.0064923216240854e-46, INFINITY, -INFINITY, NAN, 1.0, -1.0, 1e300};
  for (double d : dedge) check_narrow(d);
  // node codes
  for (int k = 0; k < 40000000; k += 7) {
    n++;
    if (rg::small_int_f64((double)k) != k) {
      if (bad < 10) printf("code %d\n", k);
      bad++;
    }
  }
  const int big[] = {0x7fffffff, 0x40000000, (7 << 8) | 63, 1 << 30};
  for (int k : big) {
    n++;
    if (rg::small_int_f64((double)k) != k) bad++;
  }
  printf("%ld %ld\n", bad, n);
  return bad != 0;
}
