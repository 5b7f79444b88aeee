#pragma once
// IEEE-754 binary32 <-> binary64 conversions in integer arithmetic.
//
// On GB300 the FP64 pipe issues at a small fraction of the FP32 / integer
// rate, and the F2F conversions between float and double issue on it.  The
// mixed-form node update converts about fifteen values per node; doing that
// with integer operations keeps the FP64 pipe for the FP64 arithmetic.
//
// Both functions return exactly what the hardware conversion returns (round
// to nearest even when narrowing).  They handle normal numbers and zeros
// themselves and hand the rare rest (subnormals, infinities, NaNs, doubles
// outside the normal float range) to the hardware conversion.  The header
// also compiles as plain C++ so that the host test can check it against the
// host's own conversions.
#include <stdint.h>
#ifdef __CUDACC__
#define RG_BITS_FN __host__ __device__ __forceinline__
#else
#include <string.h>
#define RG_BITS_FN inline
#endif

namespace rg {

RG_BITS_FN uint32_t bits_f32(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
RG_BITS_FN float f32_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
RG_BITS_FN uint64_t bits_f64(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
RG_BITS_FN double f64_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}

// float -> double (exact): the exponent is rebiased (127 -> 1023) and the
// 23-bit fraction moved to the top of the 52-bit one.
RG_BITS_FN double widen_f32(float f) {
  const uint32_t u = bits_f32(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t frac = u & 0x7fffffu;
  if (e == 0xffu || (e == 0u && frac != 0u)) return (double)f;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t body = e ? ((uint64_t)(e + 896u) << 52) | ((uint64_t)frac << 29) : 0ull;
  return f64_bits(sign | body);
}

// double -> float, round to nearest even: the 52-bit fraction keeps its top
// 23 bits; the 29 dropped bits decide the rounding (above half: up; exactly
// half: up when the kept part is odd).  A carry out of the fraction moves
// into the exponent, up to infinity as the hardware does.
RG_BITS_FN float narrow_f64(double d) {
  const uint64_t b = bits_f64(d);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e >= 897u && e <= 1150u) {
    const uint64_t frac = b & 0xfffffffffffffull;
    const uint32_t kept = ((e - 896u) << 23) | (uint32_t)(frac >> 29);
    const uint32_t rest = (uint32_t)(frac & 0x1fffffffu);
    const uint32_t up = (rest > 0x10000000u) || (rest == 0x10000000u && (kept & 1u));
    return f32_bits(sign | (kept + up));
  }
  if ((b << 1) == 0ull) return f32_bits(sign);
  return (float)d;
}

// A non-negative integer below 2^31 held in a double (a node code) as an
// int, from the bits.
RG_BITS_FN int small_int_f64(double d) {
  const uint64_t b = bits_f64(d);
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;
  if (e < 0) return 0;
  if (e > 30 || (b >> 63)) return (int)d;
  return (int)(((b & 0xfffffffffffffull) | (1ull << 52)) >> (52 - e));
}

}  // namespace rg
