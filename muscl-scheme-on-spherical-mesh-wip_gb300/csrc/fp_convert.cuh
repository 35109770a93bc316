// FP32 <-> FP64 conversions in integer arithmetic.
//
// On this GPU FP64 instructions, conversions to and from FP64 included, issue
// on a narrow shared pipe (two lanes per SM per clock), while integer
// instructions issue at full rate.  The mixed path's per-face update converts
// every state field twice per stage, so these conversions are written as bit
// manipulation of the IEEE-754 encodings:
//
//   f2d  float -> double, exact (sign, exponent re-biased by 1023 - 127 = 896,
//        mantissa shifted left by 52 - 23 = 29); FP32 subnormals read as zero,
//        like every FP32 operation of the mixed path (compiled flush-to-zero)
//   d2f  double -> float, round to nearest, ties to even; results below the
//        smallest FP32 normal are flushed to a signed zero, results beyond the
//        largest FP32 value round to infinity, NaN stays NaN
//
// Host and device: the CPU test suite checks both against numpy's conversions.
#pragma once

#include <cstdint>
#include <cstring>

#include "dual.cuh"  // SPLASH_HD

namespace splash {
namespace fpc {

SPLASH_HD uint32_t float_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return b;
#endif
}
SPLASH_HD float bits_float(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, 4);
  return x;
#endif
}
SPLASH_HD void double_halves(double x, uint32_t& hi, uint32_t& lo) {
#ifdef __CUDA_ARCH__
  hi = (uint32_t)__double2hiint(x);
  lo = (uint32_t)__double2loint(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  hi = (uint32_t)(b >> 32);
  lo = (uint32_t)b;
#endif
}
SPLASH_HD double halves_double(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t b = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

SPLASH_HD double f2d(float x) {
  const uint32_t b = float_bits(x);
  const uint32_t s = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  if (e == 0u) return halves_double(s, 0u);
  const uint32_t ed = (e == 255u) ? 2047u : e + 896u;
  return halves_double(s | (ed << 20) | (m >> 3), m << 29);
}

SPLASH_HD float d2f(double x) {
  uint32_t hi, lo;
  double_halves(x, hi, lo);
  const uint32_t s = hi & 0x80000000u, t = hi & 0x7fffffffu;
  const uint32_t e = t >> 20;
  uint32_t r;
  if (e >= 897u && e <= 1150u) {
    // exponent e - 896 in bits 23..30, the top 23 mantissa bits below it
    r = ((t - (896u << 20)) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1fffffffu;
    // a carry out of the mantissa steps the exponent, up to infinity
    if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) r += 1u;
  } else if (e < 897u) {
    r = 0u;
  } else if (e == 2047u && ((t & 0xfffffu) | lo) != 0u) {
    r = 0x7fc00000u;
  } else {
    r = 0x7f800000u;
  }
  return bits_float(s | r);
}

// x is NaN, from its encoding
SPLASH_HD bool is_nan_bits(double x) {
  uint32_t hi, lo;
  double_halves(x, hi, lo);
  const uint32_t t = hi & 0x7fffffffu;
  return t > 0x7ff00000u || (t == 0x7ff00000u && lo != 0u);
}

}  // namespace fpc
}  // namespace splash
