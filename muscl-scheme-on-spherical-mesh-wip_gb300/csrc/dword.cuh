// Double-word arithmetic on FP32 pairs, for the FP64-grade parts of the
// mixed update that would otherwise run on the narrow FP64 pipe.
//
// A double-word x = h + l is an unevaluated sum of two floats with
// |l| <= ulp(h) / 2: about 48 significant bits.  The building blocks are the
// error-free transformations TwoSum (Knuth, TAOCP vol. 2, 4.2.2), Fast2Sum
// (Dekker 1971, valid for |a| >= |b|) and TwoProd with a fused multiply-add;
// the cancellation-safe sum and the product follow the double-word
// algorithms analysed by Joldes, Muller and Popescu ("Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic", ACM
// TOMS 44, 2017: AccurateDWPlusDW and DWTimesDW), the quotient is one
// correction step of an FP32 quotient.  Every rounding is an explicit
// round-to-nearest intrinsic, so compiling with FMA contraction leaves the
// error-free transformations intact.
//
// Host and device: the CPU test suite checks the split and the pressure
// recovery against exact rational arithmetic.
#pragma once

#include <cmath>
#include <cstdint>

#include "fp_convert.cuh"

namespace splash {
namespace dw {

struct DW {
  float h, l;
};

SPLASH_HD float add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
SPLASH_HD float sub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
SPLASH_HD float mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
SPLASH_HD float fma_rn(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// s + e = a + b exactly, for |a| >= |b| (or a = 0)
SPLASH_HD DW fast_two_sum(float a, float b) {
  const float s = add_rn(a, b);
  return {s, sub_rn(b, sub_rn(s, a))};
}
// s + e = a + b exactly
SPLASH_HD DW two_sum(float a, float b) {
  const float s = add_rn(a, b);
  const float bb = sub_rn(s, a);
  return {s, add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb))};
}
// p + e = a b exactly
SPLASH_HD DW two_prod(float a, float b) {
  const float p = mul_rn(a, b);
  return {p, fma_rn(a, b, -p)};
}

SPLASH_HD DW neg(DW x) { return {-x.h, -x.l}; }

// x + y, accurate under cancellation
SPLASH_HD DW add(DW x, DW y) {
  const DW s = two_sum(x.h, y.h);
  const DW t = two_sum(x.l, y.l);
  const DW v = fast_two_sum(s.h, add_rn(s.l, t.h));
  return fast_two_sum(v.h, add_rn(t.l, v.l));
}
// x + y for operands of the same sign (no cancellation)
SPLASH_HD DW add_same_sign(DW x, DW y) {
  const DW s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, add_rn(s.l, add_rn(x.l, y.l)));
}
// x y
SPLASH_HD DW mul(DW x, DW y) {
  const DW c = two_prod(x.h, y.h);
  const float t = fma_rn(x.l, y.h, mul_rn(x.h, y.l));
  return fast_two_sum(c.h, add_rn(c.l, t));
}
// x x
SPLASH_HD DW sqr(DW x) {
  const DW c = two_prod(x.h, x.h);
  return fast_two_sum(c.h, fma_rn(add_rn(x.h, x.h), x.l, c.l));
}
// x / y: the FP32 quotient q of the high parts plus the FP32 quotient of the
// remainder x - q y (its leading part exact by Sterbenz's lemma)
SPLASH_HD DW div(DW x, DW y) {
  const float r = 1.0f / y.h;
  const float q = mul_rn(x.h, r);
  const DW p = two_prod(q, y.h);
  float d = sub_rn(x.h, p.h);
  d = sub_rn(d, p.l);
  d = add_rn(d, x.l);
  d = fma_rn(-q, y.l, d);
  return fast_two_sum(q, mul_rn(d, r));
}

// x = h + l from the encoding of a double: h = x rounded to the nearest
// float (the same as fpc::d2f), l = the residual x - h (an integer number of
// ulps of x, at most 2^28 of them) rounded to a float, so h + l is x to about
// 2^-48 relative.  Outside the FP32 normal range l = 0 (h is then 0, an
// infinity or a NaN, as fpc::d2f gives it).
SPLASH_HD DW split(double x) {
  uint32_t hi, lo;
  fpc::double_halves(x, hi, lo);
  const uint32_t s = hi & 0x80000000u, t = hi & 0x7fffffffu;
  const uint32_t e = t >> 20;
  if (e < 897u || e > 1150u) return {fpc::d2f(x), 0.f};
  uint32_t r = ((t - (896u << 20)) << 3) | (lo >> 29);
  const uint32_t rem = lo & 0x1fffffffu;
  int32_t res = (int32_t)rem;
  if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) {
    r += 1u;
    res -= 0x20000000;
  }
  if (r >= 0x7f800000u) return {fpc::bits_float(s | 0x7f800000u), 0.f};
  // ulp(x) = 2^(e - 1075) = 2^-52 * 2^(e - 1023), the latter a normal float
  const float l = mul_rn(mul_rn((float)res, 0x1p-52f), fpc::bits_float((e - 896u) << 23));
  return {fpc::bits_float(s | r), s ? -l : l};
}

// The FP32 face state of the FP64 state u: w[0..3] = (Sigma, l) rounded to
// the nearest float, w[4] = Pi = (E - |r x l|^2 / (2 Sigma)) (gam - 1)
// floored at 1e-16 (MUSCL_base.hpp:538), evaluated in double-word
// arithmetic (relative error a few 2^-44 times the cancellation ratio
// E / (E - |r x l|^2 / (2 Sigma))) and rounded to a float.  r is the unit
// face centre and gam_m1 = gam - 1, both as double-words.
SPLASH_HD void face_state_dw(const double* u, const DW* r, DW gam_m1, float* w) {
  const DW sg = split(u[0]);
  const DW lx = split(u[1]), ly = split(u[2]), lz = split(u[3]);
  const DW E = split(u[4]);
  w[0] = sg.h;
  w[1] = lx.h;
  w[2] = ly.h;
  w[3] = lz.h;
  const DW cx = add(mul(r[1], lz), neg(mul(r[2], ly)));
  const DW cy = add(mul(r[2], lx), neg(mul(r[0], lz)));
  const DW cz = add(mul(r[0], ly), neg(mul(r[1], lx)));
  const DW c2 = add_same_sign(add_same_sign(sqr(cx), sqr(cy)), sqr(cz));
  const DW ke2 = div(c2, sg);
  const DW pe = mul(add(E, {-0.5f * ke2.h, -0.5f * ke2.l}), gam_m1);
  // fmaxf returns the number for a NaN operand, like (1e-16 < p) ? p : 1e-16
  w[4] = fmaxf(pe.h, 1e-16f);
}

}  // namespace dw
}  // namespace splash
