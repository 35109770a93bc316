// FP32 physics of the mixed-precision MUSCL step.
//
// Same formulas as the FP64 path (physics_fp64.cuh, citing the reference),
// evaluated in FP32 with three deliberate differences that keep FP32 away
// from cancellation:
//   * edge states carry the pressure Pi, not the energy: the reference
//     converts Pi -> E at the edge (MUSCL_base.hpp:541-562) and every flux
//     routine converts back E -> Pi (physics/adiabatic.hpp:582-592), a round
//     trip that is exact in real arithmetic but loses digits in FP32 when the
//     kinetic energy dominates; the mixed path uses Pi directly and forms
//     E = Pi/(gam-1) + Sigma |v|^2/2 (a sum of positive terms) where the flux
//     needs it;
//   * the unit edge centre is used without the |ec| ~ 1 rescale;
//   * integer powers are multiplications, pow(1-r, 0.1) is 2^(0.1 log2) and
//     the switch's exponentials are powers of two (hardware ex2 / lg2);
//   * quotients and reciprocals are __fdividef (the approximate reciprocal
//     of the divisor times the dividend): within 2 ulp like the full-range
//     division the path is compiled with otherwise, and equal to it for
//     divisors below 2^126 in magnitude (every divisor here: densities,
//     pressures, wave-speed differences, slopes; measured bit-identical
//     states), without its range handling; zero, infinite and NaN divisors
//     give the same infinities and NaN, which the limiter and the flux
//     checks handle.
#pragma once

#include <cmath>

#include "layout.hpp"

namespace splash {
namespace mx {

struct F3 {
  float x, y, z;
};

__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 scal(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float norm3(F3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
  return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// 2^x and log2(x) as the hardware approximations (PTX ex2.approx.ftz,
// lg2.approx.ftz); e^x = 2^(x log2 e) and x^m = 2^(m log2 x) are written in
// base 2 so that no base conversion is evaluated at run time.
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kLog2e = 1.4426950408889634f;
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }

struct SlotGeomF {
  F3 ec;   // unit edge centre
  F3 en;   // edge normal
  F3 nxr;  // cross(en, ec)
};

// Primitive view of one edge state u = (Sigma, l, Pi).
struct EdgeState {
  float rho;
  F3 vel;    // cross(ec, l) / (-Sigma)
  float p;   // max(1e-16, Pi)   (pressure floor of adiabatic.hpp:586-591)
  float E;   // Pi/(gam-1) + Sigma |v|^2/2
  float vn;  // v . n
};

__device__ __forceinline__ EdgeState edge_state(const float* u, const SlotGeomF& g, float gam) {
  EdgeState s;
  s.rho = u[0];
  const float inv = __fdividef(-1.0f, u[0]);
  s.vel = scal(cross3(g.ec, f3(u[1], u[2], u[3])), inv);
  s.p = smax(1e-16f, u[4]);
  s.E = __fdividef(u[4], gam - 1.0f) + 0.5f * u[0] * dot3(s.vel, s.vel);
  s.vn = dot3(s.vel, g.en);
  return s;
}

// physics/adiabatic.hpp:352-392 with u[4] = E supplied separately
__device__ __forceinline__ void phys_flux(const float* u, const EdgeState& s, const SlotGeomF& g,
                                          float* F) {
  F[0] = s.rho * s.vn;
  F[1] = u[1] * s.vn - g.nxr.x * s.p;
  F[2] = u[2] * s.vn - g.nxr.y * s.p;
  F[3] = u[3] * s.vn - g.nxr.z * s.p;
  F[4] = (s.E + s.p) * s.vn;
}

// PVRS wave speeds, physics/adiabatic.hpp:594-683
__device__ __forceinline__ void char_vel(const EdgeState& L, const EdgeState& R, float gam,
                                         float& S_L, float& S_R, float& a_L, float& a_R) {
  a_L = sqrtf(__fdividef(gam * L.p, L.rho));
  a_R = sqrtf(__fdividef(gam * R.p, R.rho));
  const float p_pvrs = 0.5f * (L.p + R.p) - 0.125f * (R.vn - L.vn) * (L.rho + R.rho) * (a_L + a_R);
  const float p_star = smax(0.f, p_pvrs);
  const float k = __fdividef(gam + 1.0f, 2.0f * gam);
  float q_R = 1.f, q_L = 1.f;
  if (!(p_star <= R.p)) {
    q_R = sqrtf(1.f + k * (__fdividef(p_star, R.p) - 1.f));
    if (isnan(q_R) || isinf(q_R)) q_R = 1.f;
  }
  if (!(p_star <= L.p)) {
    q_L = sqrtf(1.f + k * (__fdividef(p_star, L.p) - 1.f));
    if (isnan(q_L) || isinf(q_L)) q_L = 1.f;
  }
  S_L = L.vn - a_L * q_L;
  S_R = R.vn + a_R * q_R;
}

// Riemann fluxes (HLLE_p.hpp:19-58, HLLC.hpp:138-242, HLLCplus.hpp:17-177).
// Returns the stop bits of splash_gb300.h (2 NaN wave speed, 4 ordering).
__device__ __forceinline__ unsigned flux_star(const float* uL, const float* uR, const SlotGeomF& g,
                                              float gam, int solver, float* F) {
  unsigned bits = 0;
  const EdgeState L = edge_state(uL, g, gam);
  const EdgeState R = edge_state(uR, g, gam);
  float S_L, S_R, a_L, a_R;
  char_vel(L, R, gam, S_L, S_R, a_L, a_R);
  if (isnan(S_L) || isnan(S_R)) bits |= 2u;
  float FL[kDim], FR[kDim];
  phys_flux(uL, L, g, FL);
  phys_flux(uR, R, g, FR);
  const float qL[kDim] = {uL[0], uL[1], uL[2], uL[3], L.E};
  const float qR[kDim] = {uR[0], uR[1], uR[2], uR[3], R.E};
  if (solver == 1) {
    if (S_L >= 0) {
#pragma unroll
      for (int i = 0; i < kDim; ++i) F[i] = FL[i];
    } else if (S_L < 0 && S_R > 0) {
      const float inv = __fdividef(1.0f, S_R - S_L);
#pragma unroll
      for (int i = 0; i < kDim; ++i) F[i] = (S_R * FL[i] - S_L * FR[i] + S_R * S_L * (qR[i] - qL[i])) * inv;
    } else {
      if (!(S_R <= 0)) bits |= 4u;
#pragma unroll
      for (int i = 0; i < kDim; ++i) F[i] = FR[i];
    }
    return bits;
  }
  const float V_L = L.vn, V_R = R.vn;
  float S_star = __fdividef(R.p - L.p + L.rho * V_L * (S_L - V_L) - R.rho * V_R * (S_R - V_R),
                            L.rho * (S_L - V_L) - R.rho * (S_R - V_R));
  if (isnan(S_star) || isinf(S_star)) S_star = 0.5f * (V_L + V_R);
  int side;
  if (S_L >= 0) {
    side = 0;
  } else if (S_L < 0 && S_star >= 0) {
    side = 1;
  } else if (S_star < 0 && S_R >= 0) {
    side = 2;
  } else {
    if (!(S_R < 0)) bits |= 4u;
    side = 3;
  }
  if (side == 0 || side == 3) {
    const float* src = (side == 0) ? FL : FR;
#pragma unroll
    for (int i = 0; i < kDim; ++i) F[i] = src[i];
    return bits;
  }
  const float P_LR = 0.5f * (L.p + R.p + L.rho * (S_L - V_L) * (S_star - V_L) +
                             R.rho * (S_R - V_R) * (S_star - V_R));
  const float D[kDim] = {0.f, -g.nxr.x, -g.nxr.y, -g.nxr.z, S_star};
  const float Sk = (side == 1) ? S_L : S_R;
  const float* qk = (side == 1) ? qL : qR;
  const float* Fk = (side == 1) ? FL : FR;
  const float inv = __fdividef(1.0f, Sk - S_star);
#pragma unroll
  for (int i = 0; i < kDim; ++i) F[i] = (S_star * (Sk * qk[i] - Fk[i]) + Sk * P_LR * D[i]) * inv;
  if (solver == 3) {
    const float phi_L = L.rho * (S_L - V_L);
    const float phi_R = R.rho * (S_R - V_R);
    const float M = smin(1.f, smax(__fdividef(norm3(L.vel), a_L), __fdividef(norm3(R.vel), a_R)));
    int lambd = 0;
    if ((V_L - a_L) > 0 && (V_R - a_R) < 0) lambd = 1;
    if ((V_L + a_L) > 0 && (V_R + a_R) < 0) lambd = 1;
    if ((V_R - a_R) > 0 && (V_L - a_L) < 0) lambd = 1;
    if ((V_R + a_R) > 0 && (V_L + a_L) < 0) lambd = 1;
    float f_star = 1.f;
    if (lambd == 0) f_star = __fdividef(M * sqrtf(4.f + (1.f - M * M) * (1.f - M * M)), 1.f + M * M);
    const float h = smin(__fdividef(L.p, R.p), __fdividef(R.p, L.p));
    const float gsw = 1.f - ex2_approx(M * lg2_approx(h));
    const float dV = V_R - V_L;
    const F3 dv = sub(R.vel, L.vel);
    const float cs = Sk * inv * gsw;
    const float fs = (f_star - 1.f) * dV;
    const F3 vff = f3(fs * g.en.x + cs * (dv.x - dV * g.en.x), fs * g.en.y + cs * (dv.y - dV * g.en.y),
                      fs * g.en.z + cs * (dv.z - dV * g.en.z));
    const F3 am = cross3(g.ec, vff);
    const float w = __fdividef(phi_L * phi_R, phi_R - phi_L);
    F[1] += am.x * w;
    F[2] += am.y * w;
    F[3] += am.z * w;
    F[4] += fs * S_star * w;
  }
  return bits;
}

// Isothermal solver (MUSCL_HLLE, 4 fields, pressure a^2 Sigma with a = 1):
// physical flux (physics/isothermal.hpp:141-195), wave speeds (:211-260)
// and the HLLE flux (Riemann_solvers/HLLE.hpp:17-59) in FP32.  In FP32 the
// unit edge centre needs no |ec| rescale, so one edge velocity serves flux
// and wave speeds.  F[4] is 0.  Returns the stop bits of splash_gb300.h.
__device__ __forceinline__ void iso_phys_flux(const float* u, F3 vel, float vn, const SlotGeomF& g, float* F) {
  const float PI = u[0];
  F[0] = u[0] * vn;
  F[1] = u[1] * vn - g.nxr.x * PI;
  F[2] = u[2] * vn - g.nxr.y * PI;
  F[3] = u[3] * vn - g.nxr.z * PI;
  F[4] = 0.f;
}

__device__ __forceinline__ unsigned iso_flux_star(const float* uL, const float* uR, const SlotGeomF& g, float* F) {
  const F3 vL = scal(cross3(g.ec, f3(uL[1], uL[2], uL[3])), __fdividef(-1.0f, uL[0]));
  const F3 vR = scal(cross3(g.ec, f3(uR[1], uR[2], uR[3])), __fdividef(-1.0f, uR[0]));
  const float vnL = dot3(vL, g.en), vnR = dot3(vR, g.en);
  const float S_L = smin(vnL, vnR) - 1.f;
  const float S_R = smax(vnL, vnR) + 1.f;
  unsigned bits = (isnan(S_L) || isnan(S_R)) ? 2u : 0u;
  float FL[kDim], FR[kDim];
  iso_phys_flux(uL, vL, vnL, g, FL);
  iso_phys_flux(uR, vR, vnR, g, FR);
  if (S_L >= 0) {
#pragma unroll
    for (int i = 0; i < kDim; ++i) F[i] = FL[i];
  } else if (S_L < 0 && S_R > 0) {
    const float inv = __fdividef(1.0f, S_R - S_L);
#pragma unroll
    for (int i = 0; i < 4; ++i) F[i] = (S_R * FL[i] - S_L * FR[i] + S_R * S_L * (uR[i] - uL[i])) * inv;
    F[4] = 0.f;
  } else {
    if (!(S_R <= 0)) bits |= 4u;
#pragma unroll
    for (int i = 0; i < kDim; ++i) F[i] = FR[i];
  }
  return bits;
}

// isothermal limiter (physics/isothermal.hpp:269-320, etha_minus taken as
// H_minus / BM_dist) for one field; sb_scale = 2 eta / (2 N nu_plus)
// After the NaN test no operand of the min/max below is NaN except
// r * sb_scale (0 * inf, inf * 0), where smin(1, NaN) and fminf(1, NaN) both
// give 1; so the hardware min/max (one instruction) equals the reference's
// compare-and-select form.
__device__ __forceinline__ float iso_limiter_field(float r, float eta, float sb_scale) {
  if (isnan(r)) return 0.f;
  return fmaxf(0.f, fmaxf(fminf(1.f, r * sb_scale), fminf(r, eta)));
}

// h(r) switch and the blended limiter (physics/adiabatic.hpp:685-828).
// On (0, 1) the switch is 1 - tanh(y) = 2 / (1 + e^{2y}) (no cancellation)
// with y = 4 r^2 (1 - r)^0.1; for r >= 1 it is tanh(z)^6 with
// tanh(z) = (e^{2z} - 1) / (e^{2z} + 1), 2z = 20 (r - 1)^3 clamped at 80;
// 0 elsewhere (and for NaN).  Written without branches so that a warp whose
// lanes fall on both sides evaluates one exponential and one reciprocal per
// lane, shared by the two forms, instead of both branches in turn.
__device__ __forceinline__ float limiter_switch(float r) {
  const bool lo = r < 1.f && r > 0.f;
  const bool hi = r >= 1.f;
  // 2y log2(e) and 20 x^3 log2(e), clamped at 80 log2(e): e^{2y} and
  // e^{min(20 x^3, 80)} as powers of two
  const float y2 = (8.f * kLog2e) * (r * r) * ex2_approx(0.1f * lg2_approx(lo ? 1.f - r : 1.f));
  const float x = r - 1.f;
  const float e = ex2_approx(lo ? y2 : fminf((20.f * kLog2e) * (x * x * x), 80.f * kLog2e));
  const float q = __fdividef(1.f, 1.f + e);
  const float t = (e - 1.f) * q;
  const float t2 = t * t;
  return lo ? 2.f * q : (hi ? t2 * t2 * t2 : 0.f);
}

// min/max as in iso_limiter_field: after the NaN test, smin(1, NaN) and
// fminf(1, NaN) agree, and smin(sb, NaN) = fminf(sb, NaN) = sb.
__device__ __forceinline__ float limiter_field(float r, float nu_plus, float eta_p, float sb_scale) {
  if (isnan(r)) return 0.f;
  const float sb = fmaxf(0.f, fmaxf(fminf(1.f, r * sb_scale), fminf(r, eta_p)));
  const float to = fmaxf(0.f, fminf(sb, 1.f + (1.f + nu_plus) * (1.f / 3.f) * (r - 1.f)));
  const float hv = limiter_switch(r);
  return to + hv * (sb - to);
}

// Compensated FP32 accumulator (Neumaier's scheme): the sum of the FP32
// terms is kept as hi + lo (about twice FP32 precision) and folded into FP64
// at the end.  Each addition's exact rounding error comes from Knuth's
// branch-free TwoSum, the same value Neumaier's magnitude test selects.
struct Acc {
  float hi, lo;
  __device__ __forceinline__ void add(float x) {
    const float t = hi + x;
    const float xx = t - hi;
    lo += (hi - (t - xx)) + (x - xx);
    hi = t;
  }
};

}  // namespace mx
}  // namespace splash
