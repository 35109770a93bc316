// FP64 device physics of the isothermal solver MUSCL_HLLE (4 fields:
// Sigma, l_x, l_y, l_z; pressure a^2 Sigma with a = 1).
//
// Each function restates one reference function with the reference's
// operation order, divisions included (this path has no transcendental, so
// exact IEEE division costs little), so that the FP64 kernels reproduce the
// CPU restatement bit for bit.  The reference's isothermal limiter reads an
// uninitialised etha_minus (physics/isothermal.hpp:272, 307); it is taken as
// H_minus / BM_dist (its value in the adiabatic superbee), and etha_plus keeps
// its value as written (H_minus / BM_dist, isothermal.hpp:301-302).
#pragma once

#include "dual.cuh"
#include "physics_fp64.cuh"

namespace splash {
namespace iso {

using f64::D3;
using f64::cross3;
using f64::d3;
using f64::dot3;
using f64::norm3;
using f64::smax;
using f64::smin;

constexpr int kIsoDim = 4;
constexpr double kA = 1;  // isothermal sound speed (isothermal.hpp:138)

SPLASH_HD D3 div3(const D3& a, double s) { return D3{a.x / s, a.y / s, a.z / s}; }

// physics/isothermal.hpp:141-195 ; ec is the unit edge centre
SPLASH_HD void flux(const double* u, const D3& ec, const D3& en, double* res) {
  const double PI = kA * kA * u[0];
  const D3 vel = div3(cross3(ec, d3(u[1], u[2], u[3])), -u[0]);
  const double ndv = dot3(en, vel);
  const D3 nxR = cross3(en, ec);
  res[0] = u[0] * dot3(vel, en);
  res[1] = u[1] * ndv - nxR.x * PI;
  res[2] = u[2] * ndv - nxR.y * PI;
  res[3] = u[3] * ndv - nxR.z * PI;
}

// physics/isothermal.hpp:211-260 ; ecn = |ec| as evaluated in double
SPLASH_HD void char_vel(const double* uL, const double* uR, const D3& ec, double ecn, const D3& en, double& S_L,
                        double& S_R) {
  const D3 vel_l = div3(cross3(ec, d3(uL[1], uL[2], uL[3])), (-uL[0]) * ecn);
  const D3 vel_r = div3(cross3(ec, d3(uR[1], uR[2], uR[3])), (-uR[0]) * ecn);
  const double vl = dot3(vel_l, en), vr = dot3(vel_r, en);
  const double a_L = kA, a_R = kA;
  S_L = smin(vl, vr) - smax(a_L, a_R);
  S_R = smax(vl, vr) + smax(a_L, a_R);
}

// Riemann_solvers/HLLE.hpp:17-59 ; returns the stop bits of splash_gb300.h
// (2 NaN wave speed, 4 wave ordering)
SPLASH_HD unsigned flux_star(const double* uL, const double* uR, const D3& ec, double ecn, const D3& en,
                             double* F) {
  double S_L, S_R, FL[kIsoDim], FR[kIsoDim];
  char_vel(uL, uR, ec, ecn, en, S_L, S_R);
  flux(uL, ec, en, FL);
  flux(uR, ec, en, FR);
  unsigned bits = (is_nan(S_L) || is_nan(S_R)) ? 2u : 0u;
  if (S_L >= 0) {
#pragma unroll
    for (int i = 0; i < kIsoDim; ++i) F[i] = FL[i];
  } else if (S_L < 0 && S_R > 0) {
#pragma unroll
    for (int i = 0; i < kIsoDim; ++i) F[i] = (S_R * FL[i] - S_L * FR[i] + S_R * S_L * (uR[i] - uL[i])) / (S_R - S_L);
  } else {
    if (!(S_R <= 0)) bits |= 4u;
#pragma unroll
    for (int i = 0; i < kIsoDim; ++i) F[i] = FR[i];
  }
  return bits;
}

// physics/isothermal.hpp:269-320 for one field, given the slot's Courant
// factor nu_plus, eta = H_minus / BM_dist and 2 N (N the face's edge count)
SPLASH_HD double limiter_field(double r, double eta, double twoN, double nu_plus) {
  if (is_nan(r)) return 0.;
  return smax(0., smax(smin(1., eta * r * 2 / (twoN * nu_plus)), smin(r, eta)));
}

// Courant factor of the isothermal limiter: (a + v.n) dt arc / area with
// v = cross(ec, l) / (-Sigma) of the face state w
SPLASH_HD double courant(const double* w, const D3& ec, const D3& en, double dt, double arc_a) {
  const D3 vel = div3(cross3(ec, d3(w[1], w[2], w[3])), -w[0]);
  return (kA + dot3(vel, en)) * dt * arc_a;
}

// find_v_max (MUSCL_base.hpp:311-343) of a 4-field state: the CFL speed is
// max(|v|, a) (the reference reads a fifth field for the sound speed); the
// extra constraint is 1e20 (isothermal.hpp:262-267).
SPLASH_HD void dt_candidates(const double* u, const D3& r, double area, double& vmax, double& dmin,
                             double sums[5]) {
  const D3 vel = div3(cross3(r, d3(u[1], u[2], u[3])), u[0]);
  vmax = fmax(norm3(vel), kA);
  dmin = 1e20;
#pragma unroll
  for (int k = 0; k < kIsoDim; ++k) sums[k] = u[k] * area;
  sums[4] = 0.0;
}

}  // namespace iso
}  // namespace splash
