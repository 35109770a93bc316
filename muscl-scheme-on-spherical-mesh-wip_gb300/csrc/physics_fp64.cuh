// FP64 device physics of the MUSCL step: pressures, edge velocities, the
// three Riemann solvers, the blended limiter, the accretion source and the
// dt candidates.
//
// Each function restates one reference function (cited) with the
// reference's operand order.  The state-dependent functions are templates
// over the scalar type: `double` for the time step (the translation units
// that use them are compiled with -fmad=false, so no multiply-add is fused
// and the FP64 path stays within a few ulp of the reference per operation),
// and Dual<N> (dual.cuh) for the tangent-linear and adjoint kernels, whose
// values are computed by the same operations and so follow the same branches.
#pragma once

#include <cmath>
#include <type_traits>

#include "dual.cuh"
#include "layout.hpp"

namespace splash {
namespace f64 {

template <class T>
struct V3 {
  T x, y, z;
};
using D3 = V3<double>;

template <class T>
SPLASH_HD V3<T> v3(const T& x, const T& y, const T& z) {
  return V3<T>{x, y, z};
}
SPLASH_HD D3 d3(double x, double y, double z) { return D3{x, y, z}; }
template <class T>
SPLASH_HD V3<T> sub(const V3<T>& a, const V3<T>& b) {
  return V3<T>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class T>
SPLASH_HD V3<T> sub(const V3<T>& a, const D3& b) {
  return V3<T>{a.x - b.x, a.y - b.y, a.z - b.z};
}
SPLASH_HD D3 sub(const D3& a, const D3& b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T, class S>
SPLASH_HD V3<T> scal(const V3<T>& a, const S& s) {
  return V3<T>{a.x * s, a.y * s, a.z * s};
}
template <class T, class S>
SPLASH_HD V3<T> divs(const V3<T>& a, const S& s) {
  return V3<T>{a.x / s, a.y / s, a.z / s};
}
// vec3d.hpp:56-64 : sqrt(((0 + x^2) + y^2) + z^2)
template <class T>
SPLASH_HD T norm3(const V3<T>& a) {
  T s = a.x * a.x;
  s = s + a.y * a.y;
  s = s + a.z * a.z;
  return sqrt(s);
}
template <class A, class B>
SPLASH_HD auto cross3(const V3<A>& a, const V3<B>& b) -> V3<decltype(a.x * b.x)> {
  using R = decltype(a.x * b.x);
  return V3<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class A, class B>
SPLASH_HD auto dot3(const V3<A>& a, const V3<B>& b) -> decltype(a.x * b.x) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
// std::max / std::min argument semantics
template <class T>
SPLASH_HD T smax(const T& a, const T& b) {
  return (a < b) ? b : a;
}
template <class T>
SPLASH_HD T smin(const T& a, const T& b) {
  return (b < a) ? b : a;
}

// physics/adiabatic.hpp:582-592 (u[4] = energy, |vel| given)
template <class T>
SPLASH_HD T pressure(const T* u, const T& vn, double gam) {
  return smax(T(1e-16), (u[4] - u[0] * (vn * vn) / 2) * (gam - 1));
}

// MUSCL_base.hpp:517-539 (u[4] = energy, r = unit face centre)
template <class T>
SPLASH_HD T pressure_fc(const T* u, const D3& r, double gam) {
  V3<T> vel = cross3(r, v3(u[1], u[2], u[3]));
  vel = scal(vel, 1.0 / (-u[0]));
  const T n = norm3(vel);
  return smax(T(1e-16), (u[4] - u[0] * (n * n) / 2) * (gam - 1));
}

// MUSCL_base.hpp:541-562 (u[4] = pressure, r = unit edge centre)
template <class T>
SPLASH_HD T energy_at_edge(const T* u, const D3& r, double gam) {
  V3<T> vel = cross3(r, v3(u[1], u[2], u[3]));
  vel = scal(vel, 1.0 / (-u[0]));
  const T n = norm3(vel);
  return 1 / (gam - 1) * u[4] + u[0] * (n * n) / 2;
}

// Geometry of one slot as the flux functions see it.
struct SlotGeom {
  D3 ec;       // unit edge centre
  double ecn;  // |ec|
  D3 en;       // edge normal
  D3 nxr;      // cross(en, ec/|ec|)
};

// velocity at the edge: cross(ec, l) / ((-u0) |ec|)   (adiabatic.hpp:375-376)
template <class T>
SPLASH_HD V3<T> edge_vel(const T* u, const SlotGeom& g) {
  const V3<T> v = cross3(g.ec, v3(u[1], u[2], u[3]));
  return scal(v, 1.0 / ((-u[0]) * g.ecn));
}

// physics/adiabatic.hpp:352-392
template <class T>
SPLASH_HD void phys_flux(const T* u, const SlotGeom& g, double gam, T* res) {
  const V3<T> vel = edge_vel(u, g);
  const T PI = pressure(u, norm3(vel), gam);
  const T ndv = dot3(g.en, vel);
  res[0] = u[0] * dot3(vel, g.en);
  res[1] = (u[1] * ndv - g.nxr.x * PI);
  res[2] = (u[2] * ndv - g.nxr.y * PI);
  res[3] = (u[3] * ndv - g.nxr.z * PI);
  res[4] = (u[4] + PI) * dot3(vel, g.en);
}

// physics/adiabatic.hpp:594-683 ; sets nan_flag when a wave speed is NaN
template <class T>
SPLASH_HD void char_vel(const T* uL, const T* uR, const SlotGeom& g, double gam,
                                         T& S_L, T& S_R, bool& nan_flag) {
  const V3<T> vel_l = edge_vel(uL, g);
  const V3<T> vel_r = edge_vel(uR, g);
  const T p_L = pressure(uL, norm3(vel_l), gam);
  const T p_R = pressure(uR, norm3(vel_r), gam);
  const T a_L = sqrt(gam * p_L / uL[0]);
  const T a_R = sqrt(gam * p_R / uR[0]);
  const T p_pvrs = 1 / 2. * (p_L + p_R) -
                   1 / 8. * (dot3(g.en, vel_r) - dot3(g.en, vel_l)) * (uL[0] + uR[0]) * (a_L + a_R);
  const T p_star = smax(T(0.), p_pvrs);
  T q_R = T(1.), q_L = T(1.);
  if (!(p_star <= p_R)) {
    q_R = sqrt(1 + (gam + 1) / (2 * gam) * (p_star / p_R - 1));
    if (is_nan(q_R) || is_inf(q_R)) q_R = T(1.);
  }
  if (!(p_star <= p_L)) {
    q_L = sqrt(1 + (gam + 1) / (2 * gam) * (p_star / p_L - 1));
    if (is_nan(q_L) || is_inf(q_L)) q_L = T(1.);
  }
  S_L = dot3(vel_l, g.en) - a_L * q_L;
  S_R = dot3(vel_r, g.en) + a_R * q_R;
  if (is_nan(S_L) || is_nan(S_R)) nan_flag = true;
}

// Riemann fluxes: HLLE_p.hpp:19-58 (solver 1), HLLC.hpp:138-242 (solver 2),
// HLLCplus.hpp:17-177 (solver 3).  Returns stop bits (STOP_NAN_WAVESPEED,
// STOP_WAVE_ORDER as in splash_gb300.h).
template <class T>
SPLASH_HD unsigned flux_star(const T* uL, const T* uR, const SlotGeom& g, double gam,
                                              int solver, T* F) {
  unsigned bits = 0;
  bool nan_ws = false;
  T S_L, S_R;
  char_vel(uL, uR, g, gam, S_L, S_R, nan_ws);
  if (nan_ws) bits |= 2u;
  T FL[kDim], FR[kDim];
  phys_flux(uL, g, gam, FL);
  phys_flux(uR, g, gam, FR);
  if (solver == 1) {
    if (S_L >= 0) {
#pragma unroll
      for (int i = 0; i < kDim; ++i) F[i] = FL[i];
    } else if (S_L < 0 && S_R > 0) {
      const T inv = 1.0 / (S_R - S_L);
#pragma unroll
      for (int i = 0; i < kDim; ++i) F[i] = (S_R * FL[i] - S_L * FR[i] + S_R * S_L * (uR[i] - uL[i])) * inv;
    } else {
      // S_R <= 0, or NaN wave speeds (reference prints and stops)
      if (!(S_R <= 0)) bits |= 4u;
#pragma unroll
      for (int i = 0; i < kDim; ++i) F[i] = FR[i];
    }
    return bits;
  }
  const V3<T> vel_L = edge_vel(uL, g);
  const V3<T> vel_R = edge_vel(uR, g);
  const T rho_R = uR[0];
  const T rho_L = uL[0];
  const T p_L = pressure(uL, norm3(vel_L), gam);
  const T p_R = pressure(uR, norm3(vel_R), gam);
  const T V_L = dot3(g.en, vel_L);
  const T V_R = dot3(g.en, vel_R);
  T S_star = (p_R - p_L + rho_L * V_L * (S_L - V_L) - rho_R * V_R * (S_R - V_R)) /
             (rho_L * (S_L - V_L) - rho_R * (S_R - V_R));
  if (is_nan(S_star) || is_inf(S_star)) S_star = (V_L + V_R) / 2;
  const T D[kDim] = {T(0.), T(-g.nxr.x), T(-g.nxr.y), T(-g.nxr.z), S_star};
  const T P_LR = (p_L + p_R + uL[0] * (S_L - V_L) * (S_star - V_L) + uR[0] * (S_R - V_R) * (S_star - V_R)) / 2;
  // branch choice of HLLC.hpp:218-239 / HLLCplus.hpp:153-174
  int side;  // 0: F_L, 1: F_L*, 2: F_R*, 3: F_R
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
  if (side == 0) {
#pragma unroll
    for (int i = 0; i < kDim; ++i) F[i] = FL[i];
    return bits;
  }
  if (side == 3) {
#pragma unroll
    for (int i = 0; i < kDim; ++i) F[i] = FR[i];
    return bits;
  }
  const T Sk = (side == 1) ? S_L : S_R;
  const T* uk = (side == 1) ? uL : uR;
  const T* Fk = (side == 1) ? FL : FR;
  const T inv_k = 1.0 / (Sk - S_star);
#pragma unroll
  for (int i = 0; i < kDim; ++i) F[i] = (S_star * (Sk * uk[i] - Fk[i]) + Sk * P_LR * D[i]) * inv_k;
  if (solver == 3) {
    F[0] = F[0] + 0.0;  // flux_fix[0] = 0 is added like the other fields
    const T phi_L = uL[0] * (S_L - V_L);
    const T phi_R = uR[0] * (S_R - V_R);
    const T a_L = sqrt(gam * p_L / uL[0]);
    const T a_R = sqrt(gam * p_R / uR[0]);
    const T M = smin(T(1.), smax(norm3(vel_L) / a_L, norm3(vel_R) / a_R));
    int lambd_L = 0, lambd_R = 0;
    if ((V_L - a_L) > 0 && (V_R - a_R) < 0) lambd_L = 1;
    if ((V_L + a_L) > 0 && (V_R + a_R) < 0) lambd_L = 1;
    if ((V_R - a_R) > 0 && (V_L - a_L) < 0) lambd_R = 1;
    if ((V_R + a_R) > 0 && (V_L + a_L) < 0) lambd_R = 1;
    T f_star = T(1.);
    if (lambd_L == 0 && lambd_R == 0) f_star = M * sqrt(4 + (1 - M * M) * (1 - M * M)) / ((1 + M * M));
    const T h = smin(p_L / p_R, p_R / p_L);
    const T gsw = 1 - exp(M * log(h));
    const T dV = V_R - V_L;
    const V3<T> dv = sub(vel_R, vel_L);
    const T cs = Sk * inv_k * gsw;
    const V3<T> vff = v3((f_star - 1) * dV * g.en.x + cs * (dv.x - dV * g.en.x),
                         (f_star - 1) * dV * g.en.y + cs * (dv.y - dV * g.en.y),
                         (f_star - 1) * dV * g.en.z + cs * (dv.z - dV * g.en.z));
    const V3<T> am = cross3(g.ec, vff);
    const T w = phi_L * phi_R / (phi_R - phi_L);
    F[1] = F[1] + am.x * w;
    F[2] = F[2] + am.y * w;
    F[3] = F[3] + am.z * w;
    F[4] = F[4] + (f_star - 1) * (V_R - V_L) * S_star * w;
  }
  return bits;
}

// h(r) switch of physics/adiabatic.hpp:692-702, evaluated through exact
// identities that cost fewer FP64 instructions than the reference's pow and
// tanh (GB300's FP64 pipe is the bottleneck of this path): pow(1 - r, 0.1)
// = exp(0.1 log(1 - r)), integer powers as products, and for y, z >= 0
//   1 - tanh(y) = 2 / (1 + e^{2y})          (also free of cancellation)
//   tanh(z)     = expm1(2z) / (expm1(2z) + 2),
// with 2z clamped at 80 (tanh(40) is 1 in double; e^{2z} would overflow).
template <class T>
SPLASH_HD T limiter_switch(const T& r) {
  T o = T(0.);
  if (r < 1 && r > 0) {
    const T y = 4 * (r * r) * exp(0.1 * log(1 - r));
    o = 2 / (1 + exp(2 * y));
  }
  if (r >= 1) {
    const T x = r - 1;
    const T em = expm1(smin(20 * ((x * x) * x), T(80.)));
    const T t = em / (em + 2);
    const T t2 = t * t;
    o = (t2 * t2) * t2;
  }
  return o;
}

// physics/adiabatic.hpp:685-828 for one field: blend of the third-order
// limiter and the irregular-grid superbee, NaN ratio -> 0.  sb_scale is
// eta_minus / (2 N nu_plus) and to_scale is (1 + nu_plus) / 3, both per slot.
template <class T>
SPLASH_HD T limiter_field(const T& r, double eta_p, const T& sb_scale, const T& to_scale) {
  if (is_nan(r)) return T(0.);
  if constexpr (is_dual<T>::value) {
    // r = +-inf (a zero forward difference): the limiter is flat there in r
    // and in the Courant factor; the dual chain would form 0 * inf
    if (is_inf(r)) return T(limiter_field<double>(val(r), eta_p, val(sb_scale), val(to_scale)));
  }
  const T sb = smax(T(0.), smax(smin(T(1.), r * sb_scale), smin(r, T(eta_p))));
  const T to = smax(T(0.), smin(sb, 1 + to_scale * (r - 1)));
  const T hv = limiter_switch(r);
  return ((1 - hv) * to + hv * sb);
}

// Per-face contributions to the dt clip of the NEXT step and to the
// diagnostics sums, for a conserved state u (u[4] = energy):
// find_v_max (MUSCL_base.hpp:311-343) and extra_dt_constr
// (physics/adiabatic.hpp:543-580).
SPLASH_HD void dt_candidates(const double* u, D3 r, double area, const PhysParams& P,
                                              double& vmax, double& dmin, double sums[5]) {
  D3 vpos = cross3(r, d3(u[1], u[2], u[3]));
  vpos = divs(vpos, u[0]);
  const double vn = norm3(vpos);
  const double p = pressure_fc(u, r, P.gam);
  const double c_s = sqrt(P.gam * p / u[0]);
  vmax = fmax(vn, c_s);
  // extra_dt_constr
  D3 vel = cross3(r, d3(u[1], u[2], u[3]));
  vel = divs(vel, -u[0]);
  const D3 omega0 = d3(0, 0, P.omega_ns);
  const D3 vel0 = cross3(omega0, r);
  const double nvel = norm3(vel);
  const double press = pressure(u, nvel, P.gam);
  const double GM = 0.217909;
  const double g_eff = GM - nvel * nvel;
  // P.fric_k = gam3d / (2 gam3d - 1), gam3d = 1 / (2 - gam), the same IEEE value
  const double rho = P.fric_k * g_eff * u[0] * u[0] / press;
  dmin = 0.01 * u[0] / (P.alpha * rho * norm3(sub(vel, vel0)));
#pragma unroll
  for (int k = 0; k < 5; ++k) sums[k] = u[k] * area;
}

// The parameters of the source term that the derivative kernels
// differentiate: the face's accretion profile value acc0 (res[0] of
// physics/adiabatic.hpp:415-421), the accretion angular velocity, the
// accretion rate and the initial total mass (both enter the depletion term
// without friction).
template <class Q>
struct SrcParams {
  Q acc0;
  V3<Q> omega_acc;
  Q acc_rate;
  Q total_mass;
};

// physics/adiabatic.hpp:396-541 ; w[4] is the pressure.
template <class T, class Q>
SPLASH_HD void source_term(const T* w, const D3& fcn, const SrcParams<Q>& sp, const PhysParams& P, T* res) {
  const Q& acc0 = sp.acc0;
  const V3<Q>& omega_acc = sp.omega_acc;
#pragma unroll
  for (int i = 0; i < kDim; ++i) res[i] = T(0.);
  if (!P.accretion_on) return;
  V3<T> vel = cross3(fcn, v3(w[1], w[2], w[3]));
  vel = divs(vel, -w[0]);
  res[0] = T(acc0);
  const V3<Q> omxr = cross3(omega_acc, fcn);
  const V3<Q> rxo = cross3(fcn, omxr);
  res[1] = res[0] * rxo.x;
  res[2] = res[0] * rxo.y;
  res[3] = res[0] * rxo.z;
  const T nd = norm3(v3(omxr.x - vel.x, omxr.y - vel.y, omxr.z - vel.z));
  res[4] = res[0] * (P.e_acc + (nd * nd) / 2.);
  const V3<T> rxv = cross3(fcn, vel);
  const T nvel = norm3(vel);
  if (!P.friction_on) {
    const double fall_eff = 1;
    const T dmdt = -(fall_eff * sp.acc_rate * 4 * M_PI) / sp.total_mass * w[0];
    res[0] += dmdt;
    res[1] += dmdt * rxv.x;
    res[2] += dmdt * rxv.y;
    res[3] += dmdt * rxv.z;
    res[4] += dmdt * (P.gam / (P.gam - 1) * w[4] / w[0] + (nvel * nvel) / 2.);
  }
  const double GM = 0.217909;
  const T g_eff = GM - nvel * nvel;
  const double c_sigma = 4.85e36;
  const double k_m = 1.6e-13;
  const double kappa = 3.4e6;
  const T C = 12. / 5 * k_m * w[0] / w[4] * sqrt(sqrt(3. / 4 * c_sigma * g_eff * w[0]));
  const double beta_switch = 0.736194670678821;
  const double C_switch = -1 - 1 / (beta_switch - 1);
  T beta;
  if (C <= C_switch) {
    beta = 1 - 1 / (1 + C);
  } else {
    const T x2 = (2 / C) * (2 / C);
    beta = 1 - x2 * x2;
  }
  const double beta_ceil = 1 - 1e-8, beta_floor = 1e-8;
  if (beta < beta_floor || is_nan(beta)) beta = T(beta_floor);
  if (beta > beta_ceil) beta = T(beta_ceil);
  res[4] -= g_eff / kappa * (1 - beta);
  if (P.friction_on) {
    const T rho = P.fric_k * g_eff * w[0] * w[0] / w[4];  // fric_k = gam3d / (2 gam3d - 1)
    const D3 omega0 = d3(0, 0, P.omega_ns);
    const D3 vel0 = cross3(omega0, fcn);
    const T dv = norm3(sub(vel, vel0));
    const V3<T> wr = scal(sub(vel, vel0), -P.alpha * rho * dv);
    const V3<T> l_fr = cross3(fcn, wr);
    res[1] += l_fr.x;
    res[2] += l_fr.y;
    res[3] += l_fr.z;
    res[4] += dot3(wr, vel0);
    res[0] -= P.alpha * rho * dv;
    res[1] -= P.alpha * rho * dv / w[0] * w[1];
    res[2] -= P.alpha * rho * dv / w[0] * w[2];
    res[3] -= P.alpha * rho * dv / w[0] * w[3];
    res[4] -= P.alpha * rho * dv * (nvel * nvel / 2. + w[4] * P.gam / ((P.gam - 1) * w[0]));
  }
}

}  // namespace f64
}  // namespace splash
