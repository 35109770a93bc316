// SPLASH MUSCL time step — CPU restatement used as the TEST ORACLE.
//
// This file is test infrastructure.  Only tests/, __graft_entry__.smoke()
// and the CPU-baseline leg of bench.py load it (as liboracle.so through
// oracle/oracle.py); the product library never links or calls it.
//
// It restates, in plain C++ with OpenMP, the reference's FP64 algorithm for
// one do_step(dt0), function by function, keeping the reference's
// floating-point evaluation order so that (built with -ffp-contract=off
// against the same libm) it reproduces the reference bit for bit:
//
//   do_step ..................... MUSCL_base/MUSCL_base.hpp:97-225
//   res2d ....................... MUSCL_base/MUSCL_base.hpp:238-276
//   find_v_max / pressure_fc .... MUSCL_base/MUSCL_base.hpp:311-343, 517-539
//   find_flux_var ............... MUSCL_base/MUSCL_base.hpp:345-359
//   find_U_edges, p_plus/minus .. MUSCL_base/MUSCL_base.hpp:361-515
//   E_fc ........................ MUSCL_base/MUSCL_base.hpp:541-562
//   flux ........................ physics/adiabatic.hpp:352-392
//   source ...................... physics/adiabatic.hpp:396-541
//   extra_dt_constr ............. physics/adiabatic.hpp:543-580
//   pressure, char_vel .......... physics/adiabatic.hpp:582-683
//   limiter (blend, 3rd order,
//            superbee) ......... physics/adiabatic.hpp:685-828
//   flux_star HLLE_p ............ Riemann_solvers/HLLE_p.hpp:19-58
//   flux_star HLLC .............. Riemann_solvers/HLLC.hpp:138-242
//   flux_star HLLC+ ............. Riemann_solvers/HLLCplus.hpp:17-177
//   area_coeff, total_mass ...... physics/adiabatic.hpp:70-90
//
// and the isothermal solver MUSCL_HLLE (dim 4, solver kind 4):
//   flux ........................ physics/isothermal.hpp:141-195
//   source (zero) ............... physics/isothermal.hpp:199-208
//   char_vel .................... physics/isothermal.hpp:211-260
//   extra_dt_constr (1e20) ...... physics/isothermal.hpp:262-267
//   limiter ..................... physics/isothermal.hpp:269-320
//   flux_star HLLE .............. Riemann_solvers/HLLE.hpp:17-59
//
// Geometry arrays are taken in the reference numbering (the layout of
// geometry/MUSCL_geometry.hpp:23-40 flattened per slot); they are produced by
// the library's host geometry builder, which the test-suite pins bit-exactly
// against the reference's own members.
//
// Reference defects restated in a defined form:
//   * the area_coeff loop counter is uninitialised (adiabatic.hpp:75); it is
//     taken to start at 0 (the built reference behaves that way);
//   * the static mass counters in source() (adiabatic.hpp:400-401,452,536)
//     are racy and never read; they are omitted;
//   * the isothermal path (dim 4) reads and writes a fifth state field that
//     a 4-field state does not have (MUSCL_base.hpp:203, 324, 368-370, 538)
//     and its limiter reads an uninitialised etha_minus (isothermal.hpp:272,
//     307).  Restated: no fifth field (no E <-> Pi conversion, no energy
//     sum), the CFL sound speed of find_v_max is the isothermal a = 1 (the
//     speed the isothermal char_vel and limiter use), etha_minus is
//     H_minus / BM_dist (its value in the adiabatic superbee,
//     adiabatic.hpp:813) and etha_plus keeps its value as written (the
//     second assignment, H_minus / BM_dist, isothermal.hpp:301-302).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V {
  double x, y, z;
};
inline V mk(const double* p) { return {p[0], p[1], p[2]}; }
inline V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V operator*(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V operator/(V a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double norm(V a) {  // vec3d.hpp:56-64
  double s = 0.0;
  s += a.x * a.x;
  s += a.y * a.y;
  s += a.z * a.z;
  return std::sqrt(s);
}
inline V cross(V a, V b) {  // MUSCL_geometry.hpp:1154-1162
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double gc_distance(V a, V b) {  // MUSCL_geometry.hpp:981-987
  a = a / norm(a);
  b = b / norm(b);
  const double d = norm(a - b);
  return 2 * std::asin(d / 2);
}
// std::max / std::min semantics (first argument returned on ties and NaN
// comparisons)
inline double smax(double a, double b) { return (a < b) ? b : a; }
inline double smin(double a, double b) { return (b < a) ? b : a; }

constexpr int kMaxDim = 5;

struct Oracle {
  // geometry, reference numbering
  int nf = 0, ns = 0, nv = 0;
  std::vector<double> vertices;
  std::vector<int> face_off, face_vtx, nbr_edge, rev_slot;
  std::vector<double> face_centers, area, edge_normals, bm, hp, hm, bp, bmn;
  std::vector<int> ffp, ffm;
  double h0 = 0, round_diff = 0;

  // physics
  int dim = 5;
  double gam = 1.25, omega_ns = 0;
  bool accretion_on = false, friction_on = true;
  double acc_rate = 0, e_acc = 0, omega_acc_abs = 0, tilt_angle = 0, acc_width = 0.1, alpha = 1e-6;
  double area_coeff = 0, total_mass = 0;
  int solver = 3;  // 1 HLLE_p, 2 HLLC, 3 HLLC+, 4 HLLE (isothermal, dim 4)
  static constexpr double a_iso = 1;  // isothermal sound speed (isothermal.hpp:138)
  bool iso() const { return solver == 4; }

  // state
  std::vector<double> U, U_temp, source_plus, U_plus, U_minus, flux_var;
  double t = 0, dt = 0, max_vel = 0;
  int64_t steps = 0;
  bool stop_check = false;
  double diag[5] = {0, 0, 0, 0, 0};

  int nsl(int f) const { return face_off[f + 1] - face_off[f]; }
  V vtx(int v) const { return mk(&vertices[3 * (size_t)v]); }
  V fc(int f) const { return mk(&face_centers[3 * (size_t)f]); }
  V en(int s) const { return mk(&edge_normals[3 * (size_t)s]); }
  int vslot(int f, int j) const { return face_vtx[face_off[f] + j]; }
  int vslot1(int f, int j) const { return face_vtx[face_off[f] + ((j + 1 == nsl(f)) ? 0 : j + 1)]; }

  // edge_center of flux/char_vel/limiter: ((a+b)/2)/|(a+b)/2|
  V edge_center(int f, int j) const {
    V e = (vtx(vslot(f, j)) + vtx(vslot1(f, j))) / 2.;
    return e / norm(e);
  }

  // ---- physics/adiabatic.hpp:582-592
  double pressure(const double* u, V vel) const {
    const double n = norm(vel);
    return smax(1e-16, (u[4] - u[0] * (n * n) / 2) * (gam - 1));
  }
  // ---- MUSCL_base.hpp:517-539 (u[4] is the energy)
  double pressure_fc(const double* u, int f) const {
    V r = fc(f);
    r = r / norm(r);
    V vel = cross(r, V{u[1], u[2], u[3]});
    vel = vel / (-u[0]);
    const double n = norm(vel);
    return smax(1e-16, (u[4] - u[0] * (n * n) / 2) * (gam - 1));
  }
  // ---- MUSCL_base.hpp:541-562 (u[4] is the pressure)
  double E_fc(const double* u, int f, int j) const {
    V r = vtx(vslot(f, j)) + vtx(vslot1(f, j));
    r = r / norm(r);
    V vel = cross(r, V{u[1], u[2], u[3]});
    vel = vel / (-u[0]);
    const double n = norm(vel);
    return 1 / (gam - 1) * u[4] + u[0] * (n * n) / 2;
  }
  // velocity at the edge centre: cross(ec, l) / ((-u0) |ec|)
  V edge_vel(const double* u, V ec) const {
    V vel = cross(ec, V{u[1], u[2], u[3]});
    return vel / ((-u[0]) * norm(ec));
  }
  // ---- physics/adiabatic.hpp:352-392
  void flux(const double* u, int f, int j, double* res) const {
    const V ec = edge_center(f, j);
    const V vel = edge_vel(u, ec);
    const double PI = pressure(u, vel);
    const V n = en(face_off[f] + j);
    const double ndv = dot(n, vel);
    const V nxR = cross(n, ec / norm(ec));
    res[0] = u[0] * dot(vel, n);
    res[1] = (u[1] * ndv - nxR.x * PI);
    res[2] = (u[2] * ndv - nxR.y * PI);
    res[3] = (u[3] * ndv - nxR.z * PI);
    res[4] = (u[4] + PI) * dot(vel, n);
  }
  // ---- physics/adiabatic.hpp:594-683 ; returns the NaN flag
  bool char_vel(const double* uL, const double* uR, int f, int j, double& S_L, double& S_R) const {
    const V ec = edge_center(f, j);
    const V vel_l = edge_vel(uL, ec);
    const V vel_r = edge_vel(uR, ec);
    const double p_L = pressure(uL, vel_l);
    const double p_R = pressure(uR, vel_r);
    const double a_L = std::sqrt(gam * p_L / uL[0]);
    const double a_R = std::sqrt(gam * p_R / uR[0]);
    const V n = en(face_off[f] + j);
    const double p_pvrs = 1 / 2. * (p_L + p_R) -
                          1 / 8. * (dot(n, vel_r) - dot(n, vel_l)) * (uL[0] + uR[0]) * (a_L + a_R);
    const double p_star = smax(0., p_pvrs);
    double q_R, q_L;
    if (p_star <= p_R) {
      q_R = 1;
    } else {
      q_R = std::sqrt(1 + (gam + 1) / (2 * gam) * (p_star / p_R - 1));
      if (std::isnan(q_R) || std::isinf(q_R)) q_R = 1;
    }
    if (p_star <= p_L) {
      q_L = 1;
    } else {
      q_L = std::sqrt(1 + (gam + 1) / (2 * gam) * (p_star / p_L - 1));
      if (std::isnan(q_L) || std::isinf(q_L)) q_L = 1;
    }
    S_L = dot(vel_l, n) - a_L * q_L;
    S_R = dot(vel_r, n) + a_R * q_R;
    return std::isnan(S_L) || std::isnan(S_R);
  }

  // ---- physics/isothermal.hpp:141-195 (4 fields)
  void iso_flux(const double* u, int f, int j, double* res) const {
    const int s = face_off[f] + j;
    const V ec = edge_center(f, j);
    const double PI = a_iso * a_iso * u[0];
    V vel = cross(ec, V{u[1], u[2], u[3]});
    vel = vel / (-u[0]);
    const double ndv = dot(en(s), vel);
    const V nxR = cross(en(s), ec);
    res[0] = u[0] * dot(vel, en(s));
    res[1] = u[1] * ndv - nxR.x * PI;
    res[2] = u[2] * ndv - nxR.y * PI;
    res[3] = u[3] * ndv - nxR.z * PI;
  }
  // ---- physics/isothermal.hpp:211-260
  void iso_char_vel(const double* uL, const double* uR, int f, int j, double& S_L, double& S_R) const {
    const int s = face_off[f] + j;
    const V ec = edge_center(f, j);
    V vel_l = cross(ec, V{uL[1], uL[2], uL[3]});
    vel_l = vel_l / ((-uL[0]) * norm(ec));
    V vel_r = cross(ec, V{uR[1], uR[2], uR[3]});
    vel_r = vel_r / ((-uR[0]) * norm(ec));
    const double vl = dot(vel_l, en(s)), vr = dot(vel_r, en(s));
    S_L = smin(vl, vr) - smax(a_iso, a_iso);
    S_R = smax(vl, vr) + smax(a_iso, a_iso);
  }
  // ---- Riemann_solvers/HLLE.hpp:17-59 ; returns stop bits (2 = order)
  int iso_flux_star(const double* uL, const double* uR, int f, int j, double* F) const {
    double S_L, S_R, FL[4], FR[4];
    iso_char_vel(uL, uR, f, j, S_L, S_R);
    iso_flux(uL, f, j, FL);
    iso_flux(uR, f, j, FR);
    int bits = (std::isnan(S_L) || std::isnan(S_R)) ? 1 : 0;
    if (S_L >= 0) {
      for (int i = 0; i < 4; ++i) F[i] = FL[i];
    } else if (S_L < 0 && S_R > 0) {
      for (int i = 0; i < 4; ++i) F[i] = (S_R * FL[i] - S_L * FR[i] + S_R * S_L * (uR[i] - uL[i])) / (S_R - S_L);
    } else if (S_R <= 0) {
      for (int i = 0; i < 4; ++i) F[i] = FR[i];
    } else {
      for (int i = 0; i < 4; ++i) F[i] = FR[i];
      bits |= 2;
    }
    return bits;
  }
  // ---- physics/isothermal.hpp:269-320 (defined form, see the header)
  void iso_limiter(const double* r, const double* w, int f, int j, double* res) const {
    const int s = face_off[f] + j;
    const V ec = edge_center(f, j);
    V vel = cross(ec, V{w[1], w[2], w[3]});
    vel = vel / (-w[0]);
    const double c = a_iso;
    const double nu_plus = (c + dot(vel, en(s))) * dt *
                           (gc_distance(vtx(vslot(f, j)), vtx(vslot1(f, j))) / area[f]);
    const double etha_plus = hm[s] / bm[s];
    const double etha_minus = hm[s] / bm[s];
    const double twoN = (double)(2 * (size_t)nsl(f));
    for (int i = 0; i < 4; ++i) {
      res[i] = smax(0., smax(smin(1., etha_minus * r[i] * 2 / (twoN * nu_plus)), smin(r[i], etha_plus)));
      if (std::isnan(r[i])) res[i] = 0;
    }
  }

  // ---- Riemann solvers; returns stop bits (1 = NaN wave speed, 2 = order)
  int flux_star(const double* uL, const double* uR, int f, int j, double* F) const {
    if (iso()) return iso_flux_star(uL, uR, f, j, F);
    int bits = 0;
    double S_L, S_R;
    if (solver == 1) {  // HLLE_p.hpp:19-58
      if (char_vel(uL, uR, f, j, S_L, S_R)) bits |= 1;
      double FL[kMaxDim], FR[kMaxDim];
      flux(uL, f, j, FL);
      flux(uR, f, j, FR);
      if (S_L >= 0) {
        for (int i = 0; i < dim; ++i) F[i] = FL[i];
      } else if (S_L < 0 && S_R > 0) {
        for (int i = 0; i < dim; ++i)
          F[i] = (S_R * FL[i] - S_L * FR[i] + S_R * S_L * (uR[i] - uL[i])) / (S_R - S_L);
      } else if (S_R <= 0) {
        for (int i = 0; i < dim; ++i) F[i] = FR[i];
      } else {
        for (int i = 0; i < dim; ++i) F[i] = FR[i];
        bits |= 2;
      }
      return bits;
    }
    // HLLC (HLLC.hpp:138-242) and HLLC+ (HLLCplus.hpp:17-177)
    const V ec = edge_center(f, j);
    const V vel_L = edge_vel(uL, ec);
    const V vel_R = edge_vel(uR, ec);
    if (char_vel(uL, uR, f, j, S_L, S_R)) bits |= 1;
    const V n = en(face_off[f] + j);
    const V nxR = cross(n, ec / norm(ec));
    double D[kMaxDim] = {0, -nxR.x, -nxR.y, -nxR.z, 0};
    double F_L[kMaxDim], F_R[kMaxDim];
    flux(uL, f, j, F_L);
    flux(uR, f, j, F_R);
    const double rho_R = uR[0];
    const double rho_L = uL[0];
    const double p_L = pressure(uL, vel_L);
    const double p_R = pressure(uR, vel_R);
    const double V_L = dot(n, vel_L);
    const double V_R = dot(n, vel_R);
    double S_star = (p_R - p_L + rho_L * V_L * (S_L - V_L) - rho_R * V_R * (S_R - V_R)) /
                    (rho_L * (S_L - V_L) - rho_R * (S_R - V_R));
    if (std::isnan(S_star) || std::isinf(S_star)) S_star = (V_L + V_R) / 2;
    D[4] = S_star;
    const double P_LR = (p_L + p_R + uL[0] * (S_L - dot(n, vel_L)) * (S_star - dot(n, vel_L)) +
                         uR[0] * (S_R - dot(n, vel_R)) * (S_star - dot(n, vel_R))) /
                        2;
    double fixL[kMaxDim] = {0, 0, 0, 0, 0}, fixR[kMaxDim] = {0, 0, 0, 0, 0};
    if (solver == 3) {
      const double phi_L = uL[0] * (S_L - V_L);
      const double phi_R = uR[0] * (S_R - V_R);
      const double a_L = std::sqrt(gam * p_L / uL[0]);
      const double a_R = std::sqrt(gam * p_R / uR[0]);
      const double M = smin(1., smax(norm(vel_L) / a_L, norm(vel_R) / a_R));
      int lambd_L = 0, lambd_R = 0;
      if ((V_L - a_L) > 0 && (V_R - a_R) < 0) lambd_L = 1;
      if ((V_L + a_L) > 0 && (V_R + a_R) < 0) lambd_L = 1;
      if ((V_R - a_R) > 0 && (V_L - a_L) < 0) lambd_R = 1;
      if ((V_R + a_R) > 0 && (V_L + a_L) < 0) lambd_R = 1;
      double f_star = 1;
      if (lambd_L == 0 && lambd_R == 0)
        f_star = M * std::sqrt(4 + (1 - M * M) * (1 - M * M)) / ((1 + M * M));
      const double h = smin(p_L / p_R, p_R / p_L);
      const double g = 1 - std::pow(h, M);
      const double nn[3] = {n.x, n.y, n.z};
      const double vl[3] = {vel_L.x, vel_L.y, vel_L.z};
      const double vr[3] = {vel_R.x, vel_R.y, vel_R.z};
      double vffL[3], vffR[3];
      for (int k = 0; k < 3; ++k) {
        vffL[k] = (f_star - 1) * (V_R - V_L) * nn[k] +
                  S_L / (S_L - S_star) * g * (vr[k] - vl[k] - (V_R - V_L) * nn[k]);
        vffR[k] = (f_star - 1) * (V_R - V_L) * nn[k] +
                  S_R / (S_R - S_star) * g * (vr[k] - vl[k] - (V_R - V_L) * nn[k]);
      }
      const V amL = cross(ec, V{vffL[0], vffL[1], vffL[2]});
      const V amR = cross(ec, V{vffR[0], vffR[1], vffR[2]});
      fixL[1] = amL.x * phi_L * phi_R / (phi_R - phi_L);
      fixR[1] = amR.x * phi_L * phi_R / (phi_R - phi_L);
      fixL[2] = amL.y * phi_L * phi_R / (phi_R - phi_L);
      fixR[2] = amR.y * phi_L * phi_R / (phi_R - phi_L);
      fixL[3] = amL.z * phi_L * phi_R / (phi_R - phi_L);
      fixR[3] = amR.z * phi_L * phi_R / (phi_R - phi_L);
      fixL[4] = (f_star - 1) * (V_R - V_L) * S_star * phi_L * phi_R / (phi_R - phi_L);
      fixR[4] = (f_star - 1) * (V_R - V_L) * S_star * phi_L * phi_R / (phi_R - phi_L);
    }
    double FLs[kMaxDim], FRs[kMaxDim];
    for (int i = 0; i < dim; ++i) {
      FLs[i] = (S_star * (S_L * uL[i] - F_L[i]) + S_L * P_LR * D[i]) / (S_L - S_star);
      FRs[i] = (S_star * (S_R * uR[i] - F_R[i]) + S_R * P_LR * D[i]) / (S_R - S_star);
      if (solver == 3) {
        FLs[i] = FLs[i] + fixL[i];
        FRs[i] = FRs[i] + fixR[i];
      }
    }
    const double* src;
    if (S_L >= 0) {
      src = F_L;
    } else if (S_L < 0 && S_star >= 0) {
      src = FLs;
    } else if (S_star < 0 && S_R >= 0) {
      src = FRs;
    } else if (S_R < 0) {
      src = F_R;
    } else {
      src = F_R;
      bits |= 2;
    }
    for (int i = 0; i < dim; ++i) F[i] = src[i];
    return bits;
  }

  // ---- physics/adiabatic.hpp:685-828 ; w = U[face] with w[4] the pressure
  void limiter(const double* r, const double* w, int f, int j, double* res) const {
    if (iso()) {
      iso_limiter(r, w, f, j, res);
      return;
    }
    auto h = [](double x) {
      double o = 0;
      if (x < 1 && x > 0) o = (1 - std::tanh(4 * std::pow(x, 2.0) * std::pow(1 - x, 0.1)));
      if (x >= 1) o = std::pow(std::tanh(10 * std::pow(x - 1, 3.0)), 6.0);
      return o;
    };
    const int s = face_off[f] + j;
    const V ec = edge_center(f, j);
    V vel = cross(ec, V{w[1], w[2], w[3]});
    vel = vel / ((-w[0] - 0.0) * norm(ec));
    const double p = w[4] + 0.0;
    const double c = std::sqrt(gam * p / (w[0] + 0.0));
    const double arc = gc_distance(vtx(vslot(f, j)), vtx(vslot1(f, j)));
    const double nu_plus = (c + dot(vel, en(s))) * dt * (arc / area[f]);
    const double etha_plus = hp[s] / bm[s];
    const double etha_minus = hm[s] / bm[s];
    const double twoN = (double)(2 * (size_t)nsl(f));
    for (int i = 0; i < dim; ++i) {
      double sb = smax(0., smax(smin(1., etha_minus * r[i] / (twoN * nu_plus)), smin(r[i], etha_plus)));
      if (std::isnan(r[i])) sb = 0;
      double to = smax(0., smin(sb, 1 + (1 + nu_plus) / 3 * (r[i] - 1)));
      if (std::isnan(r[i])) to = 0;
      const double hv = h(r[i]);
      res[i] = ((1 - hv) * to + hv * sb);
      if (std::isnan(r[i])) res[i] = 0;
    }
  }

  // ---- physics/adiabatic.hpp:396-541 ; u[4] is the pressure
  void source(const double* u, int f, double* res) const {
    for (int i = 0; i < dim; ++i) res[i] = 0;
    if (iso()) return;  // isothermal.hpp:199-208
    V fcn = fc(f);
    fcn = fcn / norm(fcn);
    V vel = cross(fcn, V{u[1], u[2], u[3]});
    vel = vel / (-u[0]);
    const double mu = M_PI / 2;
    const double sigma = acc_width / 2.355;
    const double theta_acc = std::acos(fcn.y * std::sin(tilt_angle) + fcn.z * std::cos(tilt_angle));
    if (!accretion_on) return;
    res[0] = 1 / area_coeff * acc_rate / std::sqrt(2 * M_PI * sigma * sigma) *
             std::exp(-(theta_acc - mu) * (theta_acc - mu) / (2 * sigma * sigma));
    const V omega_acc{0, std::sin(tilt_angle) * omega_acc_abs, std::cos(tilt_angle) * omega_acc_abs};
    const V omxr = cross(omega_acc, fcn);
    V rxv = cross(fcn, omxr);
    res[1] = res[0] * rxv.x;
    res[2] = res[0] * rxv.y;
    res[3] = res[0] * rxv.z;
    const double nd = norm(omxr - vel);
    res[4] = res[0] * (e_acc + (nd * nd) / 2.);
    const double fall_eff = 1;
    rxv = cross(fcn, vel);
    const double nvel = norm(vel);
    if (!friction_on) {
      const double dmdt = -(fall_eff * acc_rate * 4 * M_PI) / total_mass * u[0];
      res[0] += dmdt;
      res[1] += dmdt * rxv.x;
      res[2] += dmdt * rxv.y;
      res[3] += dmdt * rxv.z;
      res[4] += dmdt * (gam / (gam - 1) * u[4] / u[0] + (nvel * nvel) / 2.);
    }
    const double GM = 0.217909;
    const double g_eff = GM - nvel * nvel;
    const double c_sigma = 4.85e36;
    const double k_m = 1.6e-13;
    const double kappa = 3.4e6;
    const double C = 12. / 5 * k_m * u[0] / u[4] * std::pow(3. / 4 * c_sigma * g_eff * u[0], 1. / 4);
    const double beta_switch = 0.736194670678821;
    const double C_switch = -1 - 1 / (beta_switch - 1);
    double beta;
    if (C <= C_switch)
      beta = 1 - 1 / (1 + C);
    else
      beta = 1 - std::pow(2 / C, 4.0);
    const double beta_ceil = 1 - 1e-8, beta_floor = 1e-8;
    if (beta < beta_floor || std::isnan(beta)) beta = beta_floor;
    if (beta > beta_ceil) beta = beta_ceil;
    res[4] -= g_eff / kappa * (1 - beta);
    if (friction_on) {
      const double gam3d = 1 / (2 - gam);
      const double rho = gam3d / (2 * gam3d - 1) * g_eff * u[0] * u[0] / u[4];
      const V omega0{0, 0, omega_ns};
      const V vel0 = cross(omega0, fcn);
      V wr = vel - vel0;
      wr = wr * (-alpha * rho * norm(vel - vel0));
      const V l_fr = cross(fcn, wr);
      res[1] += l_fr.x;
      res[2] += l_fr.y;
      res[3] += l_fr.z;
      res[4] += dot(wr, vel0);
      const double dv = norm(vel - vel0);
      res[0] -= alpha * rho * dv;
      res[1] -= alpha * rho * dv / u[0] * u[1];
      res[2] -= alpha * rho * dv / u[0] * u[2];
      res[3] -= alpha * rho * dv / u[0] * u[3];
      res[4] -= alpha * rho * dv * (nvel * nvel / 2. + u[4] * gam / ((gam - 1) * u[0]));
    }
  }

  // ---- physics/adiabatic.hpp:543-580 (u[4] is the energy)
  double extra_dt_constr() {
    double dt_new = 1e20;
    if (iso()) return dt_new;  // isothermal.hpp:262-267
    for (int i = 0; i < nf; ++i) {
      const double* u = &U[(size_t)i * dim];
      V fcn = fc(i);
      fcn = fcn / norm(fcn);
      V vel = cross(fcn, V{u[1], u[2], u[3]});
      vel = vel / (-u[0]);
      const V omega0{0, 0, omega_ns};
      const V vel0 = cross(omega0, fcn);
      const double press = pressure(u, vel);
      const double gam3d = 1 / (2 - gam);
      const double GM = 0.217909;
      const double nvel = norm(vel);
      const double g_eff = GM - nvel * nvel;
      const double rho = gam3d / (2 * gam3d - 1) * g_eff * u[0] * u[0] / press;
      const double cand = 0.01 * u[0] / (alpha * rho * norm(vel - vel0));
      if (dt_new > cand) dt_new = cand;
    }
    if (dt_new < 0) {
      stop_check = true;
      dt_new = 1e20;
    }
    return dt_new;
  }

  // ---- MUSCL_base.hpp:311-343
  void find_v_max() {
    double mx = 1e-8;
    for (int i = 0; i < nf; ++i) {
      const double* u = &U[(size_t)i * dim];
      V r = fc(i);
      r = r / norm(r);
      V vel = cross(r, V{u[1], u[2], u[3]});
      vel = vel / u[0];
      // isothermal: the sound speed a (the reference reads a fifth field here)
      const double c_s = iso() ? a_iso : std::sqrt(gam * pressure_fc(u, i) / u[0]);
      if (norm(vel) > mx) mx = norm(vel);
      if (c_s > mx) mx = c_s;
    }
    max_vel = mx;
  }

  // ---- MUSCL_base.hpp:361-434
  void find_U_edges() {
    for (int i = 0; i < nf; ++i) {
      double* u = &U[(size_t)i * dim];
      if (iso()) {
        u[0] -= 0.0;  // rho_an
        continue;
      }
      u[4] = pressure_fc(u, i);
      u[0] -= 0.0;  // rho_an
      u[4] -= 0.0;  // p_an
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
      const double* ui = &U[(size_t)i * dim];
      for (int j = 0; j < nsl(i); ++j) {
        const int s = face_off[i] + j;
        double pp[kMaxDim], pm[kMaxDim], r[kMaxDim], lim[kMaxDim];
        const double* ua = &U[(size_t)ffp[2 * s] * dim];
        const double* ub = &U[(size_t)ffp[2 * s + 1] * dim];
        const double* uc = &U[(size_t)ffm[2 * s] * dim];
        const double* ud = &U[(size_t)ffm[2 * s + 1] * dim];
        for (int k = 0; k < dim; ++k) {
          const double Up = bp[2 * s] * ua[k] + bp[2 * s + 1] * ub[k];
          pp[k] = (Up - ui[k]) / hp[s];
          const double Um = bmn[2 * s] * uc[k] + bmn[2 * s + 1] * ud[k];
          pm[k] = (-Um + ui[k]) / hm[s];
        }
        for (int k = 0; k < dim; ++k) r[k] = pm[k] / pp[k];
        limiter(r, ui, i, j, lim);
        double* up = &U_plus[(size_t)s * dim];
        for (int k = 0; k < dim; ++k) {
          if (k == 0) {
            up[k] = ui[k] + 0.0 + pp[k] * lim[k] * bm[s];
          } else if (k == 4) {
            up[k] = ui[k] + 0.0 + pp[k] * lim[k] * bm[s];
            up[k] = E_fc(up, i, j);
          } else {
            up[k] = ui[k] + pp[k] * lim[k] * bm[s];
          }
        }
        double* um = &U_minus[(size_t)rev_slot[s] * dim];
        for (int k = 0; k < dim; ++k) um[k] = up[k];
      }
    }
  }

  // ---- MUSCL_base.hpp:345-359 ; returns stop bits
  int find_flux_var() {
    int bits = 0;
#pragma omp parallel for schedule(static) reduction(| : bits)
    for (int i = 0; i < nf; ++i) {
      for (int j = 0; j < nsl(i); ++j) {
        const int s = face_off[i] + j;
        bits |= flux_star(&U_plus[(size_t)s * dim], &U_minus[(size_t)s * dim], i, j,
                          &flux_var[(size_t)s * dim]);
      }
      source(&U[(size_t)i * dim], i, &source_plus[(size_t)i * dim]);
    }
    return bits;
  }

  // ---- MUSCL_base.hpp:238-276 ; returns true on a NaN flux
  bool res2d(double dt_here) {
    bool nan = false;
#pragma omp parallel for schedule(static) reduction(|| : nan)
    for (int i = 0; i < nf; ++i) {
      double* u = &U[(size_t)i * dim];
      for (int k = 0; k < dim; ++k) u[k] = dt_here * source_plus[(size_t)i * dim + k];
      for (int j = 0; j < nsl(i); ++j) {
        const int s = face_off[i] + j;
        const double chord = norm(vtx(vslot(i, j)) - vtx(vslot1(i, j)));
        for (int k = 0; k < dim; ++k) {
          const double F = flux_var[(size_t)s * dim + k];
          if (std::isnan(F)) nan = true;
          u[k] -= round_diff * dt_here * chord / area[i] * F;
        }
      }
    }
    return nan;
  }

  void combine() {
    for (int i = 0; i < nf; ++i) {
      double* u = &U[(size_t)i * dim];
      for (int k = 0; k < dim; ++k) u[k] += U_temp[(size_t)i * dim + k];
      if (u[0] < 1e-8) u[0] = 1e-8;
    }
  }

  // ---- MUSCL_base.hpp:97-225 ; returns the stop bits raised in this step
  int do_step(double dt0) {
    int bits = 0;
    dt = dt0;
    U_temp = U;
    find_v_max();
    if (dt > h0 * 0.1 / max_vel) dt = h0 * 0.1 / max_vel;
    const bool stop_before = stop_check;
    stop_check = false;
    const double extra_dt = extra_dt_constr();
    if (stop_check) bits |= 8;
    stop_check = stop_before || stop_check;
    if (dt > extra_dt) dt = extra_dt;

    // stop bits as in include/splash_gb300.h: 1 NaN flux, 2 NaN wave
    // speed, 4 wave ordering, 8 negative extra dt
    find_U_edges();
    int fb = find_flux_var();
    if (res2d(dt / 2)) bits |= 1;
    combine();

    find_U_edges();
    fb |= find_flux_var();
    if (res2d(dt)) bits |= 1;
    combine();

    if (fb & 1) bits |= 2;
    if (fb & 2) bits |= 4;
    if (bits) stop_check = true;

    double m = 0, l1 = 0, l2 = 0, l3 = 0, e = 0;
    for (int i = 0; i < nf; ++i) {
      const double* u = &U[(size_t)i * dim];
      m += u[0] * area[i];
      l1 += u[1] * area[i];
      l2 += u[2] * area[i];
      l3 += u[3] * area[i];
      if (!iso()) e += u[4] * area[i];
    }
    diag[0] = m;
    diag[1] = l1;
    diag[2] = l2;
    diag[3] = l3;
    diag[4] = e;
    t += dt;
    steps++;
    return bits;
  }
};

}  // namespace

extern "C" {

// Geometry in the reference numbering: per-face arrays [nf], per-slot
// arrays [ns] (x3 / x2 where vector-valued).  params =
// {accretion_rate, e_acc, omega_acc_abs, tilt_angle, acc_width, alpha,
//  friction_on}.  Returns nullptr on an invalid argument.
void* oracle_create(int nv, int nf, int ns, const double* vertices, const int* face_off,
                    const int* face_vtx, const int* nbr_edge, const double* face_centers,
                    const double* area, const double* edge_normals, const double* bm_dist,
                    const double* h_plus, const double* h_minus, const int* ff_plus,
                    const int* ff_minus, const double* beta_plus, const double* beta_minus,
                    double h0, double round_diff, const double* U_in, int dim, double gam,
                    double omega_ns, int accretion_on, const double* params, int solver_kind,
                    int threads) {
  if (nf <= 0 || ns <= 0) return nullptr;
  if (solver_kind < 1 || solver_kind > 4) return nullptr;
  if (dim != (solver_kind == 4 ? 4 : 5)) return nullptr;
  Oracle* o = new Oracle();
  o->nv = nv;
  o->nf = nf;
  o->ns = ns;
  o->vertices.assign(vertices, vertices + 3 * (size_t)nv);
  o->face_off.assign(face_off, face_off + nf + 1);
  o->face_vtx.assign(face_vtx, face_vtx + ns);
  o->nbr_edge.assign(nbr_edge, nbr_edge + ns);
  o->face_centers.assign(face_centers, face_centers + 3 * (size_t)nf);
  o->area.assign(area, area + nf);
  o->edge_normals.assign(edge_normals, edge_normals + 3 * (size_t)ns);
  o->bm.assign(bm_dist, bm_dist + ns);
  o->hp.assign(h_plus, h_plus + ns);
  o->hm.assign(h_minus, h_minus + ns);
  o->ffp.assign(ff_plus, ff_plus + 2 * (size_t)ns);
  o->ffm.assign(ff_minus, ff_minus + 2 * (size_t)ns);
  o->bp.assign(beta_plus, beta_plus + 2 * (size_t)ns);
  o->bmn.assign(beta_minus, beta_minus + 2 * (size_t)ns);
  o->h0 = h0;
  o->round_diff = round_diff;
  o->dim = dim;
  o->gam = gam;
  o->omega_ns = omega_ns;
  o->accretion_on = accretion_on != 0;
  o->acc_rate = params[0];
  o->e_acc = params[1];
  o->omega_acc_abs = params[2];
  o->tilt_angle = params[3];
  o->acc_width = params[4];
  o->alpha = params[5];
  o->friction_on = params[6] != 0.0;
  o->solver = solver_kind;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  // reverse slot: position of face i in neighbors_edge[nb]
  // (std::find of MUSCL_base.hpp:383-384)
  o->rev_slot.assign(ns, -1);
  for (int i = 0; i < nf; ++i) {
    for (int j = 0; j < o->nsl(i); ++j) {
      const int nb = nbr_edge[face_off[i] + j];
      int j0 = o->nsl(nb);
      for (int q = 0; q < o->nsl(nb); ++q)
        if (nbr_edge[face_off[nb] + q] == i) {
          j0 = q;
          break;
        }
      if (j0 == o->nsl(nb)) {
        delete o;
        return nullptr;
      }
      o->rev_slot[face_off[i] + j] = face_off[nb] + j0;
    }
  }
  o->U.assign(U_in, U_in + (size_t)nf * dim);
  o->U_plus.assign((size_t)ns * dim, 0.0);
  o->U_minus.assign((size_t)ns * dim, 0.0);
  o->flux_var.assign((size_t)ns * dim, 0.0);
  o->source_plus.assign((size_t)nf * dim, 0.0);
  // adiabatic.hpp:70-90
  {
    double ac = 0;
    const double mu = M_PI / 2;
    const double sigma = o->acc_width / 2.355;
    for (int n = 0; n < nf; ++n) {
      const V c = o->fc(n);
      const double theta = std::acos(c.z / norm(c));
      ac += o->area[n] / std::sqrt(2 * M_PI * sigma * sigma) *
            std::exp(-(theta - mu) * (theta - mu) / (2 * sigma * sigma));
    }
    ac /= 4 * M_PI;
    o->area_coeff = ac;
    double tm = 0;
    for (int n = 0; n < nf; ++n) tm += o->U[(size_t)n * dim] * o->area[n];
    o->total_mass = tm;
  }
  return o;
}

void oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

int oracle_do_step(void* h, double dt0) { return static_cast<Oracle*>(h)->do_step(dt0); }

int oracle_do_steps(void* h, int n, double dt0) {
  int bits = 0;
  for (int i = 0; i < n; ++i) bits |= static_cast<Oracle*>(h)->do_step(dt0);
  return bits;
}

void oracle_get_state(void* h, double* U) {
  Oracle* o = static_cast<Oracle*>(h);
  std::memcpy(U, o->U.data(), o->U.size() * sizeof(double));
}

void oracle_set_state(void* h, const double* U) {
  Oracle* o = static_cast<Oracle*>(h);
  std::memcpy(o->U.data(), U, o->U.size() * sizeof(double));
}

// out: t, dt, max_vel, stop, steps, area_coeff, total_mass, diag[5]
void oracle_info(void* h, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  out[0] = o->t;
  out[1] = o->dt;
  out[2] = o->max_vel;
  out[3] = o->stop_check ? 1.0 : 0.0;
  out[4] = (double)o->steps;
  out[5] = o->area_coeff;
  out[6] = o->total_mass;
  for (int k = 0; k < 5; ++k) out[7 + k] = o->diag[k];
}

// U_plus of the last stage, [ns][dim] (write_t_curl needs it)
void oracle_get_uplus(void* h, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  std::memcpy(out, o->U_plus.data(), o->U_plus.size() * sizeof(double));
}

// ---- per-function evaluation for known-answer tests -------------------
int oracle_flux_star(void* h, const double* uL, const double* uR, int face, int edge, double* F) {
  return static_cast<Oracle*>(h)->flux_star(uL, uR, face, edge, F);
}

// w: the face's state with w[4] the pressure; dt_member: the step's dt
void oracle_limiter(void* h, const double* r, const double* w, int face, int edge,
                    double dt_member, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  const double keep = o->dt;
  o->dt = dt_member;
  o->limiter(r, w, face, edge, out);
  o->dt = keep;
}

void oracle_source(void* h, const double* u, int face, double* out) {
  static_cast<Oracle*>(h)->source(u, face, out);
}

// isothermal solver functions: physical flux and wave speeds (S_L, S_R)
void oracle_iso_flux(void* h, const double* u, int face, int edge, double* out) {
  static_cast<Oracle*>(h)->iso_flux(u, face, edge, out);
}
void oracle_iso_char_vel(void* h, const double* uL, const double* uR, int face, int edge, double* out) {
  static_cast<Oracle*>(h)->iso_char_vel(uL, uR, face, edge, out[0], out[1]);
}

}  // extern "C"
