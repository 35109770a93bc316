// Reverse (adjoint) forms of the FP64 per-slot and per-face physics.
//
// Each reverse function recomputes the primal with exactly the operations
// of physics_fp64.cuh (so it takes the same branches as the forward step:
// limiter cases, wave-speed sides, HLLC+ switches, floors) and then
// propagates the adjoint of its outputs back to its inputs.  Conventions:
// `xb` is the adjoint (bar) of x; reverse functions ADD into the bars of
// their inputs.  At a kink the derivative of the branch taken is used,
// matching the forward-mode duals of dual.cuh.
//
//   flux_star_rev     hand-written reverse of the three Riemann solvers
//                     (HLLE_p.hpp:19-58, HLLC.hpp:138-242,
//                     HLLCplus.hpp:17-177, char_vel adiabatic.hpp:594-683)
//   recon_face_tape   find_U_edges (MUSCL_base.hpp:361-434) with the local
//                     limiter Jacobian (adiabatic.hpp:685-828) taped per slot
//   recon_face_rev    reverse of the reconstruction from that tape
//   source_rev        reverse of the source term (adiabatic.hpp:396-541)
//                     from a Dual<10> Jacobian of its 5 state and 5
//                     parameter inputs
//   prim_rev          reverse of (Sigma, l, E) -> (Sigma, l, Pi)
#pragma once

#include "dual.cuh"
#include "physics_fp64.cuh"
#include "step_body_fp64.cuh"

namespace splash {
namespace f64 {
namespace rev {

// ---------------------------------------------------------------------
// One side (left or right edge state) of a Riemann flux.
struct Side {
  double u[kDim];
  D3 c;        // cross(ec, l)
  double s;    // 1 / ((-u0) |ec|)
  D3 vel;      // edge velocity c * s
  double n;    // |vel|
  double e;    // unfloored pressure (u4 - u0 n^2 / 2)(gam - 1)
  double p;    // max(1e-16, e)
  double vn;   // en . vel
  double a;    // sqrt(gam p / u0)
  double F[kDim];
};

struct SideBar {
  double u[kDim];
  D3 vel;
  double n, p, vn, a;
  double F[kDim];
};

SPLASH_HD void zero(SideBar& b) {
#pragma unroll
  for (int k = 0; k < kDim; ++k) b.u[k] = b.F[k] = 0.0;
  b.vel = d3(0, 0, 0);
  b.n = b.p = b.vn = b.a = 0.0;
}

// edge_vel, pressure, phys_flux and the sound speed of char_vel, with the
// operation order of physics_fp64.cuh.
SPLASH_HD void side_forward(const double* u, const SlotGeom& g, double gam, Side& S) {
#pragma unroll
  for (int k = 0; k < kDim; ++k) S.u[k] = u[k];
  S.c = cross3(g.ec, d3(u[1], u[2], u[3]));
  S.s = 1.0 / ((-u[0]) * g.ecn);
  S.vel = scal(S.c, S.s);
  S.n = norm3(S.vel);
  S.e = (u[4] - u[0] * (S.n * S.n) / 2) * (gam - 1);
  S.p = smax(1e-16, S.e);
  S.vn = dot3(g.en, S.vel);
  S.a = sqrt(gam * S.p / u[0]);
  S.F[0] = u[0] * S.vn;
  S.F[1] = (u[1] * S.vn - g.nxr.x * S.p);
  S.F[2] = (u[2] * S.vn - g.nxr.y * S.p);
  S.F[3] = (u[3] * S.vn - g.nxr.z * S.p);
  S.F[4] = (u[4] + S.p) * S.vn;
}

SPLASH_HD void side_reverse(const Side& S, const SlotGeom& g, double gam, SideBar& B, double* ub) {
  double u0b = B.u[0] + B.F[0] * S.vn;
  double vnb = B.vn + B.F[0] * S.u[0];
  double l1b = B.u[1] + B.F[1] * S.vn, l2b = B.u[2] + B.F[2] * S.vn, l3b = B.u[3] + B.F[3] * S.vn;
  vnb += B.F[1] * S.u[1] + B.F[2] * S.u[2] + B.F[3] * S.u[3] + B.F[4] * (S.u[4] + S.p);
  double pb = B.p - (g.nxr.x * B.F[1] + g.nxr.y * B.F[2] + g.nxr.z * B.F[3]) + B.F[4] * S.vn;
  double u4b = B.u[4] + B.F[4] * S.vn;
  // a = sqrt(gam p / u0)
  if (S.a > 0.0) {
    const double xb = B.a * 0.5 / S.a;
    const double iu0 = 1.0 / S.u[0];
    pb += xb * gam * iu0;
    u0b -= xb * (gam * S.p * iu0) * iu0;
  }
  // vn = en . vel
  D3 vb = d3(B.vel.x + vnb * g.en.x, B.vel.y + vnb * g.en.y, B.vel.z + vnb * g.en.z);
  // p = max(1e-16, e)
  double nb = B.n;
  if (1e-16 < S.e) {
    const double eb = pb * (gam - 1);
    u4b += eb;
    u0b -= eb * (S.n * S.n) / 2;
    nb -= eb * S.u[0] * S.n;
  }
  // n = |vel|
  if (S.n > 0.0) {
    const double t = nb / S.n;
    vb = d3(vb.x + t * S.vel.x, vb.y + t * S.vel.y, vb.z + t * S.vel.z);
  }
  // vel = c * s ; s = 1 / ((-u0) ecn)
  const D3 cb = scal(vb, S.s);
  const double sb = dot3(vb, S.c);
  u0b += sb * S.s * S.s * g.ecn;
  // c = ec x l  ->  lb += cb x ec
  const D3 lb = cross3(cb, g.ec);
  ub[0] += u0b;
  ub[1] += l1b + lb.x;
  ub[2] += l2b + lb.y;
  ub[3] += l3b + lb.z;
  ub[4] += u4b;
}

// ---------------------------------------------------------------------
// Adjoint of F = flux_star(uL, uR): uLb += (dF/duL)^T Fb, uRb += (dF/duR)^T Fb.
SPLASH_HD void flux_star_rev(const double* uL, const double* uR, const SlotGeom& g, double gam, int solver,
                             const double* Fb, double* uLb, double* uRb) {
  Side L, R;
  side_forward(uL, g, gam, L);
  side_forward(uR, g, gam, R);
  SideBar BL, BR;
  zero(BL);
  zero(BR);
  // char_vel (adiabatic.hpp:594-683)
  const double p_pvrs = 1 / 2. * (L.p + R.p) - 1 / 8. * (R.vn - L.vn) * (uL[0] + uR[0]) * (L.a + R.a);
  const double p_star = smax(0., p_pvrs);
  const double kk = (gam + 1) / (2 * gam);
  double q_R = 1., q_L = 1.;
  bool qRd = false, qLd = false;
  if (!(p_star <= R.p)) {
    q_R = sqrt(1 + kk * (p_star / R.p - 1));
    if (is_nan(q_R) || is_inf(q_R))
      q_R = 1.;
    else
      qRd = true;
  }
  if (!(p_star <= L.p)) {
    q_L = sqrt(1 + kk * (p_star / L.p - 1));
    if (is_nan(q_L) || is_inf(q_L))
      q_L = 1.;
    else
      qLd = true;
  }
  const double S_L = L.vn - L.a * q_L;
  const double S_R = R.vn + R.a * q_R;
  double SLb = 0.0, SRb = 0.0;

  if (solver == 1) {
    if (S_L >= 0) {
#pragma unroll
      for (int i = 0; i < kDim; ++i) BL.F[i] += Fb[i];
    } else if (S_L < 0 && S_R > 0) {
      const double inv = 1.0 / (S_R - S_L);
      double invb = 0.0;
#pragma unroll
      for (int i = 0; i < kDim; ++i) {
        const double du = uR[i] - uL[i];
        const double N = S_R * L.F[i] - S_L * R.F[i] + S_R * S_L * du;
        const double Nb = Fb[i] * inv;
        invb += Fb[i] * N;
        SRb += Nb * (L.F[i] + S_L * du);
        SLb += Nb * (-R.F[i] + S_R * du);
        BL.F[i] += Nb * S_R;
        BR.F[i] -= Nb * S_L;
        BR.u[i] += Nb * S_R * S_L;
        BL.u[i] -= Nb * S_R * S_L;
      }
      const double db = -invb * inv * inv;
      SRb += db;
      SLb -= db;
    } else {
#pragma unroll
      for (int i = 0; i < kDim; ++i) BR.F[i] += Fb[i];
    }
  } else {
    const double rho_L = uL[0], rho_R = uR[0];
    const double V_L = L.vn, V_R = R.vn;
    const double p_L = L.p, p_R = R.p;
    const double num = p_R - p_L + rho_L * V_L * (S_L - V_L) - rho_R * V_R * (S_R - V_R);
    const double den = rho_L * (S_L - V_L) - rho_R * (S_R - V_R);
    double S_star = num / den;
    const bool ss_fb = is_nan(S_star) || is_inf(S_star);
    if (ss_fb) S_star = (V_L + V_R) / 2;
    const double P_LR =
        (p_L + p_R + uL[0] * (S_L - V_L) * (S_star - V_L) + uR[0] * (S_R - V_R) * (S_star - V_R)) / 2;
    int side;
    if (S_L >= 0)
      side = 0;
    else if (S_L < 0 && S_star >= 0)
      side = 1;
    else if (S_star < 0 && S_R >= 0)
      side = 2;
    else
      side = 3;
    if (side == 0) {
#pragma unroll
      for (int i = 0; i < kDim; ++i) BL.F[i] += Fb[i];
    } else if (side == 3) {
#pragma unroll
      for (int i = 0; i < kDim; ++i) BR.F[i] += Fb[i];
    } else {
      const bool left = (side == 1);
      const double Sk = left ? S_L : S_R;
      const double* uk = left ? uL : uR;
      const Side& K = left ? L : R;
      const double inv_k = 1.0 / (Sk - S_star);
      const double D[kDim] = {0., -g.nxr.x, -g.nxr.y, -g.nxr.z, S_star};
      double Skb = 0.0, Ssb = 0.0, PLRb = 0.0, invkb = 0.0, VLb = 0.0, VRb = 0.0;
      double ukb[kDim] = {0, 0, 0, 0, 0}, Fkb[kDim] = {0, 0, 0, 0, 0};
      if (solver == 3) {
        // HLLC+ correction (HLLCplus.hpp:17-177)
        const double phi_L = uL[0] * (S_L - V_L);
        const double phi_R = uR[0] * (S_R - V_R);
        const double a_L = L.a, a_R = R.a;
        const double mL = L.n / a_L, mR = R.n / a_R;
        const double inner = smax(mL, mR);
        const double M = smin(1., inner);
        int lambd_L = 0, lambd_R = 0;
        if ((V_L - a_L) > 0 && (V_R - a_R) < 0) lambd_L = 1;
        if ((V_L + a_L) > 0 && (V_R + a_R) < 0) lambd_L = 1;
        if ((V_R - a_R) > 0 && (V_L - a_L) < 0) lambd_R = 1;
        if ((V_R + a_R) > 0 && (V_L + a_L) < 0) lambd_R = 1;
        const bool fs_on = (lambd_L == 0 && lambd_R == 0);
        double f_star = 1., dfdM = 0.0;
        if (fs_on) {
          const Dual<1> Md = Dual<1>::seed(M, 0);
          const Dual<1> fd = Md * sqrt(4 + (1 - Md * Md) * (1 - Md * Md)) / ((1 + Md * Md));
          f_star = fd.v;
          dfdM = fd.d[0];
        }
        const double hA = p_L / p_R, hB = p_R / p_L;
        const double h = smin(hA, hB);
        const double lg = log(h);
        const double E = exp(M * lg);
        const double gsw = 1 - E;
        const double dV = V_R - V_L;
        const D3 dv = sub(R.vel, L.vel);
        const double cs = Sk * inv_k * gsw;
        const double fm = f_star - 1;
        const D3 vff = d3(fm * dV * g.en.x + cs * (dv.x - dV * g.en.x), fm * dV * g.en.y + cs * (dv.y - dV * g.en.y),
                          fm * dV * g.en.z + cs * (dv.z - dV * g.en.z));
        const D3 am = cross3(g.ec, vff);
        const double w = phi_L * phi_R / (phi_R - phi_L);
        const double X4 = fm * (V_R - V_L) * S_star;
        // reverse
        const double wb = Fb[1] * am.x + Fb[2] * am.y + Fb[3] * am.z + Fb[4] * X4;
        const D3 amb = d3(Fb[1] * w, Fb[2] * w, Fb[3] * w);
        const double X4b = Fb[4] * w;
        double fmb = X4b * (V_R - V_L) * S_star;
        const double dV2b = X4b * fm * S_star;
        VRb += dV2b;
        VLb -= dV2b;
        Ssb += X4b * fm * (V_R - V_L);
        const D3 vffb = cross3(amb, g.ec);
        double dVb = 0.0, csb = 0.0;
        fmb += vffb.x * dV * g.en.x + vffb.y * dV * g.en.y + vffb.z * dV * g.en.z;
        dVb += vffb.x * (fm * g.en.x - cs * g.en.x) + vffb.y * (fm * g.en.y - cs * g.en.y) +
               vffb.z * (fm * g.en.z - cs * g.en.z);
        csb += vffb.x * (dv.x - dV * g.en.x) + vffb.y * (dv.y - dV * g.en.y) + vffb.z * (dv.z - dV * g.en.z);
        const D3 dvb = scal(vffb, cs);
        BR.vel = d3(BR.vel.x + dvb.x, BR.vel.y + dvb.y, BR.vel.z + dvb.z);
        BL.vel = d3(BL.vel.x - dvb.x, BL.vel.y - dvb.y, BL.vel.z - dvb.z);
        VRb += dVb;
        VLb -= dVb;
        Skb += csb * inv_k * gsw;
        invkb += csb * Sk * gsw;
        const double gswb = csb * Sk * inv_k;
        const double yb = -gswb * E;
        double Mb = yb * lg;
        const double hb = yb * M / h;
        if (hB < hA) {  // h = p_R / p_L
          BR.p += hb / p_L;
          BL.p -= hb * hB / p_L;
        } else {  // h = p_L / p_R
          BL.p += hb / p_R;
          BR.p -= hb * hA / p_R;
        }
        if (fs_on) Mb += fmb * dfdM;
        if (inner < 1.) {
          if (mL < mR) {
            BR.n += Mb / a_R;
            BR.a -= Mb * mR / a_R;
          } else {
            BL.n += Mb / a_L;
            BL.a -= Mb * mL / a_L;
          }
        }
        // w = phi_L phi_R / (phi_R - phi_L)
        const double Q = phi_R - phi_L;
        const double Pb = wb / Q;
        const double Qb = -wb * w / Q;
        const double phiLb = Pb * phi_R - Qb;
        const double phiRb = Pb * phi_L + Qb;
        BL.u[0] += phiLb * (S_L - V_L);
        SLb += phiLb * uL[0];
        VLb -= phiLb * uL[0];
        BR.u[0] += phiRb * (S_R - V_R);
        SRb += phiRb * uR[0];
        VRb -= phiRb * uR[0];
      }
      // F_k* (HLLC.hpp:218-239)
#pragma unroll
      for (int i = 0; i < kDim; ++i) {
        const double Gi = S_star * (Sk * uk[i] - K.F[i]) + Sk * P_LR * D[i];
        const double Gb = Fb[i] * inv_k;
        invkb += Fb[i] * Gi;
        Ssb += Gb * (Sk * uk[i] - K.F[i]);
        const double t = Gb * S_star;
        Skb += t * uk[i];
        ukb[i] += t * Sk;
        Fkb[i] -= t;
        Skb += Gb * P_LR * D[i];
        PLRb += Gb * Sk * D[i];
      }
      Ssb += (Fb[4] * inv_k) * Sk * P_LR;  // D[4] = S_star
      // inv_k = 1 / (Sk - S_star)
      const double db = -invkb * inv_k * inv_k;
      Skb += db;
      Ssb -= db;
      SideBar& BK = left ? BL : BR;
#pragma unroll
      for (int i = 0; i < kDim; ++i) {
        BK.u[i] += ukb[i];
        BK.F[i] += Fkb[i];
      }
      if (left)
        SLb += Skb;
      else
        SRb += Skb;
      // P_LR
      const double q = PLRb / 2;
      BL.p += q;
      BR.p += q;
      {
        const double X = uL[0] * (S_L - V_L), Y = S_star - V_L;
        const double Xb = q * Y, Yb = q * X;
        BL.u[0] += Xb * (S_L - V_L);
        SLb += Xb * uL[0];
        VLb -= Xb * uL[0];
        Ssb += Yb;
        VLb -= Yb;
      }
      {
        const double X = uR[0] * (S_R - V_R), Y = S_star - V_R;
        const double Xb = q * Y, Yb = q * X;
        BR.u[0] += Xb * (S_R - V_R);
        SRb += Xb * uR[0];
        VRb -= Xb * uR[0];
        Ssb += Yb;
        VRb -= Yb;
      }
      // S_star
      if (ss_fb) {
        VLb += Ssb / 2;
        VRb += Ssb / 2;
      } else {
        const double numb = Ssb / den;
        const double denb = -Ssb * S_star / den;
        BR.p += numb;
        BL.p -= numb;
        const double A = rho_L * V_L, Bq = S_L - V_L;
        BL.u[0] += numb * Bq * V_L;
        VLb += numb * Bq * rho_L;
        SLb += numb * A;
        VLb -= numb * A;
        const double C = rho_R * V_R, Dd = S_R - V_R;
        BR.u[0] -= numb * Dd * V_R;
        VRb -= numb * Dd * rho_R;
        SRb -= numb * C;
        VRb += numb * C;
        BL.u[0] += denb * (S_L - V_L);
        SLb += denb * rho_L;
        VLb -= denb * rho_L;
        BR.u[0] -= denb * (S_R - V_R);
        SRb -= denb * rho_R;
        VRb += denb * rho_R;
      }
      BL.vn += VLb;
      BR.vn += VRb;
    }
  }
  // char_vel reverse: S_L = vn_L - a_L q_L ; S_R = vn_R + a_R q_R
  BL.vn += SLb;
  BL.a -= SLb * q_L;
  const double qLb = -SLb * L.a;
  BR.vn += SRb;
  BR.a += SRb * q_R;
  const double qRb = SRb * R.a;
  double psb = 0.0;
  if (qRd) {
    const double zb = qRb * 0.5 / q_R;
    psb += zb * kk / R.p;
    BR.p -= zb * kk * p_star / (R.p * R.p);
  }
  if (qLd) {
    const double zb = qLb * 0.5 / q_L;
    psb += zb * kk / L.p;
    BL.p -= zb * kk * p_star / (L.p * L.p);
  }
  const double ppb = (0. < p_pvrs) ? psb : 0.0;
  BL.p += 0.5 * ppb;
  BR.p += 0.5 * ppb;
  {
    const double t = -ppb * 0.125;
    const double dvn = R.vn - L.vn, rs = uL[0] + uR[0], as = L.a + R.a;
    const double dvnb = t * rs * as, rsb = t * dvn * as, asb = t * dvn * rs;
    BR.vn += dvnb;
    BL.vn -= dvnb;
    BL.u[0] += rsb;
    BR.u[0] += rsb;
    BL.a += asb;
    BR.a += asb;
  }
  side_reverse(L, g, gam, BL, uLb);
  side_reverse(R, g, gam, BR, uRb);
}

// ---------------------------------------------------------------------
// Reconstruction with its reverse-sweep tape, and the reverse from the tape.
//
// Per slot and field the limited edge state is up = w + pp phi(r, nu) bmd
// with pp = (Up - w)/H+, pm = (w - Um)/H-, r = pm/pp and nu the slot's
// Courant factor (MUSCL_base.hpp:361-434, adiabatic.hpp:685-828).  The
// recomputation evaluates phi once on Dual<2> over (r, nu) -- its value is
// the primal's, bit for bit -- and stores the three partials
//   d up / d pp = bmd (phi - r phi_r),  d up / d pm = bmd phi_r,
//   d up / d nu = pp bmd phi_nu
// so that the reverse sweep needs no transcendental.  Where phi is flat in r
// (r = +-inf or NaN) d up / d pp = bmd phi.
constexpr int kTapePlanes = 16;  // 3 per field + the edge pressure before Pi -> E

SPLASH_HD void recon_face_tape(const DevGeom& G, const PhysParams& P, double dt, const double* W, double* uplus,
                               double* LJ, int f) {
  const int fp = G.fpad;
  const int PS = G.max_slots * fp;
  double w[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) w[k] = W[(size_t)k * fp + f];
  const int n = G.nslots[f];
  const double twoN = (double)(2 * n);
  const double gam = P.gam;
  const double c = sqrt(gam * (w[4] + 0.0) / (w[0] + 0.0));
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const int ia = G.sten[s], ib = G.sten[PS + s], ic = G.sten[2 * PS + s], id = G.sten[3 * PS + s];
    const double bp0 = G.beta[s], bp1 = G.beta[PS + s], bm0 = G.beta[2 * PS + s], bm1 = G.beta[3 * PS + s];
    const double hp = G.hpm[s], hm = G.hpm[PS + s], bmd = G.bm[s];
    const double ihp = 1.0 / hp, ihm = 1.0 / hm;
    double pp[kDim], r[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      const double* Wk = W + (size_t)k * fp;
      const double Up = bp0 * Wk[ia] + bp1 * Wk[ib];
      pp[k] = (Up - w[k]) * ihp;
      const double Um = bm0 * Wk[ic] + bm1 * Wk[id];
      const double pm = (-Um + w[k]) * ihm;
      r[k] = pm / pp[k];
    }
    const D3 ec = plane3(G.ec, PS, s);
    const double ecn = G.ecn[s];
    const D3 en = plane3(G.en, PS, s);
    D3 vel = cross3(ec, d3(w[1], w[2], w[3]));
    vel = scal(vel, 1.0 / ((-w[0] - 0.0) * ecn));
    const double nu_plus = (c + dot3(vel, en)) * dt * G.arc_a[s];
    const double eta_p = G.eta[s];
    const Dual<2> nud = Dual<2>::seed(nu_plus, 1);
    const Dual<2> sb_scale = G.eta[PS + s] / (twoN * nud);
    const Dual<2> to_scale = (1 + nud) / 3;
    double up[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      const Dual<2> lim = limiter_field(Dual<2>::seed(r[k], 0), eta_p, sb_scale, to_scale);
      if (k == 0 || k == 4)
        up[k] = w[k] + 0.0 + pp[k] * lim.v * bmd;
      else
        up[k] = w[k] + pp[k] * lim.v * bmd;
      const double dpp = bmd * ((lim.d[0] != 0.0) ? lim.v - lim.d[0] * r[k] : lim.v);
      LJ[(size_t)(3 * k) * PS + s] = dpp;
      LJ[(size_t)(3 * k + 1) * PS + s] = bmd * lim.d[0];
      LJ[(size_t)(3 * k + 2) * PS + s] = pp[k] * bmd * lim.d[1];
    }
    LJ[(size_t)15 * PS + s] = up[4];
    up[4] = energy_at_edge(up, ec, gam);
#pragma unroll
    for (int k = 0; k < kDim; ++k) uplus[(size_t)k * PS + s] = up[k];
  }
}

// Sound speed of a face as a Dual<5> over its (Sigma, l, Pi).
SPLASH_HD Dual<5> face_sound_speed(const double* w, double gam) {
  const Dual<5> w0 = Dual<5>::seed(w[0], 0), w4 = Dual<5>::seed(w[4], 4);
  return sqrt(gam * (w4 + 0.0) / (w0 + 0.0));
}

// Reverse of recon_face_tape for face f.  W holds the primal (Sigma, l, Pi)
// planes, uplus and LJ the slot's tape; upb_at(k, s) returns the adjoint of
// uplus[k * PS + s].  Writes the adjoints of the slot's stencil
// interpolants to PU (planes 0..4: Up, 5..9: Um, each PS long) and adds the
// face's own contribution to wb.  The interpolants' adjoints reach the
// stencil faces through PU times the betas (scattered by the caller).
template <class UpbFn>
SPLASH_HD void recon_face_rev(const DevGeom& G, const PhysParams& P, double dt, const double* W,
                              const double* uplus, const double* LJ, UpbFn upb_at, double* PU, double* wb, int f) {
  const int fp = G.fpad;
  const int PS = G.max_slots * fp;
  double w[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) w[k] = W[(size_t)k * fp + f];
  const int n = G.nslots[f];
  const Dual<5> c = face_sound_speed(w, P.gam);
  Dual<5> wd[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) wd[k] = Dual<5>::seed(w[k], k);
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const D3 ec = plane3(G.ec, PS, s);
    const D3 en = plane3(G.en, PS, s);
    // energy at the edge centre from the limited (Sigma, l, Pi)
    Dual<5> ud[kDim];
#pragma unroll
    for (int k = 0; k < 4; ++k) ud[k] = Dual<5>::seed(uplus[(size_t)k * PS + s], k);
    ud[4] = Dual<5>::seed(LJ[(size_t)15 * PS + s], 4);
    const Dual<5> E = energy_at_edge(ud, ec, P.gam);
    double upb[kDim], preb[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) upb[k] = upb_at(k, s);
#pragma unroll
    for (int k = 0; k < 4; ++k) preb[k] = upb[k] + upb[4] * E.d[k];
    preb[4] = upb[4] * E.d[4];
    // Courant factor as a function of w
    V3<Dual<5>> vel = cross3(ec, v3(wd[1], wd[2], wd[3]));
    vel = scal(vel, 1.0 / ((-wd[0] - 0.0) * G.ecn[s]));
    const Dual<5> nu5 = (c + dot3(vel, en)) * dt * G.arc_a[s];
    const double ihp = 1.0 / G.hpm[s], ihm = 1.0 / G.hpm[PS + s];
    double nub = 0.0;
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      const double ppb = preb[k] * LJ[(size_t)(3 * k) * PS + s];
      const double pmb = preb[k] * LJ[(size_t)(3 * k + 1) * PS + s];
      nub += preb[k] * LJ[(size_t)(3 * k + 2) * PS + s];
      PU[(size_t)k * PS + s] = ppb * ihp;
      PU[(size_t)(kDim + k) * PS + s] = -pmb * ihm;
      wb[k] += preb[k] - ppb * ihp + pmb * ihm;
    }
#pragma unroll
    for (int k = 0; k < kDim; ++k) wb[k] += nub * nu5.d[k];
  }
}

// ---------------------------------------------------------------------
// Reverse of the source term.  srcb is the adjoint of res; wb += and
// pb[0..4] += the adjoints of (acc0, omega_acc.y, omega_acc.z, acc_rate,
// total_mass).  omega_acc.x is identically 0 (no derivative taken).
SPLASH_HD void source_rev(const double* w, const D3& fcn, const SrcParams<double>& sp, const PhysParams& P,
                          const double* srcb, double* wb, double* pb) {
  if (!P.accretion_on) return;
  Dual<10> wd[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) wd[k] = Dual<10>::seed(w[k], k);
  SrcParams<Dual<10>> sd;
  sd.acc0 = Dual<10>::seed(sp.acc0, 5);
  sd.omega_acc = v3(Dual<10>(sp.omega_acc.x), Dual<10>::seed(sp.omega_acc.y, 6), Dual<10>::seed(sp.omega_acc.z, 7));
  sd.acc_rate = Dual<10>::seed(sp.acc_rate, 8);
  sd.total_mass = Dual<10>::seed(sp.total_mass, 9);
  Dual<10> res[kDim];
  source_term(wd, fcn, sd, P, res);
#pragma unroll
  for (int i = 0; i < kDim; ++i) {
#pragma unroll
    for (int k = 0; k < kDim; ++k) wb[k] += srcb[i] * res[i].d[k];
#pragma unroll
    for (int j = 0; j < 5; ++j) pb[j] += srcb[i] * res[i].d[5 + j];
  }
}

// Reverse of prim_of: ub += J^T wb for w = (u0..u3, pressure_fc(u)).
SPLASH_HD void prim_rev(const double* u, const D3& r, double gam, const double* wb, double* ub) {
  Dual<5> ud[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) ud[k] = Dual<5>::seed(u[k], k);
  const Dual<5> p = pressure_fc(ud, r, gam);
#pragma unroll
  for (int k = 0; k < 4; ++k) ub[k] += wb[k] + wb[4] * p.d[k];
  ub[4] += wb[4] * p.d[4];
}

}  // namespace rev
}  // namespace f64
}  // namespace splash
