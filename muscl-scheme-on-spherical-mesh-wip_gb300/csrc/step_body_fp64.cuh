// Per-face bodies of the FP64 MUSCL step, shared by the time step
// (step_fp64.cu, scalar type double), the tangent-linear model (Dual<N>)
// and the adjoint's forward recomputation (double, extra outputs).
//
// Every body evaluates one face with the reference's operation order
// (MUSCL_base.hpp:124-161, 238-276, 345-434, 517-562), so all users of a
// body produce bit-identical primal values when compiled with -fmad=false.
#pragma once

#include <cstddef>

#include "dual.cuh"
#include "layout.hpp"
#include "physics_fp64.cuh"

namespace splash {
namespace f64 {

// A set of planes of doubles (value) and, for Dual<N>, N tangent copies
// of the same layout `tstride` doubles apart.
template <class T>
struct Planes;

template <>
struct Planes<double> {
  double* p;
  SPLASH_HD double ld(size_t i) const { return p[i]; }
  SPLASH_HD void st(size_t i, double x) const { p[i] = x; }
};

template <int N>
struct Planes<Dual<N>> {
  double* p;
  double* t;
  size_t tstride;
  SPLASH_HD Dual<N> ld(size_t i) const {
    Dual<N> r(p[i]);
#pragma unroll
    for (int j = 0; j < N; ++j) r.d[j] = t[j * tstride + i];
    return r;
  }
  SPLASH_HD void st(size_t i, const Dual<N>& x) const {
    p[i] = x.v;
#pragma unroll
    for (int j = 0; j < N; ++j) t[j * tstride + i] = x.d[j];
  }
};

SPLASH_HD D3 plane3(const double* p, int stride, int i) {
  return D3{p[i], p[stride + i], p[2 * stride + i]};
}

// (Sigma, l, Pi) of a conserved state u; MUSCL_base.hpp:124-161 stores
// U_i - 0.0 for fields 0..3 and the pressure of MUSCL_base.hpp:517-539.
template <class T>
SPLASH_HD void prim_of(const T* u, const D3& r, double gam, T* w) {
#pragma unroll
  for (int k = 0; k < 4; ++k) w[k] = u[k] - 0.0;
  w[4] = pressure_fc(u, r, gam) - 0.0;
}

// The accretion parameters of one face, in the scalar type Q.
template <class Q>
SPLASH_HD SrcParams<Q> face_src_params(const DevGeom& G, const PhysParams& P, int f) {
  return SrcParams<Q>{Q(G.acc_src[f]), v3(Q(P.omega_acc_x), Q(P.omega_acc_y), Q(P.omega_acc_z)),
                      Q(P.acc_rate), Q(P.total_mass)};
}

// find_U_edges (MUSCL_base.hpp:361-434) for every slot of face f: limited
// edge states of W, written to uplus with the energy at the edge centre.
template <class T>
SPLASH_HD void recon_face(const DevGeom& G, const PhysParams& P, double dt,
                                           const Planes<T>& W, const Planes<T>& uplus, int f) {
  const int fp = G.fpad;
  const int PS = G.max_slots * fp;  // one slot-plane set
  T w[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) w[k] = W.ld((size_t)k * fp + f);
  const int n = G.nslots[f];
  const double twoN = (double)(2 * n);
  const double gam = P.gam;
  const T c = sqrt(gam * (w[4] + 0.0) / (w[0] + 0.0));  // sound speed (per face)
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const int ia = G.sten[s], ib = G.sten[PS + s], ic = G.sten[2 * PS + s], id = G.sten[3 * PS + s];
    const double bp0 = G.beta[s], bp1 = G.beta[PS + s], bm0 = G.beta[2 * PS + s], bm1 = G.beta[3 * PS + s];
    const double hp = G.hpm[s], hm = G.hpm[PS + s], bmd = G.bm[s];
    const double ihp = 1.0 / hp, ihm = 1.0 / hm;
    T pp[kDim], r[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      const size_t o = (size_t)k * fp;
      const T Up = bp0 * W.ld(o + ia) + bp1 * W.ld(o + ib);
      pp[k] = (Up - w[k]) * ihp;
      const T Um = bm0 * W.ld(o + ic) + bm1 * W.ld(o + id);
      const T pm = (-Um + w[k]) * ihm;
      r[k] = pm / pp[k];
    }
    // Courant factor of the limiter (adiabatic.hpp:741-758, 792-810)
    const D3 ec = plane3(G.ec, PS, s);
    const double ecn = G.ecn[s];
    const D3 en = plane3(G.en, PS, s);
    V3<T> vel = cross3(ec, v3(w[1], w[2], w[3]));
    vel = scal(vel, 1.0 / ((-w[0] - 0.0) * ecn));
    const T nu_plus = (c + dot3(vel, en)) * dt * G.arc_a[s];
    const double eta_p = G.eta[s];
    const T sb_scale = G.eta[PS + s] / (twoN * nu_plus);
    const T to_scale = (1 + nu_plus) / 3;
    T up[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      const T lim = limiter_field(r[k], eta_p, sb_scale, to_scale);
      if (k == 0 || k == 4)
        up[k] = w[k] + 0.0 + pp[k] * lim * bmd;
      else
        up[k] = w[k] + pp[k] * lim * bmd;
    }
    up[4] = energy_at_edge(up, ec, gam);  // Pi -> E at the edge centre
#pragma unroll
    for (int k = 0; k < kDim; ++k) uplus.st((size_t)k * PS + s, up[k]);
  }
}

// find_flux_var + res2d + the RK combine with the density floor
// (MUSCL_base.hpp:345-359, 238-276, 124-161) for face f: the updated
// conserved state U0 + dt_here (source - flux divergence), floored.
// Returns the stop bits; `floored` reports the density floor.
template <class T, class Q>
SPLASH_HD unsigned flux_face(const DevGeom& G, const PhysParams& P, const SrcParams<Q>& sp,
                                              double dt_here, const Planes<T>& Win, const Planes<T>& U0,
                                              const Planes<T>& uplus, int f, T* u, bool& floored) {
  const int fp = G.fpad;
  const int PS = G.max_slots * fp;
  const D3 fcn = plane3(G.fcn, fp, f);
  const double area = G.area[f];
  T w[kDim], acc[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) w[k] = Win.ld((size_t)k * fp + f);
  source_term(w, fcn, sp, P, acc);
#pragma unroll
  for (int k = 0; k < kDim; ++k) acc[k] = dt_here * acc[k];
  const double rd_dt = P.round_diff * dt_here;
  const int n = G.nslots[f];
  unsigned bits = 0;
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const int rv = G.rev[s];
    T uL[kDim], uR[kDim], F[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      uL[k] = uplus.ld((size_t)k * PS + s);
      uR[k] = uplus.ld((size_t)k * PS + rv);
    }
    SlotGeom g;
    g.ec = plane3(G.ec, PS, s);
    g.ecn = G.ecn[s];
    g.en = plane3(G.en, PS, s);
    g.nxr = plane3(G.nxr, PS, s);
    bits |= flux_star(uL, uR, g, P.gam, P.solver, F);
    const double coef = rd_dt * G.chord[s] / area;
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      if (is_nan(F[k])) bits |= 1u;
      acc[k] -= coef * F[k];
    }
  }
#pragma unroll
  for (int k = 0; k < kDim; ++k) u[k] = acc[k] + U0.ld((size_t)k * fp + f);
  floored = u[0] < 1e-8;
  if (floored) u[0] = T(1e-8);
  return bits;
}

}  // namespace f64
}  // namespace splash
