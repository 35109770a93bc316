// Host build of the per-slot / per-face physics and their reverse forms
// (adjoint_rev.cuh), for CPU checks of the hand-written adjoints:
//   * full Jacobians of the Riemann fluxes, forward duals vs reverse sweep;
//   * the reconstruction of one face, tangent-linear (recon_face on
//     Dual<1>) vs reverse (recon_face_tape, recon_face_rev and the beta
//     scatter) dot products; the taped edge states equal recon_face's;
//   * source term and pressure conversion, reverse vs plain evaluations
//     (the test takes central finite differences of the latter).
// Compiled by the test with g++ -ffp-contract=off (no FMA contraction, as
// the FP64 kernels are built with -fmad=false).
#include <cstring>
#include <vector>

#include "adjoint_rev.cuh"

using namespace splash;
using namespace splash::f64;

namespace {

SlotGeom geom_from(const double* g) {
  SlotGeom s;
  s.ec = d3(g[0], g[1], g[2]);
  s.ecn = g[3];
  s.en = d3(g[4], g[5], g[6]);
  s.nxr = d3(g[7], g[8], g[9]);
  return s;
}

PhysParams phys_from(const double* p, int accretion_on, int friction_on, int solver) {
  PhysParams P{};
  P.gam = p[0];
  P.omega_ns = p[1];
  P.e_acc = p[2];
  P.alpha = p[3];
  P.accretion_on = accretion_on;
  P.friction_on = friction_on;
  P.solver = solver;
  derive_params(P);
  return P;
}

}  // namespace

extern "C" {

// flux_star in double (F), its 5x10 Jacobian over (uL, uR) by Dual<10>
// (Jf) and by flux_star_rev with unit output adjoints (Jr).  Returns 1 when
// the dual evaluation's values differ from the double evaluation.
int adj_flux_jac(const double* uL, const double* uR, const double* geom, double gam, int solver, double* F,
                 double* Jf, double* Jr) {
  const SlotGeom g = geom_from(geom);
  flux_star(uL, uR, g, gam, solver, F);
  Dual<10> L[kDim], R[kDim], Fo[kDim];
  for (int k = 0; k < kDim; ++k) {
    L[k] = Dual<10>::seed(uL[k], k);
    R[k] = Dual<10>::seed(uR[k], 5 + k);
  }
  flux_star(L, R, g, gam, solver, Fo);
  int mismatch = 0;
  for (int i = 0; i < kDim; ++i) {
    if (std::memcmp(&Fo[i].v, &F[i], sizeof(double)) != 0) mismatch = 1;
    for (int j = 0; j < 10; ++j) Jf[i * 10 + j] = Fo[i].d[j];
  }
  for (int i = 0; i < kDim; ++i) {
    double Fb[kDim] = {0, 0, 0, 0, 0}, uLb[kDim] = {0, 0, 0, 0, 0}, uRb[kDim] = {0, 0, 0, 0, 0};
    Fb[i] = 1.0;
    rev::flux_star_rev(uL, uR, g, gam, solver, Fb, uLb, uRb);
    for (int j = 0; j < kDim; ++j) {
      Jr[i * 10 + j] = uLb[j];
      Jr[i * 10 + 5 + j] = uRb[j];
    }
  }
  return mismatch;
}

// One face (index 0) with n slots; faces 1..nf-1 are its stencil faces.
// Per-slot inputs are compact ([plane][slot]); W and V are [5][nf].
// out[0] = <upb, J V> (tangent-linear), out[1] = <J^T upb, V> (reverse);
// uplus receives the primal edge states [5][n].
int adj_recon_dot(int n, int nf, const int* sten, const double* beta, const double* hpm, const double* bm,
                  const double* eta, const double* arc_a, const double* ec, const double* ecn, const double* en,
                  double gam, double dt, const double* W, const double* V, const double* upb, double* out,
                  double* uplus) {
  const int fp = nf, PS = n * nf;
  auto planes = [&](const double* src, int np) {
    std::vector<double> v((size_t)np * PS, 0.0);
    for (int p = 0; p < np; ++p)
      for (int j = 0; j < n; ++j) v[(size_t)p * PS + (size_t)j * fp] = src[p * n + j];
    return v;
  };
  std::vector<int> vsten((size_t)4 * PS, 0);
  for (int p = 0; p < 4; ++p)
    for (int j = 0; j < n; ++j) vsten[(size_t)p * PS + (size_t)j * fp] = sten[p * n + j];
  std::vector<double> vbeta = planes(beta, 4), vhpm = planes(hpm, 2), vbm = planes(bm, 1), veta = planes(eta, 2),
                      varc = planes(arc_a, 1), vec = planes(ec, 3), vecn = planes(ecn, 1), ven = planes(en, 3);
  std::vector<int8_t> nsl(fp, 0);
  nsl[0] = (int8_t)n;
  DevGeom G{};
  G.n_faces = nf;
  G.fpad = fp;
  G.max_slots = n;
  G.nslots = nsl.data();
  G.sten = vsten.data();
  G.beta = vbeta.data();
  G.hpm = vhpm.data();
  G.bm = vbm.data();
  G.eta = veta.data();
  G.arc_a = varc.data();
  G.ec = vec.data();
  G.ecn = vecn.data();
  G.en = ven.data();
  PhysParams P{};
  P.gam = gam;
  // tangent-linear
  std::vector<double> Wv(W, W + (size_t)kDim * fp), Vv(V, V + (size_t)kDim * fp);
  std::vector<double> up((size_t)kDim * PS, 0.0), dup((size_t)kDim * PS, 0.0);
  recon_face<Dual<1>>(G, P, dt, Planes<Dual<1>>{Wv.data(), Vv.data(), 0},
                      Planes<Dual<1>>{up.data(), dup.data(), 0}, 0);
  std::vector<double> upv((size_t)kDim * PS, 0.0);
  recon_face<double>(G, P, dt, Planes<double>{Wv.data()}, Planes<double>{upv.data()}, 0);
  int mismatch = 0;
  double tlm = 0.0;
  for (int k = 0; k < kDim; ++k)
    for (int j = 0; j < n; ++j) {
      const size_t s = (size_t)k * PS + (size_t)j * fp;
      tlm += upb[k * n + j] * dup[s];
      uplus[k * n + j] = upv[s];
      if (std::memcmp(&up[s], &upv[s], sizeof(double)) != 0) mismatch = 1;
    }
  // the recomputation's tape: edge states bit-identical to recon_face
  std::vector<double> upt((size_t)kDim * PS, 0.0), LJ((size_t)rev::kTapePlanes * PS, 0.0);
  rev::recon_face_tape(G, P, dt, Wv.data(), upt.data(), LJ.data(), 0);
  for (int k = 0; k < kDim; ++k)
    for (int j = 0; j < n; ++j) {
      const size_t s = (size_t)k * PS + (size_t)j * fp;
      if (std::memcmp(&upt[s], &upv[s], sizeof(double)) != 0) mismatch |= 2;
    }
  // reverse
  std::vector<double> UPB((size_t)kDim * PS, 0.0), PU((size_t)2 * kDim * PS, 0.0), Wb((size_t)kDim * fp, 0.0);
  for (int k = 0; k < kDim; ++k)
    for (int j = 0; j < n; ++j) UPB[(size_t)k * PS + (size_t)j * fp] = upb[k * n + j];
  double wb[kDim] = {0, 0, 0, 0, 0};
  rev::recon_face_rev(
      G, P, dt, Wv.data(), upt.data(), LJ.data(), [&](int k, int s) { return UPB[(size_t)k * PS + s]; }, PU.data(),
      wb, 0);
  for (int k = 0; k < kDim; ++k) Wb[(size_t)k * fp] += wb[k];
  for (int j = 0; j < n; ++j) {
    const size_t s = (size_t)j * fp;
    for (int p = 0; p < 4; ++p) {
      const int gface = vsten[(size_t)p * PS + s];
      const double bt = vbeta[(size_t)p * PS + s];
      for (int k = 0; k < kDim; ++k)
        Wb[(size_t)k * fp + gface] += bt * PU[(size_t)(k + (p >= 2 ? kDim : 0)) * PS + s];
    }
  }
  double adj = 0.0;
  for (size_t i = 0; i < Wb.size(); ++i) adj += Wb[i] * Vv[i];
  out[0] = tlm;
  out[1] = adj;
  return mismatch;
}

// Source term (res) at state w with parameters prm = (acc0, omega_y,
// omega_z, acc_rate, total_mass); phys = (gam, omega_ns, e_acc, alpha).
void adj_source_eval(const double* w, const double* fcn, const double* prm, const double* phys, int friction_on,
                     double* res) {
  const PhysParams P = phys_from(phys, 1, friction_on, 2);
  const SrcParams<double> sp{prm[0], d3(0.0, prm[1], prm[2]), prm[3], prm[4]};
  source_term(w, d3(fcn[0], fcn[1], fcn[2]), sp, P, res);
}

// Rows i of the 5x10 Jacobian of the source over (w, prm) by source_rev.
void adj_source_jac(const double* w, const double* fcn, const double* prm, const double* phys, int friction_on,
                    double* J) {
  const PhysParams P = phys_from(phys, 1, friction_on, 2);
  const SrcParams<double> sp{prm[0], d3(0.0, prm[1], prm[2]), prm[3], prm[4]};
  for (int i = 0; i < kDim; ++i) {
    double sb[kDim] = {0, 0, 0, 0, 0}, wb[kDim] = {0, 0, 0, 0, 0}, pb[5] = {0, 0, 0, 0, 0};
    sb[i] = 1.0;
    rev::source_rev(w, d3(fcn[0], fcn[1], fcn[2]), sp, P, sb, wb, pb);
    for (int k = 0; k < kDim; ++k) J[i * 10 + k] = wb[k];
    for (int k = 0; k < 5; ++k) J[i * 10 + 5 + k] = pb[k];
  }
}

// (Sigma, l, Pi) of a conserved state and the 5x5 Jacobian by prim_rev.
void adj_prim(const double* u, const double* r, double gam, double* w, double* J) {
  const D3 rr = d3(r[0], r[1], r[2]);
  prim_of(u, rr, gam, w);
  for (int i = 0; i < kDim; ++i) {
    double wb[kDim] = {0, 0, 0, 0, 0}, ub[kDim] = {0, 0, 0, 0, 0};
    wb[i] = 1.0;
    rev::prim_rev(u, rr, gam, wb, ub);
    for (int k = 0; k < kDim; ++k) J[i * kDim + k] = ub[k];
  }
}

}  // extern "C"
