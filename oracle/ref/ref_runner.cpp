// Test-oracle driver for the reference SPLASH solver.
//
// This file is test infrastructure only.  It is compiled together with the
// reference's own headers and vendored pmp sources (read in place from the
// reference checkout, never copied) by oracle/ref/Makefile, and its output
// binary lives in oracle/_ref/.  tests/golden/gen_golden.py runs it to produce
// the committed golden fixtures that pin the CPU restatement in
// oracle/splash_oracle.cpp.
//
// What it does (mirrors the reference driver test.cpp:11-149 without the
// writers):
//   * builds the mesh with the reference generators (sph_gen.h:267-295);
//   * reads input/input.dat from the working directory (test.cpp:34-77);
//   * constructs one of the four solver classes (test.cpp:79-82), which reads
//     input/parameters.json (physics/adiabatic.hpp:59-68);
//   * dumps the geometry members (geometry/MUSCL_geometry.hpp:23-40) and the
//     conserved state after selected steps as raw little-endian binary.
//
// Probe<S> exposes protected members through a derived class; nothing in the
// reference is modified.
#include <chrono>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

#include "src/Riemann_solvers/HLLE.hpp"
#include "src/Riemann_solvers/HLLE_p.hpp"
#include "src/Riemann_solvers/HLLC.hpp"
#include "src/Riemann_solvers/HLLCplus.hpp"

namespace {

FILE* open_out(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  return f;
}

void put_i64(FILE* f, int64_t v) { std::fwrite(&v, sizeof v, 1, f); }
void put_f64(FILE* f, double v) { std::fwrite(&v, sizeof v, 1, f); }

template <class Base>
class Probe : public Base {
 public:
  using Base::Base;

  // Geometry dump: a flat sequence of int64 / float64 records, in the order
  // the reader in tests/golden/gen_golden.py expects.
  void dump_geometry(const std::string& path) {
    FILE* f = open_out(path);
    const int64_t nv = (int64_t)this->vertices.size();
    const int64_t nf = (int64_t)this->faces.size();
    put_i64(f, nv);
    put_i64(f, nf);
    for (auto& v : this->vertices)
      for (int k = 0; k < 3; ++k) put_f64(f, v[k]);
    for (auto& fc : this->faces) put_i64(f, (int64_t)fc.size());
    for (auto& fc : this->faces)
      for (int v : fc) put_i64(f, v);
    for (auto& nb : this->neighbors) put_i64(f, (int64_t)nb.size());
    for (auto& nb : this->neighbors)
      for (int v : nb) put_i64(f, v);
    for (auto& nb : this->neighbors_edge) put_i64(f, (int64_t)nb.size());
    for (auto& nb : this->neighbors_edge)
      for (int v : nb) put_i64(f, v);
    for (auto& c : this->face_centers)
      for (int k = 0; k < 3; ++k) put_f64(f, c[k]);
    for (auto& c : this->normals)
      for (int k = 0; k < 3; ++k) put_f64(f, c[k]);
    for (double a : this->surface_area) put_f64(f, a);
    for (int64_t i = 0; i < nf; ++i) {
      const size_t ns = this->faces[i].size();
      for (size_t j = 0; j < ns; ++j) {
        for (int k = 0; k < 3; ++k) put_f64(f, this->edge_normals[i][j][k]);
        put_f64(f, this->BM_dist[i][j]);
        put_f64(f, this->H_plus[i][j]);
        put_f64(f, this->H_minus[i][j]);
        put_i64(f, this->flux_faces_plus[i][j][0]);
        put_i64(f, this->flux_faces_plus[i][j][1]);
        put_i64(f, this->flux_faces_minus[i][j][0]);
        put_i64(f, this->flux_faces_minus[i][j][1]);
        put_f64(f, this->betas_plus[i][j][0]);
        put_f64(f, this->betas_plus[i][j][1]);
        put_f64(f, this->betas_minus[i][j][0]);
        put_f64(f, this->betas_minus[i][j][1]);
      }
    }
    put_f64(f, this->h0);
    std::fclose(f);
  }

  void dump_state(FILE* f) {
    put_f64(f, this->t);
    put_f64(f, this->dt);
    put_i64(f, this->stop_check ? 1 : 0);
    put_i64(f, (int64_t)this->steps);
    for (auto& u : this->U)
      for (int k = 0; k < this->dim; ++k) put_f64(f, u[k]);
  }

  double get_area_coeff() { return this->area_coeff; }
  double get_total_mass() { return this->total_mass; }

  // Per-function known-answer vectors on seeded inputs.  Each record:
  // face, edge, uL, uR, u_source, r, U[face], flux_star, limiter, source.  The state U is overwritten with a seeded
  // random field (field 4 holds the pressure, as inside a stage,
  // MUSCL_base.hpp:366-371) so that the limiter sees a consistent stencil.
  void dump_functions(const std::string& path, uint64_t seed, int nsamp, double dt_member) {
    FILE* f = open_out(path);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    const int nf = (int)this->faces.size();
    const int dim = this->dim;
    this->dt = dt_member;
    // random primitive-ish state per face: field 4 = pressure
    for (int i = 0; i < nf; ++i) {
      this->U[i][0] = 0.5 + 1.5 * uni(rng);
      for (int k = 1; k < 4; ++k) this->U[i][k] = 0.2 * (uni(rng) - 0.5);
      this->U[i][4] = 0.3 + 1.2 * uni(rng);
    }
    put_i64(f, nsamp);
    put_i64(f, dim);
    put_f64(f, dt_member);
    for (int s = 0; s < nsamp; ++s) {
      int face = (int)(uni(rng) * nf);
      if (face >= nf) face = nf - 1;
      int edge = (int)(uni(rng) * this->faces[face].size());
      if (edge >= (int)this->faces[face].size()) edge = 0;
      // conserved edge states (field 4 = energy) for flux_star
      std::vector<double> ul(dim), ur(dim), uc(dim), r(dim);
      auto make_state = [&](std::vector<double>& u, double shear) {
        u[0] = 0.3 + 1.7 * uni(rng);
        for (int k = 1; k < 4; ++k) u[k] = shear * (uni(rng) - 0.5);
        double vel2_bound = 0.0;
        for (int k = 1; k < 4; ++k) vel2_bound += u[k] * u[k];
        vel2_bound /= (u[0] * u[0]);
        // E large enough that the pressure stays positive
        u[4] = u[0] * vel2_bound / 2 + (0.2 + 2.0 * uni(rng)) / (this->gam - 1);
      };
      const double shear = (s % 3 == 0) ? 2.0 : 0.4;
      make_state(ul, shear);
      make_state(ur, shear);
      if (s % 7 == 0) ur = ul;  // identical states
      // source input: field 4 is the pressure (adiabatic.hpp:398)
      uc[0] = 0.3 + 1.7 * uni(rng);
      for (int k = 1; k < 4; ++k) uc[k] = 0.4 * (uni(rng) - 0.5);
      uc[4] = 0.2 + 2.0 * uni(rng);
      // limiter ratios, including the IEEE special cases the reference hits
      for (int k = 0; k < dim; ++k) {
        const int kind = (s * 5 + k) % 11;
        switch (kind) {
          case 0: r[k] = std::nan(""); break;
          case 1: r[k] = 1.0 / 0.0; break;
          case 2: r[k] = -1.0 / 0.0; break;
          case 3: r[k] = 0.0; break;
          case 4: r[k] = 1.0; break;
          case 5: r[k] = -3.0 * uni(rng); break;
          case 6: r[k] = uni(rng); break;
          case 7: r[k] = 1.0 + 4.0 * uni(rng); break;
          case 8: r[k] = 1.0 + 1e-3 * uni(rng); break;
          case 9: r[k] = 1e-3 * uni(rng); break;
          default: r[k] = 20.0 * uni(rng); break;
        }
      }
      std::vector<double> F = this->flux_star(ul, ur, face, edge);
      std::vector<double> lim = this->limiter(r, face, edge);
      std::vector<double> src = this->source(uc, face);
      put_i64(f, face);
      put_i64(f, edge);
      for (double v : ul) put_f64(f, v);
      for (double v : ur) put_f64(f, v);
      for (double v : uc) put_f64(f, v);
      for (double v : r) put_f64(f, v);
      for (int k = 0; k < dim; ++k) put_f64(f, this->U[face][k]);
      for (double v : F) put_f64(f, v);
      for (double v : lim) put_f64(f, v);
      for (double v : src) put_f64(f, v);
    }
    std::fclose(f);
  }
};

// Isothermal solver (MUSCL_HLLE, dim 4): its flux (isothermal.hpp:141-195),
// char_vel (:211-260) and flux_star (HLLE.hpp:17-59) are defined for 4-field
// states and are dumped on seeded inputs; its limiter reads an
// uninitialised variable (:272, 301-307) and its step reads and writes a
// fifth field (MUSCL_base.hpp:203, 324, 368-370), so neither is dumped.
// Each record: face, edge, uL[4], uR[4], flux(uL)[4], char_vel[2],
// flux_star[4].
template <class Base>
class IsoProbe : public Base {
 public:
  using Base::Base;
  void dump_iso_functions(const std::string& path, uint64_t seed, int nsamp) {
    FILE* f = open_out(path);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    const int nf = (int)this->faces.size();
    put_i64(f, nsamp);
    for (int s = 0; s < nsamp; ++s) {
      int face = (int)(uni(rng) * nf);
      if (face >= nf) face = nf - 1;
      int edge = (int)(uni(rng) * this->faces[face].size());
      if (edge >= (int)this->faces[face].size()) edge = 0;
      std::vector<double> ul(4), ur(4);
      // speeds up to a few times the sound speed a = 1, both signs
      const double shear = (s % 3 == 0) ? 6.0 : 1.0;
      for (auto* u : {&ul, &ur}) {
        (*u)[0] = 0.3 + 1.7 * uni(rng);
        for (int k = 1; k < 4; ++k) (*u)[k] = shear * (uni(rng) - 0.5);
      }
      if (s % 7 == 0) ur = ul;
      std::vector<double> fl = this->flux(ul, face, edge);
      std::vector<double> cv = this->char_vel(ul, ur, face, edge);
      std::vector<double> F = this->flux_star(ul, ur, face, edge);
      put_i64(f, face);
      put_i64(f, edge);
      for (double v : ul) put_f64(f, v);
      for (double v : ur) put_f64(f, v);
      for (double v : fl) put_f64(f, v);
      for (double v : cv) put_f64(f, v);
      for (double v : F) put_f64(f, v);
    }
    std::fclose(f);
  }
};

template <class Solver>
int run(SurfaceMesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
        double omega_ns, bool acc, size_t threads, double dt, int nsteps, int dump_every,
        const std::string& out, const std::string& mode, uint64_t seed, int nsamp) {
  Probe<Solver> s(mesh, U_in, dim, gam, omega_ns, acc, threads);
  if (mode == "geometry") {
    s.dump_geometry(out + "_geom.bin");
    FILE* f = open_out(out + "_scalars.txt");
    std::fprintf(f, "%.17g %.17g\n", s.get_area_coeff(), s.get_total_mass());
    std::fclose(f);
    return 0;
  }
  if (mode == "functions") {
    s.dump_functions(out + "_funcs.bin", seed, nsamp, dt);
    return 0;
  }
  if (mode == "writers") {
    // The reference driver's output sequence (test.cpp:84-149): geometry
    // and state writers at t = 0, light curves after every step, state
    // writers and the final state at the end.  Files land in results/.
    s.write_face_centers();
    s.write_faces();
    s.write_vertices();
    s.write_t_rho();
    s.write_t_p();
    s.write_t_omega_z();
    s.write_t_L();
    FILE* lc = open_out(out + "_lightcurves.txt");
    std::vector<double> l = s.get_light_curves();
    std::fprintf(lc, "%.17g %.17g %.17g %.17g %.17g\n", s.time(), l[0], l[1], l[2], l[3]);
    for (int i = 0; i < nsteps; ++i) {
      s.do_step(dt);
      l = s.get_light_curves();
      std::fprintf(lc, "%.17g %.17g %.17g %.17g %.17g\n", s.time(), l[0], l[1], l[2], l[3]);
    }
    std::fclose(lc);
    s.write_t_rho();
    s.write_t_p();
    s.write_t_curl();
    s.write_t_omega_z();
    s.write_t_L();
    s.write_final_state();
    return 0;
  }
  if (mode == "time") {
    // Times only the do_step loop (construction excluded), stdout discarded
    // by the caller.
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < nsteps; ++i) s.do_step(dt);
    auto t1 = std::chrono::steady_clock::now();
    const double sec = std::chrono::duration<double>(t1 - t0).count();
    FILE* f = open_out(out + "_time.txt");
    std::fprintf(f, "%.9g %d %d\n", sec, nsteps, (int)U_in.size());
    std::fclose(f);
    return 0;
  }
  // mode == "run": dump the state after steps 0, dump_every, 2*dump_every ...
  FILE* f = open_out(out + "_states.bin");
  s.dump_state(f);
  for (int i = 1; i <= nsteps; ++i) {
    s.do_step(dt);
    if (dump_every > 0 && (i % dump_every == 0 || i == nsteps)) s.dump_state(f);
  }
  std::fclose(f);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 14) {
    std::fprintf(stderr,
                 "usage: ref_runner mode mesh level solver dim gam omega_ns accretion_on threads "
                 "dt nsteps dump_every outprefix [seed nsamp]\n");
    return 1;
  }
  const std::string mode = argv[1];
  const std::string meshkind = argv[2];
  const int level = std::atoi(argv[3]);
  const std::string solver = argv[4];
  const int dim = std::atoi(argv[5]);
  const double gam = std::atof(argv[6]);
  const double omega_ns = std::atof(argv[7]);
  const bool acc = std::atoi(argv[8]) != 0;
  const size_t threads = (size_t)std::atoi(argv[9]);
  const double dt = std::atof(argv[10]);
  const int nsteps = std::atoi(argv[11]);
  const int dump_every = std::atoi(argv[12]);
  const std::string out = argv[13];
  const uint64_t seed = argc > 14 ? std::strtoull(argv[14], nullptr, 10) : 0;
  const int nsamp = argc > 15 ? std::atoi(argv[15]) : 0;

  SurfaceMesh mesh;
  if (meshkind == "hex")
    mesh = icosphere_hex(level);
  else if (meshkind == "quad")
    mesh = quad_sphere(level);
  else if (meshkind == "ico")
    mesh = icosphere(level);
  else {
    std::fprintf(stderr, "unknown mesh %s\n", meshkind.c_str());
    return 1;
  }

  // input/input.dat, same reading rule as test.cpp:48-77
  std::vector<std::vector<double>> U_in(mesh.n_faces(), std::vector<double>(dim, 1.0));
  {
    std::ifstream in("input/input.dat");
    std::vector<double> tmp;
    double e;
    while (in >> e) tmp.push_back(e);
    if (tmp.size() < mesh.n_faces() * (size_t)dim) tmp.resize(mesh.n_faces() * dim, 1.0);
    for (size_t i = 0; i < mesh.n_faces(); ++i)
      for (int k = 0; k < dim; ++k) U_in[i][k] = tmp[i * dim + k];
  }

  if (solver == "HLLE") {
    if (mode != "iso_functions") {
      std::fprintf(stderr, "the isothermal solver supports only mode iso_functions\n");
      return 1;
    }
    IsoProbe<MUSCL_HLLE> s(mesh, U_in, dim, gam, threads);
    s.dump_iso_functions(out + "_isofuncs.bin", seed, nsamp);
    return 0;
  }
  if (solver == "HLLE_p")
    return run<MUSCL_HLLE_p>(mesh, U_in, dim, gam, omega_ns, acc, threads, dt, nsteps, dump_every,
                             out, mode, seed, nsamp);
  if (solver == "HLLC")
    return run<MUSCL_HLLC>(mesh, U_in, dim, gam, omega_ns, acc, threads, dt, nsteps, dump_every,
                           out, mode, seed, nsamp);
  if (solver == "HLLCplus")
    return run<MUSCL_HLLCplus>(mesh, U_in, dim, gam, omega_ns, acc, threads, dt, nsteps,
                               dump_every, out, mode, seed, nsamp);
  std::fprintf(stderr, "unknown solver %s\n", solver.c_str());
  return 1;
}
