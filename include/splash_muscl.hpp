// splash_muscl.hpp — C++ drop-in for the reference solver classes.
//
// Header-only wrappers with the reference's class names and member
// functions, forwarding to the C ABI of splash_gb300.h (link with
// -lsplash_gb300).  They behave like the reference objects a driver such as
// the reference's test.cpp uses:
//
//   MUSCL_HLLE_p / MUSCL_HLLC / MUSCL_HLLCplus (Riemann_solvers/*.hpp:11-13)
//     ctor (mesh, U_in, dim, gam, omega_ns, accretion_on, threads): reads
//     input/parameters.json like physics/adiabatic.hpp:59-68 and truncates
//     the results/*.dat files like physics/adiabatic.hpp:32-57;
//   do_step, time, get_stop_check                 (MUSCL_base.hpp:97-235)
//   write_t_rho/p/curl/omega_z/L, get_light_curves, write_final_state
//                                                  (physics/adiabatic.hpp:101-348)
//   write_face_centers/faces/vertices             (MUSCL_geometry.hpp:1069-1117)
//
// Meshes: splash::icosphere_hex / quad_sphere / icosphere produce the
// reference numbering (geometry/sph_gen.h:267-295); any mesh type with the
// pmp SurfaceMesh iteration API converts with splash::from_surface_mesh.
//
// Define SPLASH_REFERENCE_NAMES before including to also get the names a
// reference driver uses unqualified: namespace pmp { SurfaceMesh,
// icosphere_hex, quad_sphere, icosphere } and a `json` type with parse().
#pragma once

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "splash_gb300.h"

namespace splash {

// ------------------------------------------------------------------ errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const char* what) {
  if (rc != SPLASH_OK) throw Error(rc, std::string(what) + ": " + splash_last_error());
}

// ------------------------------------------------------------------ meshes
// A mesh request: a reference generator (kind, level) or explicit arrays.
struct Mesh {
  int kind = -1;
  int level = 0;
  std::vector<double> vertices;  // [nv][3]
  std::vector<int> face_off;     // [nf + 1]
  std::vector<int> face_vtx;

  size_t n_faces() const {
    if (kind < 0) return face_off.empty() ? 0 : face_off.size() - 1;
    const size_t p = (size_t)1 << (2 * level);  // 4^level
    if (kind == SPLASH_MESH_ICOSPHERE_HEX) return 10 * p + 2;
    if (kind == SPLASH_MESH_QUAD_SPHERE) return 6 * p;
    return 20 * p;
  }

  splash_mesh_desc desc() const {
    splash_mesh_desc d{};
    d.kind = kind;
    d.level = level;
    if (kind < 0) {
      d.n_vertices = (int)(vertices.size() / 3);
      d.vertices = vertices.data();
      d.n_faces = (int)n_faces();
      d.face_offsets = face_off.data();
      d.face_vertices = face_vtx.data();
    }
    return d;
  }
};

inline Mesh icosphere_hex(size_t n) { return Mesh{SPLASH_MESH_ICOSPHERE_HEX, (int)n, {}, {}, {}}; }
inline Mesh quad_sphere(size_t n) { return Mesh{SPLASH_MESH_QUAD_SPHERE, (int)n, {}, {}, {}}; }
inline Mesh icosphere(size_t n) { return Mesh{SPLASH_MESH_ICOSPHERE, (int)n, {}, {}, {}}; }

// Converts a mesh with pmp's SurfaceMesh API (vertices(), faces(),
// position(v), vertices(f), idx()) keeping its own element order.
template <class SurfaceMeshT>
Mesh from_surface_mesh(const SurfaceMeshT& m) {
  Mesh out;
  for (auto v : m.vertices()) {
    const auto& p = m.position(v);
    out.vertices.push_back((double)p[0]);
    out.vertices.push_back((double)p[1]);
    out.vertices.push_back((double)p[2]);
  }
  out.face_off.push_back(0);
  for (auto f : m.faces()) {
    for (auto v : m.vertices(f)) out.face_vtx.push_back((int)v.idx());
    out.face_off.push_back((int)out.face_vtx.size());
  }
  return out;
}

// ------------------------------------------------------- minimal JSON reader
// Reads the flat object of input/parameters.json: numbers, booleans and
// strings, with implicit conversion like nlohmann::json's value access.
class Json {
 public:
  struct Value {
    std::string text;
    bool is_string = false;
    operator double() const { return std::strtod(text.c_str(), nullptr); }
    operator float() const { return (float)std::strtod(text.c_str(), nullptr); }
    operator int() const { return (int)std::strtoll(text.c_str(), nullptr, 10); }
    operator long() const { return (long)std::strtoll(text.c_str(), nullptr, 10); }
    operator long long() const { return std::strtoll(text.c_str(), nullptr, 10); }
    operator unsigned long() const { return (unsigned long)std::strtoull(text.c_str(), nullptr, 10); }
    operator unsigned long long() const { return std::strtoull(text.c_str(), nullptr, 10); }
    operator bool() const { return text == "true" || (text != "false" && std::strtod(text.c_str(), nullptr) != 0); }
    operator std::string() const { return text; }
  };

  static Json parse(std::istream& is) {
    std::stringstream ss;
    ss << is.rdbuf();
    return parse(ss.str());
  }
  static Json parse(const std::string& s) {
    Json j;
    size_t i = 0;
    auto skip = [&] { while (i < s.size() && std::isspace((unsigned char)s[i])) ++i; };
    auto str = [&] {
      std::string out;
      ++i;  // opening quote
      while (i < s.size() && s[i] != '"') {
        if (s[i] == '\\' && i + 1 < s.size()) ++i;
        out += s[i++];
      }
      ++i;
      return out;
    };
    skip();
    if (i >= s.size() || s[i] != '{') throw Error(SPLASH_E_INVALID, "json: expected an object");
    ++i;
    for (;;) {
      skip();
      if (i < s.size() && s[i] == '}') break;
      if (i >= s.size() || s[i] != '"') throw Error(SPLASH_E_INVALID, "json: expected a key");
      const std::string key = str();
      skip();
      if (i >= s.size() || s[i] != ':') throw Error(SPLASH_E_INVALID, "json: expected ':'");
      ++i;
      skip();
      Value v;
      if (i < s.size() && s[i] == '"') {
        v.text = str();
        v.is_string = true;
      } else {
        while (i < s.size() && s[i] != ',' && s[i] != '}' && !std::isspace((unsigned char)s[i])) v.text += s[i++];
      }
      j.values_[key] = v;
      skip();
      if (i < s.size() && s[i] == ',') {
        ++i;
        continue;
      }
      if (i < s.size() && s[i] == '}') break;
      throw Error(SPLASH_E_INVALID, "json: expected ',' or '}'");
    }
    return j;
  }
  const Value& operator[](const std::string& k) const {
    auto it = values_.find(k);
    if (it == values_.end()) throw Error(SPLASH_E_INVALID, "json: missing key " + k);
    return it->second;
  }
  bool contains(const std::string& k) const { return values_.count(k) != 0; }

 private:
  std::map<std::string, Value> values_;
};

// ------------------------------------------------------------------ solvers
class Solver {
 public:
  Solver(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
         double omega_ns, bool accretion_on, size_t threads, int solver_kind,
         int precision = SPLASH_PREC_FP64, int device = 0,
         const std::string& parameters = "input/parameters.json")
      : mesh_(mesh), dim_(dim) {
    std::ifstream ifs(parameters);
    if (!ifs) throw Error(SPLASH_E_INVALID, "cannot open " + parameters);
    const Json p = Json::parse(ifs);
    splash_params par{};
    par.accretion_rate = p["accretion_rate"];
    par.e_acc = p["e_acc"];
    par.omega_acc_abs = p["omega_acc_abs"];
    par.tilt_angle = p["tilt_angle"];
    par.acc_width = p["acc_width"];
    par.alpha = p["alpha"];
    par.friction_on = (bool)p["friction_on"] ? 1 : 0;
    // the reference constructor truncates its output files
    for (const char* f : {"results/rho.dat", "results/curl.dat", "results/p.dat", "results/omega.dat",
                          "results/Lx.dat", "results/Ly.dat", "results/Lz.dat"})
      std::ofstream(f, std::ios::out | std::ios::trunc);
    create(U_in, dim, gam, omega_ns, accretion_on, threads, solver_kind, precision, device, par);
  }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;
  virtual ~Solver() { splash_destroy(h_); }

 protected:
  // The isothermal constructor (physics/isothermal.hpp:13-40): no
  // parameters.json, four output files truncated.
  struct IsothermalTag {};
  Solver(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam, size_t threads,
         int precision, int device, IsothermalTag)
      : mesh_(mesh), dim_(dim) {
    for (const char* f : {"results/rho.dat", "results/curl.dat", "results/p.dat", "results/omega.dat"})
      std::ofstream(f, std::ios::out | std::ios::trunc);
    splash_params par{};
    par.acc_width = 0.1;
    create(U_in, dim, gam, 0.0, false, threads, SPLASH_SOLVER_HLLE, precision, device, par);
  }

 private:
  void create(const std::vector<std::vector<double>>& U_in, int dim, double gam, double omega_ns,
              bool accretion_on, size_t threads, int solver_kind, int precision, int device,
              const splash_params& par) {
    std::vector<double> flat;
    flat.reserve(U_in.size() * (size_t)dim);
    for (const auto& row : U_in) {
      if ((int)row.size() != dim) throw Error(SPLASH_E_INVALID, "U_in row size differs from dim");
      flat.insert(flat.end(), row.begin(), row.end());
    }
    const splash_mesh_desc d = mesh_.desc();
    check(splash_create(&d, flat.data(), dim, gam, omega_ns, accretion_on ? 1 : 0, &par, solver_kind,
                        precision, device, (int)threads, &h_),
          "splash_create");
  }

 public:
  void do_step(double dt0) {
    check(splash_do_step(h_, dt0), "do_step");
    if (log_) log_step();
  }
  // The reference prints one line per do_step (MUSCL_base.hpp:187-213):
  // "t= <t> mass_relative_gain=<M/M_1 - 1> (l/mass)_total_norm= <|L|>
  // l_total = (<Lx>,<Ly>,<Lz>)" with M, L the area-weighted sums after the
  // step and M_1 the mass after the first step.  Here it is off by default
  // (it synchronises every step); set_step_log(&std::cout) turns it on.
  void set_step_log(std::ostream* os) { log_ = os; }
  double time() {
    double t = 0;
    check(splash_time(h_, &t), "time");
    return t;
  }
  bool get_stop_check() {
    int s = 0;
    check(splash_stop_check(h_, &s), "get_stop_check");
    return s != 0;
  }
  std::vector<std::vector<double>> state() {
    int nf = 0;
    check(splash_n_faces(h_, &nf), "n_faces");
    std::vector<double> flat((size_t)nf * dim_);
    check(splash_get_state(h_, flat.data()), "get_state");
    std::vector<std::vector<double>> U((size_t)nf, std::vector<double>(dim_));
    for (int i = 0; i < nf; ++i)
      for (int k = 0; k < dim_; ++k) U[i][k] = flat[(size_t)i * dim_ + k];
    return U;
  }

  void write_t_rho() { check(splash_write_t_rho(h_, "results/rho.dat"), "write_t_rho"); }
  void write_t_p() { check(splash_write_t_p(h_, "results/p.dat"), "write_t_p"); }
  void write_t_curl() { check(splash_write_t_curl(h_, "results/curl.dat"), "write_t_curl"); }
  void write_t_omega_z() { check(splash_write_t_omega_z(h_, "results/omega.dat"), "write_t_omega_z"); }
  void write_t_L() {
    check(splash_write_t_L(h_, "results/Lx.dat", "results/Ly.dat", "results/Lz.dat"), "write_t_L");
  }
  std::vector<double> get_light_curves() {
    std::vector<double> out(4);
    check(splash_get_light_curves(h_, out.data()), "get_light_curves");
    return out;
  }
  void write_final_state() { check(splash_write_final_state(h_, "results/final_state.dat"), "write_final_state"); }

  // geometry writers (setprecision(15), MUSCL_geometry.hpp:1069-1117)
  void write_face_centers() {
    Geometry g(mesh_);
    std::ofstream os("results/face_centers.dat");
    const std::vector<double>& u = g.d("unit_face_centers");
    for (size_t i = 0; i + 2 < u.size(); i += 3)
      os << std::setprecision(15) << u[i] << " " << u[i + 1] << " " << u[i + 2] << "\n";
  }
  void write_faces() {
    Geometry g(mesh_);
    std::ofstream os("results/faces.dat");
    const std::vector<int>& off = g.i("face_off");
    const std::vector<int>& fv = g.i("face_vtx");
    for (size_t f = 0; f + 1 < off.size(); ++f) {
      for (int s = off[f]; s < off[f + 1]; ++s) os << fv[s] << " ";
      os << "\n";
    }
  }
  void write_vertices() {
    Geometry g(mesh_);
    std::ofstream os("results/vertices.dat");
    const std::vector<double>& v = g.d("vertices");
    for (size_t i = 0; i + 2 < v.size(); i += 3) {
      for (int k = 0; k < 3; ++k) os << std::setprecision(15) << v[i + k] << " ";
      os << "\n";
    }
  }

  splash_solver* handle() { return h_; }

 private:
  // reference-numbered geometry arrays through the C ABI
  struct Geometry {
    splash_geometry* g = nullptr;
    std::map<std::string, std::vector<double>> dd;
    std::map<std::string, std::vector<int>> ii;
    explicit Geometry(const Mesh& m) {
      const splash_mesh_desc d = m.desc();
      check(splash_geometry_build(&d, 0, &g), "splash_geometry_build");
    }
    ~Geometry() { splash_geometry_free(g); }
    const std::vector<double>& d(const char* name) {
      size_t n = 0;
      check(splash_geometry_get(g, name, nullptr, 0, &n), name);
      std::vector<double>& v = dd[name];
      v.resize(n / sizeof(double));
      check(splash_geometry_get(g, name, v.data(), n, nullptr), name);
      return v;
    }
    const std::vector<int>& i(const char* name) {
      size_t n = 0;
      check(splash_geometry_get(g, name, nullptr, 0, &n), name);
      std::vector<int>& v = ii[name];
      v.resize(n / sizeof(int));
      check(splash_geometry_get(g, name, v.data(), n, nullptr), name);
      return v;
    }
  };

  void log_step() {
    double d[5];
    check(splash_diagnostics(h_, d), "diagnostics");
    if (logged_ == 0) mass_first_ = d[0];
    ++logged_;
    *log_ << "t= " << time() << " mass_relative_gain=" << d[0] / mass_first_ - 1
          << " (l/mass)_total_norm= " << std::sqrt(d[1] * d[1] + d[2] * d[2] + d[3] * d[3]) << " l_total = ("
          << d[1] << "," << d[2] << "," << d[3] << ")"
          << "\n";
  }

  Mesh mesh_;
  int dim_;
  splash_solver* h_ = nullptr;
  std::ostream* log_ = nullptr;
  long logged_ = 0;
  double mass_first_ = 0.0;
};

// Riemann_solvers/HLLE.hpp:11-13: the isothermal solver, dim 4 (its
// writers are write_t_rho, write_t_p, write_t_curl and write_t_omega_z)
class MUSCL_HLLE : public Solver {
 public:
  MUSCL_HLLE(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam, size_t threads,
             int precision = SPLASH_PREC_FP64, int device = 0)
      : Solver(mesh, U_in, dim, gam, threads, precision, device, IsothermalTag{}) {}
};

// Riemann_solvers/HLLE_p.hpp:11-13
class MUSCL_HLLE_p : public Solver {
 public:
  MUSCL_HLLE_p(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
               double omega_ns_i, bool accretion_on_i, size_t threads, int precision = SPLASH_PREC_FP64)
      : Solver(mesh, U_in, dim, gam, omega_ns_i, accretion_on_i, threads, SPLASH_SOLVER_HLLE_P, precision) {}
  // the README form (mesh, U_in, dim, gam, omega_ns): accretion off
  MUSCL_HLLE_p(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
               double omega_ns_i)
      : MUSCL_HLLE_p(mesh, U_in, dim, gam, omega_ns_i, false, 0) {}
};

// Riemann_solvers/HLLC.hpp:11-13
class MUSCL_HLLC : public Solver {
 public:
  MUSCL_HLLC(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
             double omega_ns_i, bool accretion_on_i, size_t threads, int precision = SPLASH_PREC_FP64)
      : Solver(mesh, U_in, dim, gam, omega_ns_i, accretion_on_i, threads, SPLASH_SOLVER_HLLC, precision) {}
  MUSCL_HLLC(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
             double omega_ns_i)
      : MUSCL_HLLC(mesh, U_in, dim, gam, omega_ns_i, false, 0) {}
};

// Riemann_solvers/HLLCplus.hpp:11-13
class MUSCL_HLLCplus : public Solver {
 public:
  MUSCL_HLLCplus(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
                 double omega_ns_i, bool accretion_on_i, size_t threads, int precision = SPLASH_PREC_FP64)
      : Solver(mesh, U_in, dim, gam, omega_ns_i, accretion_on_i, threads, SPLASH_SOLVER_HLLCPLUS,
               precision) {}
  MUSCL_HLLCplus(const Mesh& mesh, const std::vector<std::vector<double>>& U_in, int dim, double gam,
                 double omega_ns_i)
      : MUSCL_HLLCplus(mesh, U_in, dim, gam, omega_ns_i, false, 0) {}
};

}  // namespace splash

#ifdef SPLASH_REFERENCE_NAMES
#include <cmath>
namespace pmp {
using SurfaceMesh = splash::Mesh;
using splash::icosphere;
using splash::icosphere_hex;
using splash::quad_sphere;
}  // namespace pmp
using json = splash::Json;
using splash::MUSCL_HLLE;
using splash::MUSCL_HLLC;
using splash::MUSCL_HLLCplus;
using splash::MUSCL_HLLE_p;
#endif
