// Drives the C++ drop-in classes (include/splash_muscl.hpp) through the
// output sequence of the reference driver: geometry and state writers at
// t = 0, light curves after every step, state writers and the final state
// at the end.  Run from a directory holding input/parameters.json,
// input/input.dat and results/.
//
//   drop_in_driver <hex|quad> <level> <solver 1|2|3> <steps> <dt0> <accretion 0|1>
#define SPLASH_REFERENCE_NAMES
#include "splash_muscl.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>

using namespace pmp;

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: drop_in_driver mesh level solver steps dt0 accretion\n");
    return 2;
  }
  const std::string kind = argv[1];
  const int level = std::atoi(argv[2]);
  const int solver = std::atoi(argv[3]);
  const int steps = std::atoi(argv[4]);
  const double dt0 = std::atof(argv[5]);
  const bool accretion = std::atoi(argv[6]) != 0;
  SurfaceMesh mesh = kind == "quad" ? quad_sphere(level) : icosphere_hex(level);

  std::ifstream ifs("input/parameters.json");
  json parameters = json::parse(ifs);
  const double gam3d = parameters["gam3d"];
  const double gam = 2 - 1 / gam3d;
  const double omega_ns = parameters["omega_ns"];
  const size_t threads = parameters["threads"];

  const size_t dim = 5;
  std::vector<std::vector<double>> U_in(mesh.n_faces(), std::vector<double>(dim, 1.0));
  {
    std::ifstream in("input/input.dat");
    double e;
    size_t k = 0;
    while (k < mesh.n_faces() * dim && in >> e) {
      U_in[k / dim][k % dim] = e;
      ++k;
    }
  }
  try {
    splash::Solver* s = nullptr;
    if (solver == 1)
      s = new MUSCL_HLLE_p(mesh, U_in, (int)dim, gam, omega_ns, accretion, threads);
    else if (solver == 2)
      s = new MUSCL_HLLC(mesh, U_in, (int)dim, gam, omega_ns, accretion, threads);
    else
      s = new MUSCL_HLLCplus(mesh, U_in, (int)dim, gam, omega_ns, accretion, threads);
    s->write_face_centers();
    s->write_faces();
    s->write_vertices();
    s->write_t_rho();
    s->write_t_p();
    s->write_t_omega_z();
    s->write_t_L();
    std::ofstream steplog("results/steplog.txt");
    s->set_step_log(&steplog);
    std::ofstream lc("results/lightcurves.txt");
    lc.precision(17);
    std::vector<double> l = s->get_light_curves();
    lc << s->time() << " " << l[0] << " " << l[1] << " " << l[2] << " " << l[3] << "\n";
    for (int i = 0; i < steps; ++i) {
      s->do_step(dt0);
      l = s->get_light_curves();
      lc << s->time() << " " << l[0] << " " << l[1] << " " << l[2] << " " << l[3] << "\n";
    }
    s->write_t_rho();
    s->write_t_p();
    s->write_t_curl();
    s->write_t_omega_z();
    s->write_t_L();
    s->write_final_state();
    std::cout << "steps " << steps << " t " << s->time() << " stop " << s->get_stop_check() << "\n";
    delete s;
  } catch (const splash::Error& e) {
    std::fprintf(stderr, "splash error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
