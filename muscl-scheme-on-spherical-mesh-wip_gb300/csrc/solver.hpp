// One solver instance: the host mirror of the reference object
// (MUSCL_base + adiabatic + a Riemann solver) with its device state.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "geometry.hpp"
#include "layout.hpp"
#include "splash_gb300.h"

namespace splash {

// True when the FP32/FP64 mixed kernels are compiled into the library.
bool mixed_available();

// Records the calling thread's error message (read by splash_last_error)
// and returns `code`.
int set_error(int code, const char* fmt, ...);

struct Solver {
  // configuration
  splash_params par{};
  bool accretion_on = false;
  int precision = SPLASH_PREC_FP64;
  int solver_kind = SPLASH_SOLVER_HLLCPLUS;
  int dim = 5;  // state fields: 5 adiabatic, 4 isothermal (MUSCL_HLLE)
  int device = -1;
  double area_coeff = 0.0;
  double total_mass = 0.0;

  // sizes
  int n_faces = 0;
  int fpad = 0;
  int max_slots = 0;
  int n_partials = 0;
  size_t geometry_bytes = 0;

  // numbering: perm[internal] = reference face id, iperm = inverse
  std::vector<int> perm, iperm;
  std::vector<int> h_slot_edge;  // mixed path: slot -> edge map (the writers' edge-state lookup)

  // reference-order host copies used by the writers
  std::vector<double> wr_vertices, wr_face_centers, wr_area;
  std::vector<int> wr_face_off, wr_face_vtx;

  // device
  cudaStream_t stream = nullptr;
  PhysParams P{};
  DevGeom G{};
  DevGeomMixed GM{};
  DevState S{};
  double* d_stage = nullptr;  // [n_faces][5] reference-order staging
  int* d_perm = nullptr;
  int* d_iperm = nullptr;   // reference face -> internal face
  // device diagnostics (diagnostics.cu): observer planes, partials, results
  double* d_cos_obs = nullptr;
  double* d_diag_partial = nullptr;
  double* d_diag_out = nullptr;
  double* h_diag = nullptr;  // pinned, 9 doubles
  int run_diagnostics(double* out9);
  bool host_direct = false; // the device reads and writes pageable host memory (coherent link)
  double* h_stage = nullptr;  // pinned mirror of d_stage
  std::vector<void*> dev_allocs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  cudaGraphNode_t dt0_node = nullptr;  // mixed path: the stage-1 edge node taking dt0
  double graph_dt0 = 0.0;              // dt0 the instantiated graphs currently use
  // mixed path: kGraphSteps consecutive steps in one graph, so that each
  // step's first launch overlaps the previous step's last one (programmatic
  // dependent launch works within a graph, not across graph launches)
  static constexpr int kGraphSteps = 4;
  cudaGraph_t graph_k = nullptr;
  cudaGraphExec_t graph_k_exec = nullptr;
  std::vector<cudaGraphNode_t> dt0_nodes_k;
  int64_t steps = 0;

  ~Solver();

  template <typename T>
  T* dalloc(size_t n);
  template <typename T>
  T* upload(const std::vector<T>& h);

  void build_device_geometry(const RefGeometry& g);
  int upload_state(const double* U_ref);
  int download_state(double* U_ref);
  int read_scalars(double* out);
  int capture_graph();
  int set_graph_dt0(double dt0);  // mixed path: rewrite dt0 in the instantiated graphs
  int steps_n(int n, double dt0);  // n steps (K-step graphs where they fit)
  int step(double dt0);
  // one un-captured step; ev as for mixed_step (six events, five slots on
  // both paths)
  cudaError_t launch_step(cudaEvent_t* ev, double dt0, bool per_launch = false);
  int launches_per_step() const { return 5; }  // timing slots (the mixed step launches 4 kernels)
  cudaError_t launch_prepare();
  static int check_cuda(cudaError_t e, const char* what);
};

}  // namespace splash
