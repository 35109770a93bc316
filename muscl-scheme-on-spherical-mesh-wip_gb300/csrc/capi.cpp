// C ABI of the GB300 MUSCL step (include/splash_gb300.h).
//
// Host side of the drop-in: it reproduces the reference constructor chain
// (Riemann_solvers/*.hpp ctor -> physics/adiabatic.hpp:18-91 ->
// MUSCL_base/MUSCL_base.hpp:20-95 -> geometry/MUSCL_geometry.hpp:43-225),
// renumbers faces along a Hilbert curve, uploads the slot-plane geometry
// once, captures one do_step as a CUDA graph, and implements the accessors
// and writers of the reference class API on top of device state.
#include "splash_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "diagnostics.hpp"
#include "fp_convert.cuh"
#include "geometry.hpp"
#include "hilbert.hpp"
#include "kernels.hpp"
#include "layout.hpp"
#include "mesh.hpp"
#include "slot_planes.hpp"
#include "solver.hpp"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define SPLASH_CUDA(call)                                                                   \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(SPLASH_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                  __FILE__, __LINE__);                                                      \
  } while (0)

}  // namespace

namespace splash {
int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
}  // namespace splash

struct splash_geometry {
  splash::RefGeometry g;
};

namespace splash {

int Solver::check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) return fail(SPLASH_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return SPLASH_OK;
}

Solver::~Solver() {
  if (device >= 0) cudaSetDevice(device);
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  if (graph_k_exec) cudaGraphExecDestroy(graph_k_exec);
  if (graph_k) cudaGraphDestroy(graph_k);
  for (void* p : dev_allocs) cudaFree(p);
  if (h_stage) cudaFreeHost(h_stage);
  if (h_diag) cudaFreeHost(h_diag);
  if (stream) cudaStreamDestroy(stream);
}

template <typename T>
T* Solver::dalloc(size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(T) > 0 ? n * sizeof(T) : 16) != cudaSuccess) throw std::bad_alloc();
  dev_allocs.push_back(p);
  return static_cast<T*>(p);
}

template <typename T>
T* Solver::upload(const std::vector<T>& h) {
  T* d = dalloc<T>(h.size());
  if (!h.empty() && cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    throw std::runtime_error("cudaMemcpy upload failed");
  return d;
}

}  // namespace splash

namespace {

using splash::RefGeometry;
using splash::Solver;

// Mesh from a descriptor: generated with the reference numbering, or given.
splash::MeshArrays mesh_from_desc(const splash_mesh_desc* d) {
  if (d->vertices == nullptr) {
    return splash::mesh_arrays(splash::build_mesh(d->kind, d->level));
  }
  if (d->n_vertices <= 0 || d->n_faces <= 0 || !d->face_offsets || !d->face_vertices)
    throw std::runtime_error("incomplete mesh arrays");
  splash::MeshArrays a;
  a.vertices.assign(d->vertices, d->vertices + 3 * (size_t)d->n_vertices);
  a.face_off.assign(d->face_offsets, d->face_offsets + d->n_faces + 1);
  if (a.face_off[0] != 0 || a.face_off[d->n_faces] <= 0) throw std::runtime_error("bad face offsets");
  a.face_vtx.assign(d->face_vertices, d->face_vertices + a.face_off[d->n_faces]);
  return a;
}

struct V3 {
  double x, y, z;
};
inline V3 vadd(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 vdiv(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double vnorm(V3 a) {
  double s = 0.0;
  s += a.x * a.x;
  s += a.y * a.y;
  s += a.z * a.z;
  return std::sqrt(s);
}
inline V3 vcross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 at3(const std::vector<double>& v, size_t i) { return {v[3 * i], v[3 * i + 1], v[3 * i + 2]}; }

// std::max / std::min semantics
inline double smax(double a, double b) { return (a < b) ? b : a; }

}  // namespace

namespace splash {

// Uploads the slot planes of one mesh for the solver's precision.
void Solver::build_device_geometry(const RefGeometry& g) {
  const SlotPlanes sp = make_slot_planes(g);
  n_faces = sp.n_faces;
  max_slots = sp.max_slots;
  fpad = sp.fpad;
  perm = sp.perm;
  iperm = sp.iperm;
  const std::vector<double> acc = accretion_source(sp, par, area_coeff, accretion_on);
  if (precision == SPLASH_PREC_MIXED) {
    const MixedPlanes mp = make_mixed_planes(sp);
    GM.n_faces = n_faces;
    GM.fpad = fpad;
    GM.max_slots = max_slots;
    GM.nslots = upload(sp.nslots);
    GM.fcn = upload(sp.fcn);
    GM.fcn32 = upload(mp.fcn32);
    GM.fcn_lo = upload(mp.fcn_lo);
    GM.area = upload(sp.area);
    GM.acc_src = upload(acc);
    GM.coef = upload(mp.coef);
    GM.slot_edge = upload(mp.slot_edge);
    h_slot_edge = mp.slot_edge;
    GM.n_edges = mp.n_edges;
    GM.epad = mp.epad;
    GM.e_ids = upload(mp.e_ids);
    GM.e_ec = upload(mp.e_ec);
    GM.e_en = upload(mp.e_en);
    GM.e_sten = upload(mp.e_sten);
    GM.e_beta = upload(mp.e_beta);
    GM.e_h = upload(mp.e_h);
    geometry_bytes = sp.nslots.size() + 8 * (sp.fcn.size() + sp.area.size() + acc.size()) +
                     4 * (mp.fcn32.size() + mp.fcn_lo.size() + mp.coef.size() + mp.slot_edge.size() + mp.e_ids.size() +
                          mp.e_ec.size() + mp.e_en.size() + mp.e_sten.size() +
                          mp.e_beta.size() + mp.e_h.size());
  } else {
    G.n_faces = n_faces;
    G.fpad = fpad;
    G.max_slots = max_slots;
    G.nslots = upload(sp.nslots);
    G.fcn = upload(sp.fcn);
    G.area = upload(sp.area);
    G.acc_src = upload(acc);
    G.sten = upload(sp.sten);
    G.beta = upload(sp.beta);
    G.hpm = upload(sp.hpm);
    G.bm = upload(sp.bm);
    G.eta = upload(sp.eta);
    G.arc_a = upload(sp.arc);
    G.ec = upload(sp.ec);
    G.ecn = upload(sp.ecn);
    G.en = upload(sp.en);
    G.nxr = upload(sp.nxr);
    G.chord = upload(sp.chord);
    G.rev = upload(sp.rev);
    geometry_bytes = sp.nslots.size() + 8 * (sp.fcn.size() + sp.area.size() + acc.size()) +
                     4 * (sp.sten.size() + sp.rev.size()) +
                     8 * (sp.beta.size() + sp.hpm.size() + sp.bm.size() + sp.eta.size() +
                          sp.arc.size() + sp.ec.size() + sp.ecn.size() + sp.en.size() +
                          sp.nxr.size() + sp.chord.size());
  }
  // keep what the writers need, in reference order
  wr_vertices = g.vertices;
  wr_face_off = g.face_off;
  wr_face_vtx = g.face_vtx;
  wr_face_centers = g.face_centers;
  wr_area = g.area;
}

// The light curves' observer geometry (physics/adiabatic.hpp:233-245,
// 258-322): per observer and face, cos(alpha) = |o . fcn| / |o| where the
// observer sees the face, 0 elsewhere; internal face order.
static std::vector<double> observer_planes(const Solver& s) {
  const double D = 9.4 * 3 * 1e19 / 15000;
  const V3 obs[4] = {{D, 0, 0},
                     {std::sqrt(9.4 * 3 * 1e19 / 15000), 0, std::sqrt(9.4 * 3 * 1e19 / 15000)},
                     {0, 0, D},
                     {0, 0, -9.4 * 3 * 1e19 / 15000}};
  std::vector<double> c(4 * (size_t)s.fpad, 0.0);
  for (int r = 0; r < s.n_faces; ++r) {
    const int i = s.iperm[r];
    const V3 fc = at3(s.wr_face_centers, r);
    const double phi_fc = std::atan2(fc.y / vnorm(fc), fc.x / vnorm(fc));
    const double theta_fc = std::acos(fc.z / vnorm(fc));
    const V3 fcn = vdiv(fc, vnorm(fc));
    const bool seen[4] = {phi_fc < M_PI / 2 && phi_fc > -M_PI / 2, vdot(obs[1], fcn) > 0, theta_fc < M_PI / 2,
                          theta_fc > M_PI / 2};
    for (int o = 0; o < 4; ++o)
      if (seen[o]) c[(size_t)o * s.fpad + i] = std::abs(vdot(obs[o], fcn)) / vnorm(obs[o]);
  }
  return c;
}

int Solver::run_diagnostics(double* out9) {
  DiagInput in{};
  in.n_faces = n_faces;
  in.fpad = fpad;
  in.dim = dim;
  in.U = S.U;
  in.fcn = (precision == SPLASH_PREC_MIXED) ? GM.fcn : G.fcn;
  in.area = (precision == SPLASH_PREC_MIXED) ? GM.area : G.area;
  in.cos_obs = d_cos_obs;
  in.gam = P.gam;
  in.light_curves = dim == kDim ? 1 : 0;
  SPLASH_CUDA(diag_launch(in, d_diag_partial, d_diag_out, stream));
  SPLASH_CUDA(cudaMemcpyAsync(h_diag, d_diag_out, 9 * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SPLASH_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(out9, h_diag, 9 * sizeof(double));
  return SPLASH_OK;
}

// FP64 path: W and the dt partial records of the current U (the mixed path
// computes its face states and dt keys in the set_state pass)
cudaError_t Solver::launch_prepare() { return fp64_prepare(G, S, P, stream); }

cudaError_t Solver::launch_step(cudaEvent_t* ev, double dt0, bool per_launch) {
  if (precision == SPLASH_PREC_MIXED) return mixed_step(GM, S, P, dt0, stream, ev, per_launch);
  cudaError_t e = fp64_set_dt0(S, dt0, stream);
  if (e != cudaSuccess) return e;
  return fp64_step(G, S, P, stream, ev);
}

int Solver::upload_state(const double* U_ref) {
  const double* src = U_ref;  // with host_direct the kernels read the caller's array over the coherent link
  if (!host_direct) {
    std::memcpy(h_stage, U_ref, (size_t)n_faces * dim * sizeof(double));
    SPLASH_CUDA(cudaMemcpyAsync(d_stage, h_stage, (size_t)n_faces * dim * sizeof(double),
                                cudaMemcpyHostToDevice, stream));
    src = d_stage;
  }
  if (precision == SPLASH_PREC_MIXED) {
    SPLASH_CUDA(mixed_scatter_prepare(src, d_iperm, GM, S, P, dim, stream));
    return SPLASH_OK;
  }
  SPLASH_CUDA(fp64_scatter_state(src, d_iperm, S.U, n_faces, fpad, stream, dim));
  SPLASH_CUDA(launch_prepare());
  return SPLASH_OK;
}

int Solver::download_state(double* U_ref) {
  if (host_direct) {
    SPLASH_CUDA(fp64_gather_state(S.U, d_iperm, U_ref, n_faces, fpad, stream, dim));
    SPLASH_CUDA(cudaStreamSynchronize(stream));
    return SPLASH_OK;
  }
  SPLASH_CUDA(fp64_gather_state(S.U, d_iperm, d_stage, n_faces, fpad, stream, dim));
  SPLASH_CUDA(cudaMemcpyAsync(h_stage, d_stage, (size_t)n_faces * dim * sizeof(double),
                              cudaMemcpyDeviceToHost, stream));
  SPLASH_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(U_ref, h_stage, (size_t)n_faces * dim * sizeof(double));
  return SPLASH_OK;
}

int Solver::read_scalars(double* out) {
  SPLASH_CUDA(cudaMemcpyAsync(out, S.scal, kScCount * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SPLASH_CUDA(cudaStreamSynchronize(stream));
  return SPLASH_OK;
}

int Solver::capture_graph() {
  SPLASH_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  // FP64: the graph holds the five step launches, dt0 is set by a launch
  // before each replay; mixed: the graph holds the whole step, dt0 being an
  // argument of its first node
  cudaError_t le = (precision == SPLASH_PREC_MIXED) ? mixed_step(GM, S, P, graph_dt0, stream, nullptr)
                                                     : fp64_step(G, S, P, stream, nullptr);
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(stream, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(SPLASH_E_CUDA, "step launch during capture: %s", cudaGetErrorString(le));
  }
  SPLASH_CUDA(ce);
  graph = g;
  SPLASH_CUDA(cudaGraphInstantiate(&graph_exec, graph, 0));
  if (precision == SPLASH_PREC_MIXED) {
    size_t n = 0;
    SPLASH_CUDA(cudaGraphGetNodes(graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    SPLASH_CUDA(cudaGraphGetNodes(graph, nodes.data(), &n));
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType t;
      SPLASH_CUDA(cudaGraphNodeGetType(nd, &t));
      if (t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      SPLASH_CUDA(cudaGraphKernelNodeGetParams(nd, &kp));
      if (kp.func == mixed_dt0_kernel_ptr()) dt0_node = nd;
    }
    if (!dt0_node) return fail(SPLASH_E_CUDA, "dt node not found in the captured step");
    // the same step kGraphSteps times in one graph
    SPLASH_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t lk = cudaSuccess;
    for (int k = 0; k < kGraphSteps && lk == cudaSuccess; ++k)
      lk = mixed_step(GM, S, P, graph_dt0, stream, nullptr);
    cudaGraph_t gk = nullptr;
    cudaError_t ck = cudaStreamEndCapture(stream, &gk);
    if (lk != cudaSuccess) {
      if (gk) cudaGraphDestroy(gk);
      return fail(SPLASH_E_CUDA, "step launch during capture: %s", cudaGetErrorString(lk));
    }
    SPLASH_CUDA(ck);
    graph_k = gk;
    SPLASH_CUDA(cudaGraphInstantiate(&graph_k_exec, graph_k, 0));
    SPLASH_CUDA(cudaGraphGetNodes(graph_k, nullptr, &n));
    nodes.resize(n);
    SPLASH_CUDA(cudaGraphGetNodes(graph_k, nodes.data(), &n));
    dt0_nodes_k.clear();
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType t;
      SPLASH_CUDA(cudaGraphNodeGetType(nd, &t));
      if (t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      SPLASH_CUDA(cudaGraphKernelNodeGetParams(nd, &kp));
      if (kp.func == mixed_dt0_kernel_ptr()) dt0_nodes_k.push_back(nd);
    }
    if ((int)dt0_nodes_k.size() != kGraphSteps)
      return fail(SPLASH_E_CUDA, "dt nodes not found in the captured steps");
  }
  return SPLASH_OK;
}

int Solver::set_graph_dt0(double dt0) {
  if (dt0 == graph_dt0) return SPLASH_OK;
  // new dt0: rewrite the stage-1 edge nodes' arguments in the instantiated
  // graphs (takes effect from the next launch; launches in flight keep theirs)
  cudaKernelNodeParams kp{};
  SPLASH_CUDA(cudaGraphKernelNodeGetParams(dt0_node, &kp));
  float dt0f = splash::fpc::d2f(dt0);
  void* args[] = {&GM, &S, &P, &dt0, &dt0f};
  kp.kernelParams = args;
  kp.extra = nullptr;
  SPLASH_CUDA(cudaGraphExecKernelNodeSetParams(graph_exec, dt0_node, &kp));
  for (cudaGraphNode_t nd : dt0_nodes_k) SPLASH_CUDA(cudaGraphExecKernelNodeSetParams(graph_k_exec, nd, &kp));
  graph_dt0 = dt0;
  return SPLASH_OK;
}

int Solver::step(double dt0) {
  if (precision == SPLASH_PREC_MIXED) {
    const int rc = set_graph_dt0(dt0);
    if (rc) return rc;
  } else {
    SPLASH_CUDA(fp64_set_dt0(S, dt0, stream));
  }
  SPLASH_CUDA(cudaGraphLaunch(graph_exec, stream));
  ++steps;
  return SPLASH_OK;
}

int Solver::steps_n(int n, double dt0) {
  if (precision != SPLASH_PREC_MIXED || !graph_k_exec) {
    for (int i = 0; i < n; ++i) {
      const int rc = step(dt0);
      if (rc) return rc;
    }
    return SPLASH_OK;
  }
  const int rc = set_graph_dt0(dt0);
  if (rc) return rc;
  int left = n;
  for (; left >= kGraphSteps; left -= kGraphSteps) {
    SPLASH_CUDA(cudaGraphLaunch(graph_k_exec, stream));
    steps += kGraphSteps;
  }
  for (; left > 0; --left) {
    SPLASH_CUDA(cudaGraphLaunch(graph_exec, stream));
    ++steps;
  }
  return SPLASH_OK;
}

}  // namespace splash

// ============================ C ABI ======================================
extern "C" {

const char* splash_last_error(void) { return g_last_error.c_str(); }
const char* splash_version(void) { return "splash_gb300 1.0 (sm_103a)"; }

int splash_create(const splash_mesh_desc* mesh, const double* U_in, int dim, double gam,
                  double omega_ns, int accretion_on, const splash_params* params, int solver_kind,
                  int precision, int device, int threads, splash_solver** out) {
  if (!out) return fail(SPLASH_E_INVALID, "out is NULL");
  *out = nullptr;
  if (!mesh || !U_in || !params) return fail(SPLASH_E_INVALID, "mesh, U_in and params must be non-NULL");
  if (solver_kind < SPLASH_SOLVER_HLLE_P || solver_kind > SPLASH_SOLVER_HLLE)
    return fail(SPLASH_E_INVALID, "unknown solver kind %d", solver_kind);
  if (solver_kind == SPLASH_SOLVER_HLLE && dim != 4)
    return fail(SPLASH_E_UNSUPPORTED,
                "dim=%d: the isothermal solver needs dim=4 (the reference prints \"check dim\" and "
                "latches stop_check, physics/isothermal.hpp:18-22)",
                dim);
  if (solver_kind != SPLASH_SOLVER_HLLE && dim != splash::kDim)
    return fail(SPLASH_E_UNSUPPORTED,
                "dim=%d: the adiabatic solvers need dim=5 (the reference latches stop_check and "
                "then indexes out of bounds, physics/adiabatic.hpp:26-30)",
                dim);
  if (precision != SPLASH_PREC_FP64 && precision != SPLASH_PREC_MIXED)
    return fail(SPLASH_E_INVALID, "unknown precision %d", precision);
  if (precision == SPLASH_PREC_MIXED && !splash::mixed_available())
    return fail(SPLASH_E_UNSUPPORTED, "mixed precision path not built");
  if (!(gam > 1.0 && gam < 2.0)) return fail(SPLASH_E_INVALID, "gam=%g must lie in (1, 2)", gam);

  std::unique_ptr<Solver> s(new (std::nothrow) Solver());
  if (!s) return fail(SPLASH_E_NOMEM, "host allocation failed");
  try {
    splash::MeshArrays arrays = mesh_from_desc(mesh);
    RefGeometry g = splash::build_ref_geometry(arrays, threads);
    s->par = *params;
    s->dim = dim;
    // the isothermal solver has no source term (physics/isothermal.hpp:199-208)
    s->accretion_on = accretion_on != 0 && solver_kind != SPLASH_SOLVER_HLLE;
    s->precision = precision;
    s->solver_kind = solver_kind;
    s->device = device;
    // adiabatic ctor: area_coeff and total_mass (physics/adiabatic.hpp:70-90)
    s->area_coeff = splash::area_coefficient(g, params->acc_width);
    {
      double tm = 0;
      for (int n = 0; n < g.n_faces; ++n) tm += U_in[(size_t)n * dim] * g.area[n];
      s->total_mass = tm;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      return fail(SPLASH_E_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(SPLASH_E_INVALID, "device %d out of range", device);
    SPLASH_CUDA(cudaSetDevice(device));
    SPLASH_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));

    if (precision == SPLASH_PREC_MIXED && g.max_slots > 8)
      return fail(SPLASH_E_UNSUPPORTED, "the mixed path handles faces of up to 8 edges (mesh has %d)",
                  g.max_slots);
    s->build_device_geometry(g);
    splash::PhysParams& P = s->P;
    P.gam = gam;
    P.omega_ns = omega_ns;
    P.e_acc = params->e_acc;
    P.omega_acc_x = 0;
    P.omega_acc_y = std::sin(params->tilt_angle) * params->omega_acc_abs;
    P.omega_acc_z = std::cos(params->tilt_angle) * params->omega_acc_abs;
    P.alpha = params->alpha;
    P.acc_rate = params->accretion_rate;
    P.total_mass = s->total_mass;
    P.h0 = g.h0;
    P.round_diff = g.round_diff;
    P.accretion_on = s->accretion_on ? 1 : 0;
    P.friction_on = params->friction_on ? 1 : 0;
    P.solver = solver_kind;
    splash::derive_params(P);

    const size_t fp = (size_t)s->fpad;
    const size_t PS = (size_t)s->max_slots * fp;
    splash::DevState& S = s->S;
    S.U = s->dalloc<double>(splash::kDim * fp);
    if (precision == SPLASH_PREC_MIXED) {
      S.W32 = s->dalloc<float>(splash::kDim * fp);
      S.W32b = s->dalloc<float>(splash::kDim * fp);
      S.uplus32 = s->dalloc<float>(splash::kDim * 2 * (size_t)s->GM.epad);
      S.fe32 = s->dalloc<float>(splash::kDim * (size_t)s->GM.epad);
      S.uplus = nullptr;
      SPLASH_CUDA(cudaMemset(S.W32, 0, splash::kDim * fp * sizeof(float)));
      SPLASH_CUDA(cudaMemset(S.W32b, 0, splash::kDim * fp * sizeof(float)));
      SPLASH_CUDA(cudaMemset(S.uplus32, 0, splash::kDim * 2 * (size_t)s->GM.epad * sizeof(float)));
      s->n_partials = 0;  // the mixed path reduces the dt candidates as keys
    } else {
      S.W0 = s->dalloc<double>(splash::kDim * fp);
      S.W1 = s->dalloc<double>(splash::kDim * fp);
      SPLASH_CUDA(cudaMemset(S.W0, 0, splash::kDim * fp * sizeof(double)));
      SPLASH_CUDA(cudaMemset(S.W1, 0, splash::kDim * fp * sizeof(double)));
      S.uplus = s->dalloc<double>(splash::kDim * PS);
      SPLASH_CUDA(cudaMemset(S.uplus, 0, splash::kDim * PS * sizeof(double)));
      s->n_partials = splash::fp64_partial_blocks(s->n_faces);
      S.partial = s->dalloc<double>((size_t)s->n_partials * splash::kPartialStride);
    }
    S.scal = s->dalloc<double>(splash::kScCount);
    S.err = s->dalloc<unsigned int>(4);
    S.keys = s->dalloc<unsigned>(2);
    s->d_stage = s->dalloc<double>((size_t)s->n_faces * dim);
    s->d_perm = s->upload(s->perm);
    s->d_iperm = s->upload(s->iperm);
    s->d_cos_obs = s->upload(observer_planes(*s));
    s->d_diag_partial = s->dalloc<double>((size_t)splash::diag_partial_blocks(s->n_faces) * 9);
    s->d_diag_out = s->dalloc<double>(9);
    SPLASH_CUDA(cudaMallocHost(&s->h_diag, 9 * sizeof(double)));
    {
      // Grace-class hosts: the device can dereference pageable host memory,
      // so states cross the boundary without a staging copy
      int pma = 0;
      if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess)
        s->host_direct = pma != 0 && std::getenv("SPLASH_STAGED_TRANSFERS") == nullptr;
    }
    SPLASH_CUDA(cudaMemset(S.U, 0, splash::kDim * fp * sizeof(double)));
    SPLASH_CUDA(cudaMemset(S.scal, 0, splash::kScCount * sizeof(double)));
    SPLASH_CUDA(cudaMemset(S.err, 0, 4 * sizeof(unsigned int)));
    SPLASH_CUDA(cudaMallocHost(&s->h_stage, (size_t)s->n_faces * dim * sizeof(double)));

    int rc = s->upload_state(U_in);
    if (rc) return rc;
    rc = s->capture_graph();
    if (rc) return rc;
    SPLASH_CUDA(cudaStreamSynchronize(s->stream));
  } catch (const std::bad_alloc&) {
    return fail(SPLASH_E_NOMEM, "allocation failed while building the solver");
  } catch (const std::exception& e) {
    return fail(SPLASH_E_MESH, "%s", e.what());
  }
  *out = reinterpret_cast<splash_solver*>(s.release());
  return SPLASH_OK;
}

int splash_destroy(splash_solver* h) {
  delete reinterpret_cast<Solver*>(h);
  return SPLASH_OK;
}

#define GET_SOLVER(h)                                                   \
  Solver* s = reinterpret_cast<Solver*>(h);                             \
  if (!s) return fail(SPLASH_E_INVALID, "solver handle is NULL");      \
  SPLASH_CUDA(cudaSetDevice(s->device))

int splash_do_step(splash_solver* h, double dt0) {
  GET_SOLVER(h);
  return s->step(dt0);
}

int splash_do_steps(splash_solver* h, int n, double dt0) {
  GET_SOLVER(h);
  if (n < 0) return fail(SPLASH_E_INVALID, "n < 0");
  return s->steps_n(n, dt0);
}

int splash_do_steps_host(splash_solver* h, const double* U_in, int n, double dt0, double* U_out) {
  GET_SOLVER(h);
  if (n < 0) return fail(SPLASH_E_INVALID, "n < 0");
  if (U_in) {
    const int rc = s->upload_state(U_in);
    if (rc) return rc;
  }
  const int rc = s->steps_n(n, dt0);
  if (rc) return rc;
  if (U_out) return s->download_state(U_out);  // synchronises the stream
  SPLASH_CUDA(cudaStreamSynchronize(s->stream));  // U_in has been read
  return SPLASH_OK;
}

int splash_stream(splash_solver* h, void** stream) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s || !stream) return fail(SPLASH_E_INVALID, "NULL argument");
  *stream = (void*)s->stream;
  return SPLASH_OK;
}

int splash_kernel_times(splash_solver* h, int reps, double dt0, double ms[5]) {
  GET_SOLVER(h);
  if (reps <= 0 || !ms) return fail(SPLASH_E_INVALID, "reps must be > 0 and ms non-NULL");
  cudaEvent_t ev[6];
  for (auto& e : ev) SPLASH_CUDA(cudaEventCreate(&e));
  double acc[5] = {0, 0, 0, 0, 0};
  int rc = SPLASH_OK;
  for (int r = 0; r < reps && rc == SPLASH_OK; ++r) {
    cudaError_t e = s->launch_step(ev, dt0);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[5]);
    if (e != cudaSuccess) {
      rc = fail(SPLASH_E_CUDA, "kernel timing: %s", cudaGetErrorString(e));
      break;
    }
    for (int k = 0; k < 5; ++k) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      acc[k] += t;
    }
    ++s->steps;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  for (int k = 0; k < 5; ++k) ms[k] = acc[k] / reps;
  return SPLASH_OK;
}

int splash_launch_times(splash_solver* h, int reps, double dt0, double* ms, int cap, int* count) {
  GET_SOLVER(h);
  if (reps <= 0 || !ms || !count || cap < 0) return fail(SPLASH_E_INVALID, "reps must be > 0, ms and count non-NULL");
  const int nl = s->launches_per_step();
  cudaEvent_t ev[8];
  for (int k = 0; k <= nl; ++k) SPLASH_CUDA(cudaEventCreate(&ev[k]));
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  int rc = SPLASH_OK;
  for (int r = 0; r < reps && rc == SPLASH_OK; ++r) {
    cudaError_t e = s->launch_step(ev, dt0, true);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[nl]);
    if (e != cudaSuccess) {
      rc = fail(SPLASH_E_CUDA, "launch timing: %s", cudaGetErrorString(e));
      break;
    }
    for (int k = 0; k < nl; ++k) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      acc[k] += t;
    }
    ++s->steps;
  }
  for (int k = 0; k <= nl; ++k) cudaEventDestroy(ev[k]);
  if (rc) return rc;
  for (int k = 0; k < nl && k < cap; ++k) ms[k] = acc[k] / reps;
  *count = nl;
  return SPLASH_OK;
}

int splash_memory(splash_solver* h, int64_t out[2]) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s || !out) return fail(SPLASH_E_INVALID, "NULL argument");
  const size_t fp = (size_t)s->fpad, PS = (size_t)s->max_slots * fp;
  out[0] = (int64_t)s->geometry_bytes;
  if (s->precision == SPLASH_PREC_MIXED)  // U; W32 and W32b; edge states (2 per edge); edge fluxes
    out[1] = (int64_t)(8 * splash::kDim * fp + 4 * splash::kDim * (2 * fp + 3 * (size_t)s->GM.epad));
  else
    out[1] = (int64_t)(8 * (3 * splash::kDim * fp + splash::kDim * PS) +
                       8 * (size_t)s->n_partials * splash::kPartialStride);
  return SPLASH_OK;
}

int splash_synchronize(splash_solver* h) {
  GET_SOLVER(h);
  SPLASH_CUDA(cudaStreamSynchronize(s->stream));
  return SPLASH_OK;
}

int splash_time(splash_solver* h, double* t) {
  GET_SOLVER(h);
  if (!t) return fail(SPLASH_E_INVALID, "t is NULL");
  double sc[splash::kScCount];
  const int rc = s->read_scalars(sc);
  if (rc) return rc;
  *t = sc[splash::kScTime];
  return SPLASH_OK;
}

int splash_last_dt(splash_solver* h, double* dt) {
  GET_SOLVER(h);
  if (!dt) return fail(SPLASH_E_INVALID, "dt is NULL");
  double sc[splash::kScCount];
  const int rc = s->read_scalars(sc);
  if (rc) return rc;
  *dt = sc[splash::kScDt];
  return SPLASH_OK;
}

int splash_error_word(splash_solver* h, uint32_t* bits) {
  GET_SOLVER(h);
  if (!bits) return fail(SPLASH_E_INVALID, "bits is NULL");
  unsigned int e = 0;
  SPLASH_CUDA(cudaMemcpyAsync(&e, s->S.err, sizeof e, cudaMemcpyDeviceToHost, s->stream));
  SPLASH_CUDA(cudaStreamSynchronize(s->stream));
  *bits = e;
  return SPLASH_OK;
}

int splash_stop_check(splash_solver* h, int* stop) {
  if (!stop) return fail(SPLASH_E_INVALID, "stop is NULL");
  uint32_t bits = 0;
  const int rc = splash_error_word(h, &bits);
  if (rc) return rc;
  *stop = bits != 0;
  return SPLASH_OK;
}

int splash_steps(splash_solver* h, int64_t* steps) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s || !steps) return fail(SPLASH_E_INVALID, "NULL argument");
  *steps = s->steps;
  return SPLASH_OK;
}

int splash_n_faces(splash_solver* h, int* n) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s || !n) return fail(SPLASH_E_INVALID, "NULL argument");
  *n = s->n_faces;
  return SPLASH_OK;
}

int splash_dim(splash_solver* h, int* d) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s || !d) return fail(SPLASH_E_INVALID, "NULL argument");
  *d = s->dim;
  return SPLASH_OK;
}

int splash_get_state(splash_solver* h, double* U) {
  GET_SOLVER(h);
  if (!U) return fail(SPLASH_E_INVALID, "U is NULL");
  return s->download_state(U);
}

int splash_set_state(splash_solver* h, const double* U) {
  GET_SOLVER(h);
  if (!U) return fail(SPLASH_E_INVALID, "U is NULL");
  const int rc = s->upload_state(U);
  if (rc) return rc;
  SPLASH_CUDA(cudaStreamSynchronize(s->stream));
  return SPLASH_OK;
}

int splash_diagnostics(splash_solver* h, double out[5]) {
  GET_SOLVER(h);
  if (!out) return fail(SPLASH_E_INVALID, "out is NULL");
  double v[9];
  const int rc = s->run_diagnostics(v);
  if (rc) return rc;
  for (int k = 0; k < 5; ++k) out[k] = v[k];
  return SPLASH_OK;
}

int splash_get_permutation(splash_solver* h, int* internal_to_ref) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s || !internal_to_ref) return fail(SPLASH_E_INVALID, "NULL argument");
  std::copy(s->perm.begin(), s->perm.end(), internal_to_ref);
  return SPLASH_OK;
}

int splash_face_geometry(splash_solver* h, double* unit_centres, double* area) {
  Solver* s = reinterpret_cast<Solver*>(h);
  if (!s) return fail(SPLASH_E_INVALID, "solver handle is NULL");
  for (int i = 0; i < s->n_faces; ++i) {
    if (unit_centres) {
      const V3 fc = at3(s->wr_face_centers, i);
      const V3 u = vdiv(fc, vnorm(fc));
      unit_centres[3 * (size_t)i] = u.x;
      unit_centres[3 * (size_t)i + 1] = u.y;
      unit_centres[3 * (size_t)i + 2] = u.z;
    }
    if (area) area[i] = s->wr_area[i];
  }
  return SPLASH_OK;
}

// ---------------- writers (physics/adiabatic.hpp:101-348) ----------------
static int open_append(std::ofstream& os, const char* path) {
  if (!path) return fail(SPLASH_E_INVALID, "path is NULL");
  os.open(path, std::ios::out | std::ios::app);
  if (!os) return fail(SPLASH_E_INVALID, "cannot open %s", path);
  return SPLASH_OK;
}

int splash_write_t_rho(splash_solver* h, const char* path) {
  GET_SOLVER(h);
  std::ofstream os;
  int rc = open_append(os, path);
  if (rc) return rc;
  std::vector<double> U((size_t)s->n_faces * s->dim);
  if ((rc = s->download_state(U.data()))) return rc;
  double t;
  if ((rc = splash_time(h, &t))) return rc;
  os << t << "  ";
  for (int i = 0; i < s->n_faces; ++i) os << U[(size_t)i * s->dim] << " ";
  os << "\n";
  return SPLASH_OK;
}

int splash_write_t_p(splash_solver* h, const char* path) {
  GET_SOLVER(h);
  std::ofstream os;
  int rc = open_append(os, path);
  if (rc) return rc;
  std::vector<double> U((size_t)s->n_faces * s->dim);
  if ((rc = s->download_state(U.data()))) return rc;
  double t;
  if ((rc = splash_time(h, &t))) return rc;
  os << t << "  ";
  for (int i = 0; i < s->n_faces; ++i) {
    const double* u = &U[(size_t)i * s->dim];
    if (s->dim == 4) {  // physics/isothermal.hpp:63-73: a * a * Sigma, a = 1
      os << 1.0 * 1.0 * u[0] << " ";
      continue;
    }
    const V3 fc = at3(s->wr_face_centers, i);
    V3 vel = vcross(vdiv(fc, vnorm(fc)), V3{u[1], u[2], u[3]});
    vel = vdiv(vel, -u[0]);
    const double n = vnorm(vel);
    os << smax(1e-16, (u[4] - u[0] * (n * n) / 2) * (s->P.gam - 1)) << " ";
  }
  os << "\n";
  return SPLASH_OK;
}

int splash_write_t_curl(splash_solver* h, const char* path) {
  GET_SOLVER(h);
  std::ofstream os;
  int rc = open_append(os, path);
  if (rc) return rc;
  std::vector<double> U((size_t)s->n_faces * s->dim);
  if ((rc = s->download_state(U.data()))) return rc;
  // U_plus of the last stage, slot planes -> host
  const size_t PS = (size_t)s->max_slots * s->fpad;
  std::vector<double> up(splash::kDim * PS);
  if (s->S.uplus) {
    SPLASH_CUDA(cudaMemcpy(up.data(), s->S.uplus, up.size() * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    // packed FP32 edge states of the last stage, edge-major (owner side of
    // edge e at e, reverse side at epad + e): [2 epad][4] (Sigma, l), then Pi,
    // recomputed from the last stage-2 input (zeros before the first step,
    // like the reference's freshly allocated U_plus)
    const size_t ne = 2 * (size_t)s->GM.epad;
    std::vector<float> up32(splash::kDim * ne);
    if (s->steps > 0) SPLASH_CUDA(splash::mixed_edge_states(s->GM, s->S, s->P, s->stream));
    SPLASH_CUDA(cudaStreamSynchronize(s->stream));
    SPLASH_CUDA(cudaMemcpy(up32.data(), s->S.uplus32, up32.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int i = 0; i < s->n_faces; ++i) {
      const int n = s->wr_face_off[s->perm[i] + 1] - s->wr_face_off[s->perm[i]];
      for (int j = 0; j < n; ++j) {
        const size_t q = (size_t)j * s->fpad + i;
        const unsigned se = (unsigned)s->h_slot_edge[q];
        const size_t x = (se & 0x7fffffffu) + ((se >> 31) ? (size_t)s->GM.epad : 0);
        for (int k = 0; k < 4; ++k) up[k * PS + q] = up32[4 * x + k];
        up[4 * PS + q] = up32[4 * ne + x];
      }
    }
  }
  double t;
  if ((rc = splash_time(h, &t))) return rc;
  os << t << "  ";
  for (int r = 0; r < s->n_faces; ++r) {
    const int i = s->iperm[r];
    const int n = s->wr_face_off[r + 1] - s->wr_face_off[r];
    double vort = 0;
    for (int j = 0; j < n; ++j) {
      const size_t sl = (size_t)j * s->fpad + i;
      const V3 l{up[PS + sl], up[2 * PS + sl], up[3 * PS + sl]};
      const int va = s->wr_face_vtx[s->wr_face_off[r] + j];
      const int vb = s->wr_face_vtx[s->wr_face_off[r] + ((j + 1 == n) ? 0 : j + 1)];
      V3 ec = vdiv(vadd(at3(s->wr_vertices, va), at3(s->wr_vertices, vb)), 2.);
      ec = vdiv(ec, vnorm(ec));
      V3 vel = vcross(ec, l);
      vel = vdiv(vel, -U[(size_t)r * s->dim]);
      const V3 rr = vsub(at3(s->wr_vertices, va), at3(s->wr_vertices, vb));
      vort += vdot(vel, rr);
    }
    os << vort / s->wr_area[r] << " ";
  }
  os << "\n";
  return SPLASH_OK;
}

int splash_write_t_L(splash_solver* h, const char* px, const char* py, const char* pz) {
  GET_SOLVER(h);
  if (s->dim == 4) return fail(SPLASH_E_UNSUPPORTED, "the isothermal solver has no such member (physics/isothermal.hpp)");
  std::vector<double> U((size_t)s->n_faces * s->dim);
  int rc;
  if ((rc = s->download_state(U.data()))) return rc;
  double t;
  if ((rc = splash_time(h, &t))) return rc;
  const char* paths[3] = {px, py, pz};
  for (int k = 0; k < 3; ++k) {
    std::ofstream os;
    if ((rc = open_append(os, paths[k]))) return rc;
    os << t << "  ";
    for (int i = 0; i < s->n_faces; ++i) os << U[(size_t)i * s->dim + k + 1] << " ";
    os << "\n";
  }
  return SPLASH_OK;
}

int splash_write_t_omega_z(splash_solver* h, const char* path) {
  GET_SOLVER(h);
  std::ofstream os;
  int rc = open_append(os, path);
  if (rc) return rc;
  std::vector<double> U((size_t)s->n_faces * s->dim);
  if ((rc = s->download_state(U.data()))) return rc;
  double t;
  if ((rc = splash_time(h, &t))) return rc;
  os << t << "  ";
  for (int i = 0; i < s->n_faces; ++i) {
    const double* u = &U[(size_t)i * s->dim];
    const V3 fc = at3(s->wr_face_centers, i);
    const double theta = std::acos(fc.z / vnorm(fc));
    const V3 fcn = vdiv(fc, vnorm(fc));
    V3 vel = vcross(fcn, V3{u[1], u[2], u[3]});
    vel = vdiv(vel, -u[0]);
    if (s->dim == 4) {  // physics/isothermal.hpp:112-133: z of (face centre x v)
      os << vcross(fc, vel).z << " ";
      continue;
    }
    const V3 rxv = vcross(fcn, vel);
    double om_z = rxv.z / (std::sin(theta) * std::sin(theta));
    if (std::isnan(om_z) || std::isinf(om_z) || std::abs(om_z) > 1e4) om_z = 0;
    os << om_z << " ";
  }
  os << "\n";
  return SPLASH_OK;
}

int splash_get_light_curves(splash_solver* h, double out[4]) {
  GET_SOLVER(h);
  if (s->dim == 4) return fail(SPLASH_E_UNSUPPORTED, "the isothermal solver has no such member (physics/isothermal.hpp)");
  if (!out) return fail(SPLASH_E_INVALID, "out is NULL");
  double v[9];
  const int rc = s->run_diagnostics(v);
  if (rc) return rc;
  for (int k = 0; k < 4; ++k) out[k] = v[5 + k];
  return SPLASH_OK;
}

int splash_write_final_state(splash_solver* h, const char* path) {
  GET_SOLVER(h);
  if (s->dim == 4) return fail(SPLASH_E_UNSUPPORTED, "the isothermal solver has no such member (physics/isothermal.hpp)");
  if (!path) return fail(SPLASH_E_INVALID, "path is NULL");
  std::vector<double> U((size_t)s->n_faces * s->dim);
  int rc;
  if ((rc = s->download_state(U.data()))) return rc;
  std::ofstream os(path, std::ios::out | std::ios::trunc);
  if (!os) return fail(SPLASH_E_INVALID, "cannot open %s", path);
  for (int i = 0; i < s->n_faces; ++i) {
    for (int k = 0; k < s->dim; ++k) os << U[(size_t)i * s->dim + k] << " ";
    os << "\n";
  }
  return SPLASH_OK;
}

// ---------------- geometry export ----------------
int splash_geometry_build(const splash_mesh_desc* mesh, int threads, splash_geometry** out) {
  if (!mesh || !out) return fail(SPLASH_E_INVALID, "NULL argument");
  *out = nullptr;
  try {
    std::unique_ptr<splash_geometry> g(new splash_geometry());
    g->g = splash::build_ref_geometry(mesh_from_desc(mesh), threads);
    *out = g.release();
  } catch (const std::bad_alloc&) {
    return fail(SPLASH_E_NOMEM, "allocation failed");
  } catch (const std::exception& e) {
    return fail(SPLASH_E_MESH, "%s", e.what());
  }
  return SPLASH_OK;
}

int splash_geometry_free(splash_geometry* g) {
  delete g;
  return SPLASH_OK;
}

int splash_geometry_info(const splash_geometry* gh, int64_t sizes[4], double scalars[2]) {
  if (!gh || !sizes || !scalars) return fail(SPLASH_E_INVALID, "NULL argument");
  const RefGeometry& g = gh->g;
  sizes[0] = g.n_vertices;
  sizes[1] = g.n_faces;
  sizes[2] = g.n_slots;
  sizes[3] = g.max_slots;
  scalars[0] = g.h0;
  scalars[1] = g.round_diff;
  return SPLASH_OK;
}

int splash_geometry_get(const splash_geometry* gh, const char* name, void* dst, size_t bytes,
                        size_t* written) {
  if (!gh || !name) return fail(SPLASH_E_INVALID, "NULL argument");
  const RefGeometry& g = gh->g;
  const void* src = nullptr;
  size_t n = 0;
  auto pick_d = [&](const std::vector<double>& v) { src = v.data(); n = v.size() * sizeof(double); };
  auto pick_i = [&](const std::vector<int>& v) { src = v.data(); n = v.size() * sizeof(int); };
  const std::string k(name);
  if (k == "vertices") pick_d(g.vertices);
  else if (k == "face_off") pick_i(g.face_off);
  else if (k == "face_vtx") pick_i(g.face_vtx);
  else if (k == "nbr_off") pick_i(g.nbr_off);
  else if (k == "nbr") pick_i(g.nbr);
  else if (k == "nbr_edge") pick_i(g.nbr_edge);
  else if (k == "face_centers") pick_d(g.face_centers);
  else if (k == "normals") pick_d(g.normals);
  else if (k == "area") pick_d(g.area);
  else if (k == "edge_normals") pick_d(g.edge_normals);
  else if (k == "bm_dist") pick_d(g.bm_dist);
  else if (k == "h_plus") pick_d(g.h_plus);
  else if (k == "h_minus") pick_d(g.h_minus);
  else if (k == "ff_plus") pick_i(g.ff_plus);
  else if (k == "ff_minus") pick_i(g.ff_minus);
  else if (k == "beta_plus") pick_d(g.beta_plus);
  else if (k == "beta_minus") pick_d(g.beta_minus);
  else if (k == "unit_face_centers") {
    // fc / |fc| as write_face_centers prints it (MUSCL_geometry.hpp:1076-1077),
    // evaluated here so the caller's compiler flags cannot change the digits
    static thread_local std::vector<double> unit;
    unit.resize(g.face_centers.size());
    for (size_t i = 0; i + 2 < g.face_centers.size(); i += 3) {
      const V3 c = at3(g.face_centers, i / 3);
      const double n = vnorm(c);
      unit[i] = c.x / n;
      unit[i + 1] = c.y / n;
      unit[i + 2] = c.z / n;
    }
    pick_d(unit);
  }
  else if (k == "hilbert_order") {
    // the internal face numbering a solver built on this mesh uses
    static thread_local std::vector<int> order;
    order = splash::hilbert_order(g.face_centers.data(), g.n_faces);
    pick_i(order);
  }
  else return fail(SPLASH_E_INVALID, "unknown geometry array '%s'", name);
  if (written) *written = n;
  if (dst) {
    if (bytes < n) return fail(SPLASH_E_INVALID, "buffer too small for '%s' (%zu < %zu)", name, bytes, n);
    std::memcpy(dst, src, n);
  }
  return SPLASH_OK;
}

}  // extern "C"
