// Ensemble of independent solver instances advanced by shared batched
// launches (the batched workload: many small meshes, each with its own
// parameters and its own CFL dt).
//
// Members on the same mesh level share one copy of the level's slot planes;
// each member owns its state, its accretion source (it depends on its tilt
// and rate) and its scalars.  One do_step of the ensemble is five launches
// over all members, captured once as a CUDA graph: the per-member dt
// finalize, then reconstruction and flux+update twice.  Blocks map to
// (member, face tile) pairs; the order of those tiles and the width of the
// reconstruction tiles form the schedule, chosen at creation by timing every
// candidate on the ensemble itself (state restored afterwards).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

#include "geometry.hpp"
#include "kernels.hpp"
#include "layout.hpp"
#include "mesh.hpp"
#include "slot_planes.hpp"
#include "solver.hpp"
#include "splash_gb300.h"

namespace splash {
namespace {

#define ENS_CUDA(call)                                                                             \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return splash::set_error(SPLASH_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                       __LINE__);                                                                  \
  } while (0)

struct Level {
  int kind = 0, level = 0;
  RefGeometry geom;
  SlotPlanes sp;
  DevGeomMixed G{};  // acc_src filled per member
};

}  // namespace

struct Ensemble {
  int device = 0;
  cudaStream_t stream = nullptr;
  int n = 0;
  int max_slots = 0;
  std::vector<Level> levels;
  std::vector<int> member_level;
  std::vector<size_t> off_face;   // member offset into per-face pools (multiples of fpad)
  std::vector<size_t> off_slot;   // member offset into the per-slot pool
  std::vector<size_t> off_edge;   // member offset into the per-edge pool (multiples of epad)
  std::vector<EnsInstance> inst;
  EnsInstance* d_inst = nullptr;
  double *U = nullptr, *acc = nullptr, *scal = nullptr, *U_snap = nullptr, *scal_snap = nullptr;
  float *W32 = nullptr, *W32b = nullptr, *fe32 = nullptr;
  unsigned int *err = nullptr, *err_snap = nullptr;
  unsigned* keys = nullptr;
  int2 *d_ftiles = nullptr, *d_etiles = nullptr;
  int n_ftiles = 0, n_etiles = 0;
  int order = 0, recon_width = 128;  // tile order; threads per block of the edge launch
  double tuned_ms[12] = {0};         // [order * 3 + width index], then [9 + order] persistent
  // the persistent schedule: one cooperative launch of pgrid blocks per
  // do_steps call (pgrid 0: the device's occupancy could not be read)
  bool persistent = false;
  int pgrid = 0;
  unsigned* d_bar = nullptr;  // [0..1] grid barrier, [2] status (kEnsBarrierTimeout)
  cudaGraphNode_t p_node = nullptr;
  int graph_steps = 1;
  std::vector<void*> allocs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t dt0_node = nullptr;
  double graph_dt0 = 0.0;
  size_t total_faces = 0;
  double* h_stage = nullptr;
  size_t stage_len = 0;

  ~Ensemble() {
    cudaSetDevice(device);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : allocs) cudaFree(p);
    if (h_stage) cudaFreeHost(h_stage);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  T* dalloc(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count * sizeof(T), 16)) != cudaSuccess) throw std::bad_alloc();
    allocs.push_back(p);
    return static_cast<T*>(p);
  }
  template <typename T>
  T* upload(const std::vector<T>& h) {
    T* d = dalloc<T>(h.size());
    if (!h.empty() && cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
      throw std::runtime_error("upload failed");
    return d;
  }

  // Tiles of `width` faces (edges, with `edges`) of every member, in
  // schedule order: 0 member order, 1 largest members first, 2 round-robin
  // across members.
  std::vector<int2> make_tiles(int width, int ord, bool edges = false) const {
    auto count = [&](int i) { return edges ? inst[i].G.n_edges : inst[i].G.n_faces; };
    std::vector<int> members(n);
    for (int i = 0; i < n; ++i) members[i] = i;
    if (ord != 0)
      std::stable_sort(members.begin(), members.end(), [&](int a, int b) {
        return count(a) > count(b);
      });
    std::vector<int2> t;
    if (ord == 2) {
      for (int k = 0;; ++k) {
        bool any = false;
        for (int i : members) {
          if (k * width < count(i)) {
            t.push_back(make_int2(i, k * width));
            any = true;
          }
        }
        if (!any) break;
      }
    } else {
      for (int i : members)
        for (int f0 = 0; f0 < count(i); f0 += width) t.push_back(make_int2(i, f0));
    }
    return t;
  }

  int set_schedule(int ord, int width) {
    const std::vector<int2> ft = make_tiles(32, ord);
    const std::vector<int2> et = make_tiles(32, ord, true);
    if (!d_ftiles) {
      d_ftiles = dalloc<int2>(ft.size());
      d_etiles = dalloc<int2>(et.size());
    }
    ENS_CUDA(cudaMemcpy(d_ftiles, ft.data(), ft.size() * sizeof(int2), cudaMemcpyHostToDevice));
    ENS_CUDA(cudaMemcpy(d_etiles, et.data(), et.size() * sizeof(int2), cudaMemcpyHostToDevice));
    n_ftiles = (int)ft.size();
    n_etiles = (int)et.size();
    order = ord;
    recon_width = width;
    return SPLASH_OK;
  }

  int prepare() {
    ENS_CUDA(ensemble_prepare(d_inst, n, d_ftiles, n_ftiles, stream));
    return SPLASH_OK;
  }

  cudaError_t launch_step(double dt0) {
    return ensemble_step(d_inst, n, d_ftiles, n_ftiles, d_etiles, n_etiles, recon_width, max_slots, dt0, stream);
  }
  cudaError_t launch_persistent(double dt0, int steps) {
    return ensemble_persistent(d_inst, n, d_ftiles, n_ftiles, d_etiles, n_etiles, dt0, steps, d_bar, d_bar + 2,
                               pgrid, stream);
  }
  // the persistent launch's status word (after the stream has drained)
  int check_status() {
    unsigned st = 0;
    ENS_CUDA(cudaMemcpy(&st, d_bar + 2, sizeof st, cudaMemcpyDeviceToHost));
    if (st & kEnsBarrierTimeout)
      return set_error(SPLASH_E_CUDA, "ensemble: a grid barrier of the persistent launch timed out");
    return SPLASH_OK;
  }

  // Times every (order, width) candidate over a few steps, keeps the
  // fastest, and restores the state the trials advanced.
  int autotune(double dt0) {
    const size_t nU = total_faces * kDim;
    ENS_CUDA(cudaMemcpyAsync(U_snap, U, nU * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    ENS_CUDA(cudaMemcpyAsync(scal_snap, scal, (size_t)n * kScCount * sizeof(double),
                             cudaMemcpyDeviceToDevice, stream));
    ENS_CUDA(cudaMemcpyAsync(err_snap, err, (size_t)n * 4 * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                             stream));
    cudaEvent_t a, b;
    ENS_CUDA(cudaEventCreate(&a));
    ENS_CUDA(cudaEventCreate(&b));
    const int widths[3] = {32, 64, 128};  // threads per edge block (at most 128, the kernel's bound)
    double best = 1e30;
    int best_o = 0, best_w = 128;
    for (int o = 0; o < 3; ++o)
      for (int wi = 0; wi < 3; ++wi) {
        int rc = set_schedule(o, widths[wi]);
        if (rc) return rc;
        ENS_CUDA(launch_step(dt0));  // warm-up
        ENS_CUDA(cudaEventRecord(a, stream));
        for (int r = 0; r < 3; ++r) ENS_CUDA(launch_step(dt0));
        ENS_CUDA(cudaEventRecord(b, stream));
        ENS_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        ENS_CUDA(cudaEventElapsedTime(&ms, a, b));
        tuned_ms[o * 3 + wi] = ms / 3;
        if (ms < best) {
          best = ms;
          best_o = o;
          best_w = widths[wi];
        }
      }
    // the persistent launch, each tile order: 3 steps in one launch
    bool best_p = false;
    for (int o = 0; o < 3 && pgrid > 0; ++o) {
      int rc = set_schedule(o, 128);
      if (rc) return rc;
      ENS_CUDA(launch_persistent(dt0, 1));  // warm-up
      ENS_CUDA(cudaEventRecord(a, stream));
      ENS_CUDA(launch_persistent(dt0, 3));
      ENS_CUDA(cudaEventRecord(b, stream));
      ENS_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      ENS_CUDA(cudaEventElapsedTime(&ms, a, b));
      tuned_ms[9 + o] = ms / 3;
      if (ms < best) {
        best = ms;
        best_o = o;
        best_w = 128;
        best_p = true;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    int rc = check_status();
    if (rc) return rc;
    rc = set_schedule(best_o, best_w);
    if (rc) return rc;
    persistent = best_p;
    ENS_CUDA(cudaMemcpyAsync(U, U_snap, nU * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    ENS_CUDA(cudaMemcpyAsync(scal, scal_snap, (size_t)n * kScCount * sizeof(double),
                             cudaMemcpyDeviceToDevice, stream));
    ENS_CUDA(cudaMemcpyAsync(err, err_snap, (size_t)n * 4 * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                             stream));
    return prepare();
  }

  int capture() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    dt0_node = p_node = nullptr;
    graph_steps = 1;
    ENS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t le = persistent ? launch_persistent(graph_dt0, 1) : launch_step(graph_dt0);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(stream, &g);
    if (le != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return set_error(SPLASH_E_CUDA, "ensemble capture: %s", cudaGetErrorString(le));
    }
    ENS_CUDA(ce);
    graph = g;
    ENS_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    size_t nn = 0;
    ENS_CUDA(cudaGraphGetNodes(graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    ENS_CUDA(cudaGraphGetNodes(graph, nodes.data(), &nn));
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType t;
      ENS_CUDA(cudaGraphNodeGetType(nd, &t));
      if (t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      ENS_CUDA(cudaGraphKernelNodeGetParams(nd, &kp));
      if (kp.func == ensemble_finalize_kernel_ptr()) dt0_node = nd;
      if (kp.func == ensemble_persistent_kernel_ptr()) p_node = nd;
    }
    if (!(persistent ? p_node : dt0_node)) return set_error(SPLASH_E_CUDA, "ensemble dt node not found");
    return SPLASH_OK;
  }

  // do_steps: the five-launch graph replayed once per step, or the
  // persistent graph (one launch) replayed once for all n steps
  int steps(int nst, double dt0) {
    if (nst <= 0) return SPLASH_OK;
    if (!persistent) {
      for (int i = 0; i < nst; ++i) {
        const int rc = step(dt0);
        if (rc) return rc;
      }
      return SPLASH_OK;
    }
    if (dt0 != graph_dt0 || nst != graph_steps) {
      cudaKernelNodeParams kp{};
      ENS_CUDA(cudaGraphKernelNodeGetParams(p_node, &kp));
      const EnsInstance* di = d_inst;
      int nn = n, nft = n_ftiles, net = n_etiles, ns = nst;
      const int2 *ft = d_ftiles, *et = d_etiles;
      unsigned *bar = d_bar, *status = d_bar + 2;
      double d0 = dt0;
      void* args[] = {&di, &nn, &ft, &nft, &et, &net, &d0, &ns, &bar, &status};
      kp.kernelParams = args;
      kp.extra = nullptr;
      ENS_CUDA(cudaGraphExecKernelNodeSetParams(exec, p_node, &kp));
      graph_dt0 = dt0;
      graph_steps = nst;
    }
    ENS_CUDA(cudaGraphLaunch(exec, stream));
    return SPLASH_OK;
  }

  int step(double dt0) {
    if (dt0 != graph_dt0) {
      cudaKernelNodeParams kp{};
      ENS_CUDA(cudaGraphKernelNodeGetParams(dt0_node, &kp));
      const EnsInstance* di = d_inst;
      int nn = n;
      void* args[] = {&di, &nn, &dt0};
      kp.kernelParams = args;
      kp.extra = nullptr;
      ENS_CUDA(cudaGraphExecKernelNodeSetParams(exec, dt0_node, &kp));
      graph_dt0 = dt0;
    }
    ENS_CUDA(cudaGraphLaunch(exec, stream));
    return SPLASH_OK;
  }
};

}  // namespace splash

using splash::Ensemble;

extern "C" {

int splash_ensemble_create(const splash_member* members, int n, int device, int autotune,
                           splash_ensemble** out) {
  using namespace splash;
  if (!out) return set_error(SPLASH_E_INVALID, "out is NULL");
  *out = nullptr;
  if (!members || n <= 0) return set_error(SPLASH_E_INVALID, "need at least one member");
  for (int i = 0; i < n; ++i) {
    const splash_member& m = members[i];
    if (!m.U_in) return set_error(SPLASH_E_INVALID, "member %d: U_in is NULL", i);
    if (m.solver_kind < SPLASH_SOLVER_HLLE_P || m.solver_kind > SPLASH_SOLVER_HLLE)
      return set_error(SPLASH_E_INVALID, "member %d: unknown solver kind %d", i, m.solver_kind);
    if (!(m.gam > 1.0 && m.gam < 2.0)) return set_error(SPLASH_E_INVALID, "member %d: gam outside (1, 2)", i);
  }
  std::unique_ptr<Ensemble> e(new (std::nothrow) Ensemble());
  if (!e) return set_error(SPLASH_E_NOMEM, "host allocation failed");
  try {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      return set_error(SPLASH_E_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return set_error(SPLASH_E_INVALID, "device %d out of range", device);
    e->device = device;
    ENS_CUDA(cudaSetDevice(device));
    ENS_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    e->n = n;
    // one geometry per distinct mesh
    std::map<std::pair<int, int>, int> level_of;
    for (int i = 0; i < n; ++i) {
      const auto key = std::make_pair(members[i].mesh_kind, members[i].level);
      auto it = level_of.find(key);
      if (it == level_of.end()) {
        splash::Level L;
        L.kind = key.first;
        L.level = key.second;
        L.geom = build_ref_geometry(mesh_arrays(build_mesh(L.kind, L.level)), 0);
        if (L.geom.max_slots > 8)
          return set_error(SPLASH_E_UNSUPPORTED, "faces of more than 8 edges");
        L.sp = make_slot_planes(L.geom);
        const MixedPlanes mp = make_mixed_planes(L.sp);
        L.G.n_faces = L.sp.n_faces;
        L.G.fpad = L.sp.fpad;
        L.G.max_slots = L.sp.max_slots;
        L.G.nslots = e->upload(L.sp.nslots);
        L.G.fcn = e->upload(L.sp.fcn);
        L.G.fcn32 = e->upload(mp.fcn32);
        L.G.fcn_lo = e->upload(mp.fcn_lo);
        L.G.area = e->upload(L.sp.area);
        L.G.coef = e->upload(mp.coef);
        L.G.slot_edge = e->upload(mp.slot_edge);
        L.G.n_edges = mp.n_edges;
        L.G.epad = mp.epad;
        L.G.e_ids = e->upload(mp.e_ids);
        L.G.e_ec = e->upload(mp.e_ec);
        L.G.e_en = e->upload(mp.e_en);
        L.G.e_sten = e->upload(mp.e_sten);
        L.G.e_beta = e->upload(mp.e_beta);
        L.G.e_h = e->upload(mp.e_h);
        it = level_of.emplace(key, (int)e->levels.size()).first;
        e->levels.push_back(std::move(L));
      }
      e->member_level.push_back(it->second);
      e->max_slots = std::max(e->max_slots, e->levels[it->second].sp.max_slots);
    }
    // pooled state
    size_t faces = 0, slots = 0, edges = 0;
    for (int i = 0; i < n; ++i) {
      const splash::Level& L = e->levels[e->member_level[i]];
      e->off_face.push_back(faces);
      e->off_slot.push_back(slots);
      e->off_edge.push_back(edges);
      faces += (size_t)L.sp.fpad;
      slots += L.sp.PS();
      edges += (size_t)L.G.epad;
    }
    e->total_faces = faces;
    e->U = e->dalloc<double>(faces * kDim);
    e->U_snap = e->dalloc<double>(faces * kDim);
    e->acc = e->dalloc<double>(faces);
    e->W32 = e->dalloc<float>(faces * kDim);
    e->W32b = e->dalloc<float>(faces * kDim);
    e->fe32 = e->dalloc<float>(edges * kDim);
    e->scal = e->dalloc<double>((size_t)n * kScCount);
    e->scal_snap = e->dalloc<double>((size_t)n * kScCount);
    e->err = e->dalloc<unsigned int>((size_t)n * 4);
    e->err_snap = e->dalloc<unsigned int>((size_t)n * 4);
    e->keys = e->dalloc<unsigned>((size_t)n * 2);
    ENS_CUDA(cudaMemset(e->U, 0, faces * kDim * sizeof(double)));
    ENS_CUDA(cudaMemset(e->W32, 0, faces * kDim * sizeof(float)));
    ENS_CUDA(cudaMemset(e->W32b, 0, faces * kDim * sizeof(float)));
    ENS_CUDA(cudaMemset(e->scal, 0, (size_t)n * kScCount * sizeof(double)));
    ENS_CUDA(cudaMemset(e->err, 0, (size_t)n * 4 * sizeof(unsigned)));
    size_t max_fpad = 0;
    for (const auto& L : e->levels) max_fpad = std::max(max_fpad, (size_t)L.sp.fpad);
    e->stage_len = max_fpad * kDim;
    ENS_CUDA(cudaMallocHost(&e->h_stage, e->stage_len * sizeof(double)));
    for (int i = 0; i < n; ++i) {
      const splash_member& m = members[i];
      const splash::Level& L = e->levels[e->member_level[i]];
      const int nf = L.sp.n_faces, fp = L.sp.fpad;
      EnsInstance I{};
      I.G = L.G;
      // the member's accretion source (depends on its tilt, rate and width)
      const double ac = area_coefficient(L.geom, m.params.acc_width);
      // the isothermal solver (4 state fields) has no source term
      const bool iso = m.solver_kind == SPLASH_SOLVER_HLLE;
      const int mdim = iso ? 4 : kDim;
      const bool acc_on = m.accretion_on != 0 && !iso;
      const std::vector<double> acc = accretion_source(L.sp, m.params, ac, acc_on);
      ENS_CUDA(cudaMemcpy(e->acc + e->off_face[i], acc.data(), fp * sizeof(double), cudaMemcpyHostToDevice));
      I.G.acc_src = e->acc + e->off_face[i];
      I.S.U = e->U + e->off_face[i] * kDim;
      I.S.W32 = e->W32 + e->off_face[i] * kDim;
      I.S.W32b = e->W32b + e->off_face[i] * kDim;
      I.S.uplus32 = nullptr;  // no writer reads a member's edge states
      I.S.fe32 = e->fe32 + e->off_edge[i] * kDim;
      I.S.scal = e->scal + (size_t)i * kScCount;
      I.S.err = e->err + (size_t)i * 4;
      I.S.keys = e->keys + (size_t)i * 2;
      double tm = 0;
      for (int r = 0; r < nf; ++r) tm += m.U_in[(size_t)r * mdim] * L.geom.area[r];
      PhysParams& P = I.P;
      P.gam = m.gam;
      P.omega_ns = m.omega_ns;
      P.e_acc = m.params.e_acc;
      P.omega_acc_x = 0;
      P.omega_acc_y = std::sin(m.params.tilt_angle) * m.params.omega_acc_abs;
      P.omega_acc_z = std::cos(m.params.tilt_angle) * m.params.omega_acc_abs;
      P.alpha = m.params.alpha;
      P.acc_rate = m.params.accretion_rate;
      P.total_mass = tm;
      P.h0 = L.geom.h0;
      P.round_diff = L.geom.round_diff;
      P.accretion_on = acc_on ? 1 : 0;
      P.friction_on = m.params.friction_on ? 1 : 0;
      P.solver = m.solver_kind;
      derive_params(P);
      // state, reference order -> internal planes
      std::vector<double> planes((size_t)fp * kDim, 0.0);
      for (int q = 0; q < nf; ++q)
        for (int k = 0; k < mdim; ++k) planes[(size_t)k * fp + q] = m.U_in[(size_t)L.sp.perm[q] * mdim + k];
      ENS_CUDA(cudaMemcpy(I.S.U, planes.data(), planes.size() * sizeof(double), cudaMemcpyHostToDevice));
      e->inst.push_back(I);
    }
    e->d_inst = e->upload(e->inst);
    e->d_bar = e->dalloc<unsigned>(4);
    ENS_CUDA(cudaMemset(e->d_bar, 0, 4 * sizeof(unsigned)));
    e->pgrid = ensemble_persistent_grid(device);
    int rc = e->set_schedule(0, 128);
    if (rc) return rc;
    rc = e->prepare();
    if (rc) return rc;
    if (autotune) {
      rc = e->autotune(1e-4);
      if (rc) return rc;
    }
    rc = e->capture();
    if (rc && e->persistent) {
      // a driver that cannot capture the cooperative launch: the fastest
      // five-launch schedule of the same tile order
      cudaGetLastError();
      const int o = e->order;
      int wi = 0;
      for (int k = 1; k < 3; ++k)
        if (e->tuned_ms[o * 3 + k] > 0 && e->tuned_ms[o * 3 + k] < e->tuned_ms[o * 3 + wi]) wi = k;
      e->persistent = false;
      rc = e->set_schedule(o, 32 << wi);
      if (!rc) rc = e->capture();
    }
    if (rc) return rc;
    ENS_CUDA(cudaStreamSynchronize(e->stream));
  } catch (const std::bad_alloc&) {
    return set_error(SPLASH_E_NOMEM, "allocation failed while building the ensemble");
  } catch (const std::exception& ex) {
    return set_error(SPLASH_E_MESH, "%s", ex.what());
  }
  *out = reinterpret_cast<splash_ensemble*>(e.release());
  return SPLASH_OK;
}

int splash_ensemble_destroy(splash_ensemble* h) {
  delete reinterpret_cast<Ensemble*>(h);
  return SPLASH_OK;
}

#define GET_ENS(h)                                                               \
  Ensemble* e = reinterpret_cast<Ensemble*>(h);                                  \
  if (!e) return splash::set_error(SPLASH_E_INVALID, "ensemble handle is NULL"); \
  ENS_CUDA(cudaSetDevice(e->device))

int splash_ensemble_do_steps(splash_ensemble* h, int n, double dt0) {
  GET_ENS(h);
  if (n < 0) return splash::set_error(SPLASH_E_INVALID, "n < 0");
  return e->steps(n, dt0);
}

int splash_ensemble_synchronize(splash_ensemble* h) {
  GET_ENS(h);
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  return e->check_status();
}

int splash_ensemble_set_schedule(splash_ensemble* h, int order, int edge_block) {
  GET_ENS(h);
  if (order < 0 || order > 2) return splash::set_error(SPLASH_E_INVALID, "order must be 0, 1 or 2");
  if (edge_block != 0 && edge_block != 32 && edge_block != 64 && edge_block != 128)
    return splash::set_error(SPLASH_E_INVALID, "edge_block must be 0 (persistent), 32, 64 or 128");
  if (edge_block == 0 && e->pgrid <= 0)
    return splash::set_error(SPLASH_E_UNSUPPORTED, "the device's occupancy for the persistent launch is unknown");
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  int rc = e->set_schedule(order, edge_block == 0 ? 128 : edge_block);
  if (rc) return rc;
  e->persistent = edge_block == 0;
  return e->capture();
}

int splash_ensemble_stream(splash_ensemble* h, void** stream) {
  Ensemble* e = reinterpret_cast<Ensemble*>(h);
  if (!e || !stream) return splash::set_error(SPLASH_E_INVALID, "NULL argument");
  *stream = (void*)e->stream;
  return SPLASH_OK;
}

int splash_ensemble_get_state(splash_ensemble* h, int member, double* U) {
  GET_ENS(h);
  if (member < 0 || member >= e->n || !U) return splash::set_error(SPLASH_E_INVALID, "bad member or U");
  const splash::Level& L = e->levels[e->member_level[member]];
  const int nf = L.sp.n_faces, fp = L.sp.fpad;
  const int mdim = (e->inst[member].P.solver == splash::kSolverIsoHLLE) ? 4 : splash::kDim;
  ENS_CUDA(cudaMemcpyAsync(e->h_stage, e->inst[member].S.U, (size_t)fp * splash::kDim * sizeof(double),
                           cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  const int rc = e->check_status();
  if (rc) return rc;
  for (int q = 0; q < nf; ++q)
    for (int k = 0; k < mdim; ++k) U[(size_t)L.sp.perm[q] * mdim + k] = e->h_stage[(size_t)k * fp + q];
  return SPLASH_OK;
}

int splash_ensemble_member_info(splash_ensemble* h, int member, double out[4], uint32_t* err) {
  GET_ENS(h);
  if (member < 0 || member >= e->n || !out) return splash::set_error(SPLASH_E_INVALID, "bad member or out");
  double sc[splash::kScCount];
  unsigned int ew = 0;
  ENS_CUDA(cudaMemcpyAsync(sc, e->inst[member].S.scal, sizeof sc, cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(cudaMemcpyAsync(&ew, e->inst[member].S.err, sizeof ew, cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  const int rc = e->check_status();
  if (rc) return rc;
  out[0] = sc[splash::kScTime];
  out[1] = sc[splash::kScDt];
  out[2] = sc[splash::kScMaxVel];
  out[3] = sc[splash::kScExtraDt];
  if (err) *err = ew;
  return SPLASH_OK;
}

int splash_ensemble_schedule(splash_ensemble* h, int* order, int* recon_width, double trial_ms[12]) {
  Ensemble* e = reinterpret_cast<Ensemble*>(h);
  if (!e) return splash::set_error(SPLASH_E_INVALID, "ensemble handle is NULL");
  if (order) *order = e->order;
  if (recon_width) *recon_width = e->persistent ? 0 : e->recon_width;
  if (trial_ms)
    for (int i = 0; i < 12; ++i) trial_ms[i] = e->tuned_ms[i];
  return SPLASH_OK;
}

int splash_ensemble_size(splash_ensemble* h, int* n_members, int64_t* total_faces) {
  Ensemble* e = reinterpret_cast<Ensemble*>(h);
  if (!e) return splash::set_error(SPLASH_E_INVALID, "ensemble handle is NULL");
  if (n_members) *n_members = e->n;
  if (total_faces) {
    int64_t t = 0;
    for (int i = 0; i < e->n; ++i) t += e->inst[i].G.n_faces;
    *total_faces = t;
  }
  return SPLASH_OK;
}

}  // extern "C"
