// Host-callable launchers of the device kernels.  All are asynchronous on
// the given stream and return the launch status.
#pragma once

#include <cuda_runtime.h>

#include "layout.hpp"

namespace splash {

// ---- FP64 path (step_fp64.cu) ----
int fp64_partial_blocks(int n_faces);
// W0 and the dt partials of the current U (after the state is set).
cudaError_t fp64_prepare(const DevGeom& G, const DevState& S, const PhysParams& P, cudaStream_t st);
cudaError_t fp64_set_dt0(const DevState& S, double dt0, cudaStream_t st);
// The dt clip of one step alone (first launch of fp64_step): reduces the
// per-block partials of the current state into S.scal.
cudaError_t fp64_dt(const DevState& S, const PhysParams& P, int n_faces, cudaStream_t st);
// One do_step (five launches; capturable).  With `ev` non-null (6 events)
// an event is recorded before the first and after every launch.
cudaError_t fp64_step(const DevGeom& G, const DevState& S, const PhysParams& P, cudaStream_t st,
                      cudaEvent_t* ev = nullptr);
// reference-order [n_faces][dim] <-> internal planes (dim 5, or 4 for the
// isothermal solver, whose fifth plane is zero); iperm[reference face] =
// internal face.  aos may be host memory the device can access.
cudaError_t fp64_scatter_state(const double* aos, const int* iperm, double* U, int n_faces, int fpad,
                               cudaStream_t st, int dim = kDim);
cudaError_t fp64_gather_state(const double* U, const int* iperm, double* aos, int n_faces, int fpad,
                              cudaStream_t st, int dim = kDim);

// ---- FP32/FP64 mixed path (step_mixed.cu) ----
// One do_step: four stage launches (edge, update per stage); the stage-1
// edge launch (argument dt0) clips the step's dt from the keys the previous
// stage-2 update (or set_state) folded, and the stage-1 update restarts
// them.  Capturable; the stage-1 edge node's dt0 can be updated in an
// instantiated graph (mixed_dt0_kernel_ptr identifies the node).
// ev (optional): six events recorded on st (before the step, an empty dt
// slot, after each stage's edge launch and update launch); per_launch gives
// the same layout.
cudaError_t mixed_step(const DevGeomMixed& G, const DevState& S, const PhysParams& P, double dt0,
                       cudaStream_t st, cudaEvent_t* ev = nullptr, bool per_launch = false);
const void* mixed_dt0_kernel_ptr();
// The last step's stage-2 edge states into S.uplus32 (for write_t_curl),
// recomputed from the stage-2 input face states S.W32b and the step's dt.
cudaError_t mixed_edge_states(const DevGeomMixed& G, const DevState& S, const PhysParams& P, cudaStream_t st);
// set_state + prepare in one pass: aos is the caller's [n_faces][dim] array
// in reference order (host memory the device can access, or device memory),
// iperm maps reference to internal face indices.
cudaError_t mixed_scatter_prepare(const double* aos, const int* iperm, const DevGeomMixed& G, const DevState& S,
                                  const PhysParams& P, int dim, cudaStream_t st);

// ---- ensemble (step_mixed.cu): batched launches over instances ----
// ftiles: (instance, first face) of 32-face tiles; etiles: (instance,
// first edge) of 32-edge tiles; edge_block: threads per block of the
// reconstruction + edge-flux launch (a multiple of 32; one tile per warp);
// max_slots: the largest face degree over the members' meshes.
cudaError_t ensemble_prepare(const EnsInstance* inst, int n_inst, const int2* ftiles, int n_ftiles,
                             cudaStream_t st);
cudaError_t ensemble_step(const EnsInstance* inst, int n_inst, const int2* ftiles, int n_ftiles,
                          const int2* etiles, int n_etiles, int edge_block, int max_slots, double dt0,
                          cudaStream_t st);
const void* ensemble_finalize_kernel_ptr();
// The same n_steps steps as one cooperative launch of `grid` resident blocks
// (ensemble_persistent_grid: the occupancy of the current device, 0 if it
// cannot be read): per step the dt clip, edge and update of each stage,
// separated by grid barriers on bar[0..1] (zeroed here before the launch).
// A barrier wait that runs out sets kEnsBarrierTimeout in *status.
constexpr unsigned kEnsBarrierTimeout = 1u;
int ensemble_persistent_grid(int device);
cudaError_t ensemble_persistent(const EnsInstance* inst, int n_inst, const int2* ftiles, int n_ftiles,
                                const int2* etiles, int n_etiles, double dt0, int n_steps, unsigned* bar,
                                unsigned* status, int grid, cudaStream_t st);
const void* ensemble_persistent_kernel_ptr();

}  // namespace splash
