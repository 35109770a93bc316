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
// One do_step (five launches; capturable).  With `ev` non-null (6 events)
// an event is recorded before the first and after every launch.
cudaError_t fp64_step(const DevGeom& G, const DevState& S, const PhysParams& P, cudaStream_t st,
                      cudaEvent_t* ev = nullptr);
// The dt clip (one block) shared by both paths.
// squared_speeds: the partials hold max |v|^2 (mixed path), so the finalize
// takes the square root of the reduced maximum.
cudaError_t dt_reduce(const DevState& S, const PhysParams& P, int nblocks, cudaStream_t st,
                      bool squared_speeds = false);
cudaError_t fp64_scatter_state(const double* aos, const int* perm, double* U, int n_faces, int fpad,
                               cudaStream_t st);
cudaError_t fp64_gather_state(const double* U, const int* perm, double* aos, int n_faces, int fpad,
                              cudaStream_t st);

// ---- FP32/FP64 mixed path (step_mixed.cu) ----
cudaError_t mixed_prepare(const DevGeomMixed& G, const DevState& S, const PhysParams& P,
                          cudaStream_t st);
cudaError_t mixed_step(const DevGeomMixed& G, const DevState& S, const PhysParams& P,
                       cudaStream_t st, cudaEvent_t* ev = nullptr);
int mixed_partial_blocks(int n_faces);

}  // namespace splash
