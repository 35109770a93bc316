// Device launchers of the tangent-linear model and of the discrete adjoint
// of the FP64 do_step (adjoint.cu), and the buffers they work on.
//
// The differentiated map is N FP64 steps with the dt schedule of the
// forward run frozen (the CFL clip is a min() whose derivative is taken on
// the branch the forward took: dt does not depend on the state).  One step
// is the reference's midpoint RK2 (MUSCL_base.hpp:124-161):
//   W0 = prim(U)      P0 = recon(W0)      U1 = floor(U + dt/2 Phi(W0, P0))
//   W1 = prim(U1)     P1 = recon(W1)      U2 = floor(U + dt   Phi(W1, P1))
// with Phi = source - flux divergence and floor the density floor.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "layout.hpp"

namespace splash {

constexpr int kTapeJ = 16;  // limiter-Jacobian tape planes per slot and stage

// Tangents of the TLM beside a value DevState.
struct TlmTangents {
  double* dU;
  double* dW0;
  double* dW1;
  double* duplus;
  const double* dacc;  // tangent of the per-face accretion profile
  double d_omega_y, d_omega_z, d_rate, d_total_mass;
};

// Primal data of one step, stored by the recomputation: the step's input
// state and its stage-1 state, their (Sigma, l, Pi), both stages' edge
// states, both stages' limiter Jacobians (16 planes per slot, see
// adjoint_rev.cuh) and the density-floor bits (1: stage 1, 2: stage 2).
struct StepTape {
  double* U;
  double* W0;
  double* U1;
  double* W1;
  double* P0;
  double* P1;
  double* J0;
  double* J1;
  uint8_t* mask;
};

// Scratch of the reverse sweep.
struct AdjScratch {
  double* A;    // [5][PS]  (dF/duL)^T Fb per slot
  double* B;    // [5][PS]  (dF/duR)^T Fb per slot
  double* PU;   // [10][PS] adjoints of the stencil interpolants
  double* Lw;   // [5][fp]  own-face reconstruction adjoint
  double* la2;  // [5][fp]  masked adjoint of the stage-2 increment
  double* la1;  // [5][fp]  masked adjoint of the stage-1 increment
  double* lam1; // [5][fp]  adjoint of U1
  double* th;   // [5][fp]  per-face adjoints of (acc0, omega_y, omega_z, acc_rate, total_mass)
  const int* inv_off;  // inverse stencil CSR: faces -> (slot * 4 + position)
  const int* inv_ent;
};

// ---- tangent-linear model (value state S + tangents T) ----
cudaError_t tlm_prepare(const DevGeom& G, const DevState& S, const TlmTangents& T, const PhysParams& P,
                        cudaStream_t st);
// One step: dt clip of the value state, then the four stage launches on
// Dual<1> (values bit-identical to fp64_step).
cudaError_t tlm_step(const DevGeom& G, const DevState& S, const TlmTangents& T, const PhysParams& P,
                     cudaStream_t st);

// ---- recomputation of one step from tape.U with dt = *dtp ----
// tape.W0 must hold prim(tape.U) (rc_prim).  Writes the rest of the tape
// and the step's output state to (U_next, W_next).
cudaError_t rc_prim(const DevGeom& G, const PhysParams& P, const double* U, double* W, cudaStream_t st);
cudaError_t rc_step(const DevGeom& G, const PhysParams& P, const double* dtp, const StepTape& t,
                    double* U_next, double* W_next, cudaStream_t st);

// ---- reverse of one step: lam (adjoint of the step's output) is replaced
// by the adjoint of its input; per-face parameter adjoints accumulate in
// X.th.  dt is the step's dt (host value).
cudaError_t adj_step(const DevGeom& G, const PhysParams& P, double dt, const StepTape& t, const AdjScratch& X,
                     double* lam, cudaStream_t st);

// ---- branch tape of the FP64 step (validation of the derivatives, taped.cuh) ----
// The FP64 step bodies on a scalar whose comparison outcomes are recorded
// (mode 0), replayed (mode 1: the branch-frozen map) or compared with the
// recording (mode 2: the plain step, counting departures), per face and
// launch in `tape`, a region of kTapeWords 32-bit words per face and launch:
// one launch for the initial prim(U) and four per step, in that order, each
// region n_faces * kTapeWords words.  pos: [n_faces] scratch; err (4 words,
// 8-byte aligned): err[0] bit 1 a face ran out of tape, bit 2 a replay read
// past what was recorded; err[2..3] a 64-bit count (replay: outcomes the
// values would have decided otherwise; compare: faces per launch whose
// branch path departed from the recording).
// taped_prim writes W = prim(U) (region 0); taped_step advances (U, W0)
// by one step with dt = *dtp, using W1, uplus and U1 as scratch (regions
// 4 i + 1 .. 4 i + 4 of step i, passed as `region`).
cudaError_t taped_prim(const DevGeom& G, const PhysParams& P, double* U, double* W, uint32_t* region,
                       uint32_t* pos, unsigned* err, int mode, cudaStream_t st);
cudaError_t taped_step(const DevGeom& G, const PhysParams& P, const double* dtp, double* U, double* W0,
                       double* W1, double* uplus, double* U1, uint32_t* region, uint32_t* pos, unsigned* err,
                       int mode, cudaStream_t st);
int taped_words_per_face();

}  // namespace splash
