// Tangent-linear model, forward recomputation and discrete adjoint of the
// FP64 MUSCL step (launchers declared in adjoint.hpp).
//
// Compiled with -fmad=false like step_fp64.cu: the TLM and the
// recomputation run the same per-face bodies (step_body_fp64.cuh), so their
// primal values are bit-identical to the FP64 time step and every branch
// (limiter cases, Riemann sides, HLLC+ switches, floors) is the one the
// forward run took.  The reverse kernels recompute their local primal and
// apply the hand-written reverses of adjoint_rev.cuh.
//
// Reverse of one step (adjoint.hpp gives the forward map), per stage:
//   adj_flux    per face: la = mask(lam); per slot Fb = -coef la,
//               A = (dF/duL)^T Fb, B = (dF/duR)^T Fb
//   adj_recon   per face: the adjoint of slot s's edge state is
//               A[s] + B[rev s] (the edge seen from both faces);
//               reverse reconstruction from the recomputation's limiter
//               tape -> interpolant adjoints PU, own Lw
//   adj_face    per face: lamW = Lw + sum over the inverse stencil of
//               beta * PU, + source reverse (dt_here la), -> prim reverse
// Every sum has a fixed order (no atomics): the adjoint is deterministic.
#include <cuda_runtime.h>

#include <cstdint>

#include "adjoint.hpp"
#include "adjoint_rev.cuh"
#include "dual.cuh"
#include "kernels.hpp"
#include "physics_fp64.cuh"
#include "reduce.cuh"
#include "step_body_fp64.cuh"
#include "taped.cuh"

namespace splash {
namespace f64 {
// state planes read and written as Taped values (taped.cuh)
template <>
struct Planes<Taped> {
  double* p;
  __device__ Taped ld(size_t i) const { return Taped(p[i]); }
  __device__ void st(size_t i, const Taped& x) const { p[i] = x.v; }
};
}  // namespace f64
}  // namespace splash

namespace splash {
namespace adj {
namespace {

using namespace splash::f64;
using D1 = Dual<1>;
static_assert(kTapeJ == rev::kTapePlanes, "tape plane count");
constexpr int kBlock = 64;     // TLM kernels: must match the FP64 step (partials per block)
constexpr int kRevBlock = 64;  // recomputation and reverse kernels (FP64-bound, register-heavy:
                               // small blocks spread the faces evenly over the SMs)

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }
inline int rev_blocks_for(int n) { return (n + kRevBlock - 1) / kRevBlock; }

__device__ __forceinline__ D1 dual1(double v, double d) {
  D1 r(v);
  r.d[0] = d;
  return r;
}

// ---------------------------------------------------------------------
// tangent-linear model
__global__ void __launch_bounds__(kBlock) tlm_prepare_kernel(DevGeom G, DevState S, TlmTangents T, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    const int fp = G.fpad;
    const Planes<D1> U{S.U, T.dU, 0}, W{S.W0, T.dW0, 0};
    D1 u[kDim], w[kDim];
    double uv[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      u[k] = U.ld((size_t)k * fp + f);
      uv[k] = u[k].v;
    }
    const D3 r = plane3(G.fcn, fp, f);
    prim_of(u, r, P.gam, w);
#pragma unroll
    for (int k = 0; k < kDim; ++k) W.st((size_t)k * fp + f, w[k]);
    dt_candidates(uv, r, G.area[f], P, vmax, dmin, sums);
  }
  red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

__global__ void __launch_bounds__(kBlock) tlm_recon_kernel(DevGeom G, PhysParams P, const double* __restrict__ sc,
                                                           Planes<D1> W, Planes<D1> uplus) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  recon_face<D1>(G, P, sc[kScDt], W, uplus, f);
}

template <int STAGE>
__global__ void __launch_bounds__(kBlock) tlm_flux_kernel(DevGeom G, DevState S, TlmTangents T, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    const int fp = G.fpad;
    const double dt = S.scal[kScDt];
    const double dt_here = (STAGE == 1) ? dt / 2 : dt;
    const SrcParams<D1> sp{dual1(G.acc_src[f], T.dacc[f]),
                           v3(D1(P.omega_acc_x), dual1(P.omega_acc_y, T.d_omega_y), dual1(P.omega_acc_z, T.d_omega_z)),
                           dual1(P.acc_rate, T.d_rate), dual1(P.total_mass, T.d_total_mass)};
    const Planes<D1> Win = (STAGE == 1) ? Planes<D1>{S.W0, T.dW0, 0} : Planes<D1>{S.W1, T.dW1, 0};
    const Planes<D1> U{S.U, T.dU, 0};
    D1 u[kDim];
    bool floored;
    const unsigned bits =
        flux_face<D1, D1>(G, P, sp, dt_here, Win, U, Planes<D1>{S.uplus, T.duplus, 0}, f, u, floored);
    if (bits) atomicOr(S.err, bits);
    const D3 fcn = plane3(G.fcn, fp, f);
    D1 w[kDim];
    prim_of(u, fcn, P.gam, w);
    const Planes<D1> Wout = (STAGE == 1) ? Planes<D1>{S.W1, T.dW1, 0} : Planes<D1>{S.W0, T.dW0, 0};
#pragma unroll
    for (int k = 0; k < kDim; ++k) Wout.st((size_t)k * fp + f, w[k]);
    if (STAGE == 2) {
      double uv[kDim];
#pragma unroll
      for (int k = 0; k < kDim; ++k) {
        U.st((size_t)k * fp + f, u[k]);
        uv[k] = u[k].v;
      }
      dt_candidates(uv, fcn, G.area[f], P, vmax, dmin, sums);
    }
  }
  if (STAGE == 2) red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

// ---------------------------------------------------------------------
// branch-frozen forward: the step bodies on Taped (taped.cuh)
__global__ void __launch_bounds__(kRevBlock) tp_prim_kernel(DevGeom G, PhysParams P, const double* __restrict__ U,
                                                         double* __restrict__ W) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  Taped u[kDim], w[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) u[k] = Taped(U[(size_t)k * fp + f]);
  prim_of(u, plane3(G.fcn, fp, f), P.gam, w);
#pragma unroll
  for (int k = 0; k < kDim; ++k) W[(size_t)k * fp + f] = w[k].v;
}

__global__ void __launch_bounds__(kRevBlock) tp_recon_kernel(DevGeom G, PhysParams P, const double* __restrict__ dtp,
                                                          double* W, double* uplus) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  recon_face<Taped>(G, P, *dtp, Planes<Taped>{W}, Planes<Taped>{uplus}, f);
}

template <int STAGE>
__global__ void __launch_bounds__(kRevBlock) tp_flux_kernel(DevGeom G, PhysParams P, const double* __restrict__ dtp,
                                                         double* Win, double* U0, double* uplus, double* Uout,
                                                         double* Wout) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  const double dt = *dtp;
  const double dt_here = (STAGE == 1) ? dt / 2 : dt;
  Taped u[kDim], w[kDim];
  bool floored;
  flux_face<Taped, double>(G, P, face_src_params<double>(G, P, f), dt_here, Planes<Taped>{Win}, Planes<Taped>{U0},
                           Planes<Taped>{uplus}, f, u, floored);
  prim_of(u, plane3(G.fcn, fp, f), P.gam, w);
#pragma unroll
  for (int k = 0; k < kDim; ++k) {
    Uout[(size_t)k * fp + f] = u[k].v;
    Wout[(size_t)k * fp + f] = w[k].v;
  }
}

// ---------------------------------------------------------------------
// recomputation (double, extra outputs)
__global__ void __launch_bounds__(kRevBlock) rc_prim_kernel(DevGeom G, PhysParams P, const double* __restrict__ U,
                                                         double* __restrict__ W) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  double u[kDim], w[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) u[k] = U[(size_t)k * fp + f];
  prim_of(u, plane3(G.fcn, fp, f), P.gam, w);
#pragma unroll
  for (int k = 0; k < kDim; ++k) W[(size_t)k * fp + f] = w[k];
}

__global__ void __launch_bounds__(kRevBlock) rc_recon_kernel(DevGeom G, PhysParams P, const double* __restrict__ dtp,
                                                             const double* __restrict__ W, double* __restrict__ uplus,
                                                             double* __restrict__ LJ) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  rev::recon_face_tape(G, P, *dtp, W, uplus, LJ, f);
}

template <int STAGE>
__global__ void __launch_bounds__(kRevBlock) rc_flux_kernel(DevGeom G, PhysParams P, const double* __restrict__ dtp,
                                                         const double* __restrict__ Win, const double* __restrict__ U0,
                                                         const double* __restrict__ uplus, double* __restrict__ Uout,
                                                         double* __restrict__ Wout, uint8_t* __restrict__ mask) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  const double dt = *dtp;
  const double dt_here = (STAGE == 1) ? dt / 2 : dt;
  double u[kDim], w[kDim];
  bool floored;
  flux_face<double, double>(G, P, face_src_params<double>(G, P, f), dt_here, Planes<double>{const_cast<double*>(Win)},
                            Planes<double>{const_cast<double*>(U0)}, Planes<double>{const_cast<double*>(uplus)}, f, u,
                            floored);
  const D3 fcn = plane3(G.fcn, fp, f);
  prim_of(u, fcn, P.gam, w);
#pragma unroll
  for (int k = 0; k < kDim; ++k) {
    Uout[(size_t)k * fp + f] = u[k];
    Wout[(size_t)k * fp + f] = w[k];
  }
  const uint8_t bit = floored ? (uint8_t)STAGE : (uint8_t)0;
  mask[f] = (STAGE == 1) ? bit : (uint8_t)(mask[f] | bit);
}

// ---------------------------------------------------------------------
// reverse sweep
__global__ void __launch_bounds__(kRevBlock) adj_flux_kernel(DevGeom G, PhysParams P, double dt_here,
                                                          const double* __restrict__ uplus,
                                                          const double* __restrict__ lam,
                                                          const uint8_t* __restrict__ mask, int bit,
                                                          double* __restrict__ la_out, double* __restrict__ A,
                                                          double* __restrict__ B) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  const size_t PS = (size_t)G.max_slots * fp;
  double la[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) la[k] = lam[(size_t)k * fp + f];
  if (mask[f] & bit) la[0] = 0.0;  // density floor: the output's Sigma is a constant
#pragma unroll
  for (int k = 0; k < kDim; ++k) la_out[(size_t)k * fp + f] = la[k];
  const double rd_dt = P.round_diff * dt_here;
  const double area = G.area[f];
  const int n = G.nslots[f];
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const int rv = G.rev[s];
    const double coef = rd_dt * G.chord[s] / area;
    double uL[kDim], uR[kDim], Fb[kDim], uLb[kDim], uRb[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      uL[k] = uplus[(size_t)k * PS + s];
      uR[k] = uplus[(size_t)k * PS + rv];
      Fb[k] = -coef * la[k];
      uLb[k] = 0.0;
      uRb[k] = 0.0;
    }
    SlotGeom g;
    g.ec = plane3(G.ec, (int)PS, s);
    g.ecn = G.ecn[s];
    g.en = plane3(G.en, (int)PS, s);
    g.nxr = plane3(G.nxr, (int)PS, s);
    rev::flux_star_rev(uL, uR, g, P.gam, P.solver, Fb, uLb, uRb);
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      A[(size_t)k * PS + s] = uLb[k];
      B[(size_t)k * PS + s] = uRb[k];
    }
  }
}

__global__ void __launch_bounds__(kRevBlock) adj_recon_kernel(DevGeom G, PhysParams P, double dt,
                                                              const double* __restrict__ W,
                                                              const double* __restrict__ uplus,
                                                              const double* __restrict__ LJ,
                                                              const double* __restrict__ A,
                                                              const double* __restrict__ B, double* __restrict__ PU,
                                                              double* __restrict__ Lw) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  const size_t PS = (size_t)G.max_slots * fp;
  double wb[kDim] = {0, 0, 0, 0, 0};
  rev::recon_face_rev(
      G, P, dt, W, uplus, LJ, [&](int k, int s) { return A[(size_t)k * PS + s] + B[(size_t)k * PS + G.rev[s]]; },
      PU, wb, f);
#pragma unroll
  for (int k = 0; k < kDim; ++k) Lw[(size_t)k * fp + f] = wb[k];
}

template <int STAGE>
__global__ void __launch_bounds__(kRevBlock) adj_face_kernel(DevGeom G, PhysParams P, double dt_here, AdjScratch X,
                                                          const double* __restrict__ Win,
                                                          const double* __restrict__ Uin,
                                                          const double* __restrict__ la,
                                                          double* __restrict__ lam_out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G.n_faces) return;
  const int fp = G.fpad;
  const size_t PS = (size_t)G.max_slots * fp;
  double wb[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) wb[k] = X.Lw[(size_t)k * fp + g];
  // the interpolants of the slots whose stencils hold face g
  for (int e = X.inv_off[g]; e < X.inv_off[g + 1]; ++e) {
    const int code = X.inv_ent[e];
    const size_t s = (size_t)(code >> 2);
    const int pos = code & 3;
    const double bt = G.beta[(size_t)pos * PS + s];
    const double* src = X.PU + (size_t)(pos >= 2 ? kDim : 0) * PS;
#pragma unroll
    for (int k = 0; k < kDim; ++k) wb[k] += bt * src[(size_t)k * PS + s];
  }
  const D3 fcn = plane3(G.fcn, fp, g);
  double w[kDim], u[kDim], srcb[kDim], ub[kDim] = {0, 0, 0, 0, 0}, pb[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < kDim; ++k) {
    w[k] = Win[(size_t)k * fp + g];
    u[k] = Uin[(size_t)k * fp + g];
    srcb[k] = dt_here * la[(size_t)k * fp + g];
  }
  if (P.accretion_on) {
    rev::source_rev(w, fcn, face_src_params<double>(G, P, g), P, srcb, wb, pb);
#pragma unroll
    for (int j = 0; j < 5; ++j) X.th[(size_t)j * fp + g] += pb[j];
  }
  rev::prim_rev(u, fcn, P.gam, wb, ub);
  if (STAGE == 2) {
#pragma unroll
    for (int k = 0; k < kDim; ++k) lam_out[(size_t)k * fp + g] = ub[k];
  } else {
    // U1 = floor(U + acc1) and U2 = floor(U + acc2) both hold U directly
#pragma unroll
    for (int k = 0; k < kDim; ++k)
      lam_out[(size_t)k * fp + g] = ub[k] + X.la1[(size_t)k * fp + g] + X.la2[(size_t)k * fp + g];
  }
}

}  // namespace
}  // namespace adj

// ---- launchers ----------------------------------------------------------
cudaError_t tlm_prepare(const DevGeom& G, const DevState& S, const TlmTangents& T, const PhysParams& P,
                        cudaStream_t st) {
  adj::tlm_prepare_kernel<<<adj::blocks_for(G.n_faces), adj::kBlock, 0, st>>>(G, S, T, P);
  return cudaGetLastError();
}

cudaError_t tlm_step(const DevGeom& G, const DevState& S, const TlmTangents& T, const PhysParams& P,
                     cudaStream_t st) {
  using adj::D1;
  const int nb = adj::blocks_for(G.n_faces);
  cudaError_t e = fp64_dt(S, P, G.n_faces, st);
  if (e != cudaSuccess) return e;
  const f64::Planes<D1> W0{S.W0, T.dW0, 0}, W1{S.W1, T.dW1, 0}, up{S.uplus, T.duplus, 0};
  adj::tlm_recon_kernel<<<nb, adj::kBlock, 0, st>>>(G, P, S.scal, W0, up);
  adj::tlm_flux_kernel<1><<<nb, adj::kBlock, 0, st>>>(G, S, T, P);
  adj::tlm_recon_kernel<<<nb, adj::kBlock, 0, st>>>(G, P, S.scal, W1, up);
  adj::tlm_flux_kernel<2><<<nb, adj::kBlock, 0, st>>>(G, S, T, P);
  return cudaGetLastError();
}

namespace {
// points the comparisons of the next launch at its tape region (the
// __constant__ update is ordered on the stream before the launch) and
// restarts every face's position
cudaError_t tape_region(const DevGeom& G, uint32_t* region, uint32_t* pos, unsigned* err, int mode,
                        cudaStream_t st) {
  // err[2..3] hold the 64-bit flip count
  const tape::TapeCfg cfg{region, pos, err, reinterpret_cast<unsigned long long*>(err + 2), mode};
  cudaError_t e = cudaMemcpyToSymbolAsync(tape::g_tape, &cfg, sizeof cfg, 0, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(pos, 0, (size_t)G.n_faces * sizeof(uint32_t), st);
}
}  // namespace

int taped_words_per_face() { return tape::kTapeWords; }

cudaError_t taped_prim(const DevGeom& G, const PhysParams& P, double* U, double* W, uint32_t* region,
                       uint32_t* pos, unsigned* err, int mode, cudaStream_t st) {
  cudaError_t e = tape_region(G, region, pos, err, mode, st);
  if (e != cudaSuccess) return e;
  adj::tp_prim_kernel<<<adj::rev_blocks_for(G.n_faces), adj::kRevBlock, 0, st>>>(G, P, U, W);
  return cudaGetLastError();
}

cudaError_t taped_step(const DevGeom& G, const PhysParams& P, const double* dtp, double* U, double* W0,
                       double* W1, double* uplus, double* U1, uint32_t* region, uint32_t* pos, unsigned* err,
                       int mode, cudaStream_t st) {
  const int nb = adj::rev_blocks_for(G.n_faces);
  constexpr int B = adj::kRevBlock;
  const size_t RW = (size_t)G.n_faces * tape::kTapeWords;
  cudaError_t e;
  if ((e = tape_region(G, region, pos, err, mode, st)) != cudaSuccess) return e;
  adj::tp_recon_kernel<<<nb, B, 0, st>>>(G, P, dtp, W0, uplus);
  if ((e = tape_region(G, region + RW, pos, err, mode, st)) != cudaSuccess) return e;
  adj::tp_flux_kernel<1><<<nb, B, 0, st>>>(G, P, dtp, W0, U, uplus, U1, W1);
  if ((e = tape_region(G, region + 2 * RW, pos, err, mode, st)) != cudaSuccess) return e;
  adj::tp_recon_kernel<<<nb, B, 0, st>>>(G, P, dtp, W1, uplus);
  if ((e = tape_region(G, region + 3 * RW, pos, err, mode, st)) != cudaSuccess) return e;
  adj::tp_flux_kernel<2><<<nb, B, 0, st>>>(G, P, dtp, W1, U, uplus, U, W0);
  return cudaGetLastError();
}

cudaError_t rc_prim(const DevGeom& G, const PhysParams& P, const double* U, double* W, cudaStream_t st) {
  adj::rc_prim_kernel<<<adj::rev_blocks_for(G.n_faces), adj::kRevBlock, 0, st>>>(G, P, U, W);
  return cudaGetLastError();
}

cudaError_t rc_step(const DevGeom& G, const PhysParams& P, const double* dtp, const StepTape& t, double* U_next,
                    double* W_next, cudaStream_t st) {
  const int nb = adj::rev_blocks_for(G.n_faces);
  constexpr int B = adj::kRevBlock;
  adj::rc_recon_kernel<<<nb, B, 0, st>>>(G, P, dtp, t.W0, t.P0, t.J0);
  adj::rc_flux_kernel<1><<<nb, B, 0, st>>>(G, P, dtp, t.W0, t.U, t.P0, t.U1, t.W1, t.mask);
  adj::rc_recon_kernel<<<nb, B, 0, st>>>(G, P, dtp, t.W1, t.P1, t.J1);
  adj::rc_flux_kernel<2><<<nb, B, 0, st>>>(G, P, dtp, t.W1, t.U, t.P1, U_next, W_next, t.mask);
  return cudaGetLastError();
}

cudaError_t adj_step(const DevGeom& G, const PhysParams& P, double dt, const StepTape& t, const AdjScratch& X,
                     double* lam, cudaStream_t st) {
  const int nb = adj::rev_blocks_for(G.n_faces);
  constexpr int B = adj::kRevBlock;
  // stage 2: U2 = floor(U + dt Phi(W1, P1))
  adj::adj_flux_kernel<<<nb, B, 0, st>>>(G, P, dt, t.P1, lam, t.mask, 2, X.la2, X.A, X.B);
  adj::adj_recon_kernel<<<nb, B, 0, st>>>(G, P, dt, t.W1, t.P1, t.J1, X.A, X.B, X.PU, X.Lw);
  adj::adj_face_kernel<2><<<nb, B, 0, st>>>(G, P, dt, X, t.W1, t.U1, X.la2, X.lam1);
  // stage 1: U1 = floor(U + dt/2 Phi(W0, P0))
  const double dt_half = dt / 2;
  adj::adj_flux_kernel<<<nb, B, 0, st>>>(G, P, dt_half, t.P0, X.lam1, t.mask, 1, X.la1, X.A, X.B);
  adj::adj_recon_kernel<<<nb, B, 0, st>>>(G, P, dt, t.W0, t.P0, t.J0, X.A, X.B, X.PU, X.Lw);
  adj::adj_face_kernel<1><<<nb, B, 0, st>>>(G, P, dt_half, X, t.W0, t.U, X.la1, lam);
  return cudaGetLastError();
}

}  // namespace splash
