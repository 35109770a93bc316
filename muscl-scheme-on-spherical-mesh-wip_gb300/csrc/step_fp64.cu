// FP64 kernels of the MUSCL time step (the reference method in FP64).
//
// One do_step(dt0) (MUSCL_base/MUSCL_base.hpp:97-225) is five launches on
// one stream, captured once into a CUDA graph by the host:
//
//   dt_kernel          1 block  : reduce the previous launch's per-block
//                                 partials -> max_vel, extra_dt, clipped dt,
//                                 time; diagnostics sums
//   reconstruct(W0)    per face : limited edge states of every slot
//   flux_update(1)     per face : Riemann fluxes, source, res2d(dt/2) + U0
//                                 -> W1 (Sigma, l, Pi)
//   reconstruct(W1)    per face
//   flux_update(2)     per face : res2d(dt) + U0 -> U, W0 for the next step,
//                                 per-block partials of the new state
//
// Per-face threads loop over the face's slots in the reference slot order,
// so the flux divergence accumulates in exactly the reference order.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"
#include "physics_fp64.cuh"
#include "physics_iso.cuh"
#include "step_body_fp64.cuh"
#include "reduce.cuh"

namespace splash {
namespace f64 {
namespace {

constexpr int kBlock = 64;  // FP64-pipe bound, register-heavy: small blocks balance the SMs

// ---------------------------------------------------------------------
// W = (Sigma, l, Pi) of the conserved state and the partials of it
// (used once after the state is set; afterwards flux_update stage 2
// produces both).
__global__ void __launch_bounds__(kBlock) prepare_kernel(DevGeom G, DevState S, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) u[k] = S.U[k * G.fpad + f];
    const D3 r = plane3(G.fcn, G.fpad, f);
    double w[kDim];
    prim_of(u, r, P.gam, w);
#pragma unroll
    for (int k = 0; k < kDim; ++k) S.W0[k * G.fpad + f] = w[k];
    dt_candidates(u, r, G.area[f], P, vmax, dmin, sums);
  }
  red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

// dt = min(dt0, 0.1 h0 / max_vel, extra_dt)  (MUSCL_base.hpp:100-115)
__global__ void __launch_bounds__(256) dt_kernel(DevState S, PhysParams P, int nblocks) {
  __shared__ double sm[256][7];
  double v[7] = {1e-8, 1e20, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double* p = S.partial + (size_t)b * kPartialStride;
    v[0] = fmax(v[0], p[0]);
    v[1] = fmin(v[1], p[1]);
#pragma unroll
    for (int k = 2; k < 7; ++k) v[k] = v[k] + p[k];
  }
#pragma unroll
  for (int k = 0; k < 7; ++k) sm[threadIdx.x][k] = v[k];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sm[threadIdx.x][0] = fmax(sm[threadIdx.x][0], sm[threadIdx.x + s][0]);
      sm[threadIdx.x][1] = fmin(sm[threadIdx.x][1], sm[threadIdx.x + s][1]);
#pragma unroll
      for (int k = 2; k < 7; ++k) sm[threadIdx.x][k] = sm[threadIdx.x][k] + sm[threadIdx.x + s][k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double max_vel = sm[0][0];
    double extra = sm[0][1];
    if (extra < 0) {
      atomicOr(S.err, 8u);  // SPLASH_STOP_NEG_EXTRA_DT
      extra = 1e20;
    }
    double dt = S.scal[kScDt0];
    if (dt > P.h0 * 0.1 / max_vel) dt = P.h0 * 0.1 / max_vel;
    if (dt > extra) dt = extra;
    S.scal[kScDt] = dt;
    S.scal[kScMaxVel] = max_vel;
    S.scal[kScExtraDt] = extra;
#pragma unroll
    for (int k = 0; k < 5; ++k) S.scal[kScMass + k] = sm[0][2 + k];
    S.scal[kScTime] = S.scal[kScTime] + dt;
  }
}

// find_U_edges (MUSCL_base.hpp:361-434) for every slot of one face.
__global__ void __launch_bounds__(kBlock) reconstruct_kernel(DevGeom G, const double* __restrict__ W,
                                                             double* __restrict__ uplus,
                                                             const double* __restrict__ sc,
                                                             PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  recon_face<double>(G, P, sc[kScDt], Planes<double>{const_cast<double*>(W)}, Planes<double>{uplus}, f);
}

// find_flux_var + res2d + the RK combine with the density floor
// (MUSCL_base.hpp:345-359, 238-276, 124-161).  stage 1: dt_here = dt/2,
// writes W1; stage 2: dt_here = dt, writes U, W0 and the partials.
template <int STAGE>
__global__ void __launch_bounds__(kBlock) flux_update_kernel(DevGeom G, DevState S, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    const int fp = G.fpad;
    const double dt = S.scal[kScDt];
    const double dt_here = (STAGE == 1) ? dt / 2 : dt;
    double u[kDim];
    bool floored;
    const unsigned bits =
        flux_face<double, double>(G, P, face_src_params<double>(G, P, f), dt_here,
                                  Planes<double>{(STAGE == 1) ? S.W0 : S.W1}, Planes<double>{S.U},
                                  Planes<double>{S.uplus}, f, u, floored);
    if (bits) atomicOr(S.err, bits);
    const D3 fcn = plane3(G.fcn, fp, f);
    double w[kDim];
    prim_of(u, fcn, P.gam, w);
    double* Wout = (STAGE == 1) ? S.W1 : S.W0;
#pragma unroll
    for (int k = 0; k < kDim; ++k) Wout[k * fp + f] = w[k];
    if (STAGE == 2) {
#pragma unroll
      for (int k = 0; k < kDim; ++k) S.U[k * fp + f] = u[k];
      dt_candidates(u, fcn, G.area[f], P, vmax, dmin, sums);
    }
  }
  if (STAGE == 2) red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

// ---- isothermal solver (MUSCL_HLLE, 4 fields; planes 0..3 of U/W/U+) ----
// W of a 4-field state is the state itself (find_U_edges subtracts the
// zero profile rho_an from field 0, MUSCL_base.hpp:366-371).
__global__ void __launch_bounds__(kBlock) iso_prepare_kernel(DevGeom G, DevState S) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    double u[kDim];
#pragma unroll
    for (int k = 0; k < iso::kIsoDim; ++k) u[k] = S.U[k * G.fpad + f];
    u[4] = 0.0;
    S.W0[f] = u[0] - 0.0;
#pragma unroll
    for (int k = 1; k < iso::kIsoDim; ++k) S.W0[k * G.fpad + f] = u[k];
    iso::dt_candidates(u, plane3(G.fcn, G.fpad, f), G.area[f], vmax, dmin, sums);
  }
  red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

// find_U_edges with the isothermal limiter (MUSCL_base.hpp:361-434,
// physics/isothermal.hpp:269-320) for every slot of one face
__global__ void __launch_bounds__(kBlock) iso_reconstruct_kernel(DevGeom G, const double* __restrict__ W,
                                                                 double* __restrict__ uplus,
                                                                 const double* __restrict__ sc) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  const int PS = G.max_slots * fp;
  const double dt = sc[kScDt];
  double w[iso::kIsoDim];
#pragma unroll
  for (int k = 0; k < iso::kIsoDim; ++k) w[k] = W[k * fp + f];
  const int n = G.nslots[f];
  const double twoN = (double)(2 * n);
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const int ia = G.sten[s], ib = G.sten[PS + s], ic = G.sten[2 * PS + s], id = G.sten[3 * PS + s];
    const double bp0 = G.beta[s], bp1 = G.beta[PS + s], bm0 = G.beta[2 * PS + s], bm1 = G.beta[3 * PS + s];
    const double hp = G.hpm[s], hm = G.hpm[PS + s], bmd = G.bm[s];
    const D3 ec = plane3(G.ec, PS, s);
    const D3 en = plane3(G.en, PS, s);
    const double nu_plus = iso::courant(w, ec, en, dt, G.arc_a[s]);
    const double eta = G.eta[PS + s];
#pragma unroll
    for (int k = 0; k < iso::kIsoDim; ++k) {
      const double* Wk = W + k * fp;
      const double Up = bp0 * Wk[ia] + bp1 * Wk[ib];
      const double pp = (Up - w[k]) / hp;
      const double Um = bm0 * Wk[ic] + bm1 * Wk[id];
      const double pm = (-Um + w[k]) / hm;
      const double lim = iso::limiter_field(pm / pp, eta, twoN, nu_plus);
      uplus[k * PS + s] = (k == 0) ? w[k] + 0.0 + pp * lim * bmd : w[k] + pp * lim * bmd;
    }
  }
}

// find_flux_var + res2d + the RK combine (zero source) for one face;
// stage 1: dt/2, writes W1; stage 2: dt, writes U, W0 and the partials
template <int STAGE>
__global__ void __launch_bounds__(kBlock) iso_flux_update_kernel(DevGeom G, DevState S, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    const int fp = G.fpad;
    const int PS = G.max_slots * fp;
    const double dt = S.scal[kScDt];
    const double dt_here = (STAGE == 1) ? dt / 2 : dt;
    const double area = G.area[f];
    double acc[iso::kIsoDim];
#pragma unroll
    for (int k = 0; k < iso::kIsoDim; ++k) acc[k] = dt_here * 0.0;
    const double rd_dt = P.round_diff * dt_here;
    const int n = G.nslots[f];
    unsigned bits = 0;
    for (int j = 0; j < n; ++j) {
      const int s = j * fp + f;
      const int rv = G.rev[s];
      double uL[iso::kIsoDim], uR[iso::kIsoDim], F[iso::kIsoDim];
#pragma unroll
      for (int k = 0; k < iso::kIsoDim; ++k) {
        uL[k] = S.uplus[k * PS + s];
        uR[k] = S.uplus[k * PS + rv];
      }
      bits |= iso::flux_star(uL, uR, plane3(G.ec, PS, s), G.ecn[s], plane3(G.en, PS, s), F);
      const double coef = rd_dt * G.chord[s] / area;
#pragma unroll
      for (int k = 0; k < iso::kIsoDim; ++k) {
        if (isnan(F[k])) bits |= 1u;
        acc[k] -= coef * F[k];
      }
    }
    if (bits) atomicOr(S.err, bits);
    double u[kDim];
#pragma unroll
    for (int k = 0; k < iso::kIsoDim; ++k) u[k] = acc[k] + S.U[k * fp + f];
    u[4] = 0.0;
    if (u[0] < 1e-8) u[0] = 1e-8;
    double* Wout = (STAGE == 1) ? S.W1 : S.W0;
    Wout[f] = u[0] - 0.0;
#pragma unroll
    for (int k = 1; k < iso::kIsoDim; ++k) Wout[k * fp + f] = u[k];
    if (STAGE == 2) {
#pragma unroll
      for (int k = 0; k < iso::kIsoDim; ++k) S.U[k * fp + f] = u[k];
      iso::dt_candidates(u, plane3(G.fcn, fp, f), area, vmax, dmin, sums);
    }
  }
  if (STAGE == 2) red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

__global__ void set_scalar_kernel(double* dst, double v) { *dst = v; }

// reference order [F][dim] <-> internal planes
// One thread per element of the [n_faces][dim] array, in its memory order,
// so that every warp reads or writes 256 contiguous bytes of it -- device
// memory or, on a coherent host link, the caller's host memory, where
// partial-line accesses are expensive; the planes take the permuted side.
// (dim = 4: the fifth plane is written as zero by the scatter.)
__global__ void scatter_state_kernel(const double* __restrict__ aos, const int* __restrict__ iperm,
                                     double* __restrict__ U, int n_faces, int fpad, int dim) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n_faces * dim) return;
  const int r = (int)(e / dim), k = (int)(e % dim);
  const int i = iperm[r];
  U[(size_t)k * fpad + i] = aos[e];
  if (dim == 4 && k == 3) U[(size_t)4 * fpad + i] = 0.0;
}
__global__ void gather_state_kernel(const double* __restrict__ U, const int* __restrict__ iperm,
                                    double* __restrict__ aos, int n_faces, int fpad, int dim) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n_faces * dim) return;
  const int r = (int)(e / dim), k = (int)(e % dim);
  aos[e] = U[(size_t)k * fpad + iperm[r]];
}
// Two consecutive elements per thread with one 16-byte access on the
// caller's side (used when the caller's array is 16-byte aligned): half the
// warp instructions on the host link, 512 contiguous bytes per warp access.
__global__ void gather_state2_kernel(const double* __restrict__ U, const int* __restrict__ iperm,
                                     double* __restrict__ aos, int n_faces, int fpad, int dim) {
  const unsigned ne = (unsigned)n_faces * (unsigned)dim;
  const unsigned e0 = 2u * (blockIdx.x * blockDim.x + threadIdx.x);
  if (e0 >= ne) return;
  double v[2] = {0.0, 0.0};
#pragma unroll
  for (unsigned q = 0; q < 2; ++q) {
    const unsigned e = e0 + q;
    if (e < ne) {
      const unsigned r = e / (unsigned)dim, k = e - r * (unsigned)dim;
      v[q] = U[(size_t)k * fpad + iperm[r]];
    }
  }
  if (e0 + 1 < ne)
    *reinterpret_cast<double2*>(aos + e0) = make_double2(v[0], v[1]);
  else
    aos[e0] = v[0];
}
constexpr int kMoveBlock = 256;

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace
}  // namespace f64

// ---- launchers (declared in kernels.hpp) --------------------------------
int fp64_partial_blocks(int n_faces) { return f64::blocks_for(n_faces); }

cudaError_t fp64_prepare(const DevGeom& G, const DevState& S, const PhysParams& P,
                         cudaStream_t st) {
  if (P.solver == kSolverIsoHLLE)
    f64::iso_prepare_kernel<<<f64::blocks_for(G.n_faces), f64::kBlock, 0, st>>>(G, S);
  else
    f64::prepare_kernel<<<f64::blocks_for(G.n_faces), f64::kBlock, 0, st>>>(G, S, P);
  return cudaGetLastError();
}

cudaError_t fp64_dt(const DevState& S, const PhysParams& P, int n_faces, cudaStream_t st) {
  f64::dt_kernel<<<1, 256, 0, st>>>(S, P, f64::blocks_for(n_faces));
  return cudaGetLastError();
}

cudaError_t fp64_set_dt0(const DevState& S, double dt0, cudaStream_t st) {
  f64::set_scalar_kernel<<<1, 1, 0, st>>>(S.scal + kScDt0, dt0);
  return cudaGetLastError();
}

cudaError_t fp64_step(const DevGeom& G, const DevState& S, const PhysParams& P, cudaStream_t st,
                      cudaEvent_t* ev) {
  const int nb = f64::blocks_for(G.n_faces);
  if (ev) cudaEventRecord(ev[0], st);
  f64::dt_kernel<<<1, 256, 0, st>>>(S, P, nb);
  if (ev) cudaEventRecord(ev[1], st);
  if (P.solver == kSolverIsoHLLE) {
    f64::iso_reconstruct_kernel<<<nb, f64::kBlock, 0, st>>>(G, S.W0, S.uplus, S.scal);
    if (ev) cudaEventRecord(ev[2], st);
    f64::iso_flux_update_kernel<1><<<nb, f64::kBlock, 0, st>>>(G, S, P);
    if (ev) cudaEventRecord(ev[3], st);
    f64::iso_reconstruct_kernel<<<nb, f64::kBlock, 0, st>>>(G, S.W1, S.uplus, S.scal);
    if (ev) cudaEventRecord(ev[4], st);
    f64::iso_flux_update_kernel<2><<<nb, f64::kBlock, 0, st>>>(G, S, P);
    if (ev) cudaEventRecord(ev[5], st);
    return cudaGetLastError();
  }
  f64::reconstruct_kernel<<<nb, f64::kBlock, 0, st>>>(G, S.W0, S.uplus, S.scal, P);
  if (ev) cudaEventRecord(ev[2], st);
  f64::flux_update_kernel<1><<<nb, f64::kBlock, 0, st>>>(G, S, P);
  if (ev) cudaEventRecord(ev[3], st);
  f64::reconstruct_kernel<<<nb, f64::kBlock, 0, st>>>(G, S.W1, S.uplus, S.scal, P);
  if (ev) cudaEventRecord(ev[4], st);
  f64::flux_update_kernel<2><<<nb, f64::kBlock, 0, st>>>(G, S, P);
  if (ev) cudaEventRecord(ev[5], st);
  return cudaGetLastError();
}

cudaError_t fp64_scatter_state(const double* aos, const int* iperm, double* U, int n_faces,
                               int fpad, cudaStream_t st, int dim) {
  const size_t ne = (size_t)n_faces * dim;
  f64::scatter_state_kernel<<<(unsigned)((ne + f64::kMoveBlock - 1) / f64::kMoveBlock), f64::kMoveBlock, 0, st>>>(
      aos, iperm, U, n_faces, fpad, dim);
  return cudaGetLastError();
}

cudaError_t fp64_gather_state(const double* U, const int* iperm, double* aos, int n_faces,
                              int fpad, cudaStream_t st, int dim) {
  const size_t ne = (size_t)n_faces * dim;
  if (((uintptr_t)aos & 15) == 0) {
    const size_t nt = (ne + 1) / 2;
    f64::gather_state2_kernel<<<(unsigned)((nt + f64::kMoveBlock - 1) / f64::kMoveBlock), f64::kMoveBlock, 0, st>>>(
        U, iperm, aos, n_faces, fpad, dim);
    return cudaGetLastError();
  }
  f64::gather_state_kernel<<<(unsigned)((ne + f64::kMoveBlock - 1) / f64::kMoveBlock), f64::kMoveBlock, 0, st>>>(
      U, iperm, aos, n_faces, fpad, dim);
  return cudaGetLastError();
}

}  // namespace splash
