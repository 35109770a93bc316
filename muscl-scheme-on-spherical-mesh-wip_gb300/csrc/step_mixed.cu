// FP32/FP64 mixed-precision kernels of the MUSCL time step.
//
// Same launch structure as the FP64 path (dt clip, then per stage a
// reconstruction and a flux + update launch), with the work split:
//   FP32: slopes and limiter, edge states, Riemann fluxes, source terms,
//         the per-slot flux contributions;
//   FP64: the conserved state U, the RK combine U0 + dt*Phi, pressure
//         recovery Pi = (E - |r x l|^2 / (2 Sigma)) (gam - 1), the CFL / extra
//         dt reduction, simulation time, and the accretion mass source;
//   compensated: the per-face sum of the FP32 contributions is carried as an
//         FP32 (hi, lo) pair and folded into FP64.
// W32 holds (Sigma, l, Pi) of the current stage input in FP32; every thread
// writes only its own face, so one buffer serves both stages.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"
#include "physics_fp64.cuh"
#include "physics_mixed.cuh"
#include "reduce.cuh"
#include "solver.hpp"

namespace splash {

bool mixed_available() { return true; }

namespace mx {
namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ F3 plane3f(const float* p, int stride, int i) {
  return F3{p[i], p[stride + i], p[2 * stride + i]};
}
__device__ __forceinline__ f64::D3 plane3d(const double* p, int stride, int i) {
  return f64::D3{p[i], p[stride + i], p[2 * stride + i]};
}

// FP64 pressure recovery with one division: Pi = (E - |r x l|^2/(2 Sigma))(gam-1),
// floored at 1e-16 like MUSCL_base.hpp:538.  Also returns |v|^2 and 1/Sigma
// for the dt candidates.
__device__ __forceinline__ double pressure_recover(const double* u, f64::D3 r, double gam,
                                                   double& v2, double& inv_rho) {
  const f64::D3 c = f64::cross3(r, f64::d3(u[1], u[2], u[3]));
  inv_rho = 1.0 / u[0];
  const double c2 = c.x * c.x + c.y * c.y + c.z * c.z;
  v2 = c2 * inv_rho * inv_rho;
  const double p = (u[4] - 0.5 * c2 * inv_rho) * (gam - 1.0);
  return (1e-16 < p) ? p : 1e-16;
}

__device__ __forceinline__ void store_w32(float* W32, int fp, int f, const double* u, double p) {
#pragma unroll
  for (int k = 0; k < 4; ++k) W32[k * fp + f] = (float)u[k];
  W32[4 * fp + f] = (float)p;
}

// dt candidates in FP64 with one sqrt and one division: the CFL maximum is
// reduced over squared speeds max(|v|^2, gam p / Sigma) (the square root is
// monotone, so the dt finalize takes one sqrt of the maximum), and
// extra_dt_constr (physics/adiabatic.hpp:543-580) simplifies to
// 0.01 p / (alpha k g_eff Sigma |v - v0|) with k = gam3d / (2 gam3d - 1).
__device__ __forceinline__ void dt_candidates_sq(const double* u, f64::D3 r, double area, double p,
                                                 double v2, double inv_rho, const PhysParams& P,
                                                 double& vmax2, double& dmin, double sums[5]) {
  vmax2 = fmax(v2, P.gam * p * inv_rho);
  const f64::D3 c = f64::cross3(r, f64::d3(u[1], u[2], u[3]));
  // v = (r x l) / (-Sigma) ; v0 = omega_ns z x r
  const double vx = -c.x * inv_rho + P.omega_ns * r.y;
  const double vy = -c.y * inv_rho - P.omega_ns * r.x;
  const double vz = -c.z * inv_rho;
  const double dv = sqrt(vx * vx + vy * vy + vz * vz);
  const double gam3d = 1 / (2 - P.gam);
  const double k = gam3d / (2 * gam3d - 1);
  const double g_eff = 0.217909 - v2;
  dmin = 0.01 * p / (P.alpha * k * g_eff * u[0] * dv);
#pragma unroll
  for (int q = 0; q < 5; ++q) sums[q] = u[q] * area;
}

// physics/adiabatic.hpp:396-541 in FP32, except the accretion mass source
// (a geometric constant kept in FP64 and added by the caller).  w[4] = Pi.
__device__ __forceinline__ void source_f32(const float* w, F3 fcn, float acc0, const PhysParams& P,
                                           float* res) {
#pragma unroll
  for (int i = 0; i < kDim; ++i) res[i] = 0.f;
  if (!P.accretion_on) return;
  const float gam = (float)P.gam;
  const F3 vel = scal(cross3(fcn, f3(w[1], w[2], w[3])), -1.0f / w[0]);
  const F3 omega_acc = f3((float)P.omega_acc_x, (float)P.omega_acc_y, (float)P.omega_acc_z);
  const F3 omxr = cross3(omega_acc, fcn);
  const F3 rxo = cross3(fcn, omxr);
  res[1] = acc0 * rxo.x;
  res[2] = acc0 * rxo.y;
  res[3] = acc0 * rxo.z;
  const F3 dvo = sub(omxr, vel);
  res[4] = acc0 * ((float)P.e_acc + 0.5f * dot3(dvo, dvo));
  const F3 rxv = cross3(fcn, vel);
  const float v2 = dot3(vel, vel);
  if (!P.friction_on) {
    const float dmdt = (float)(-(P.acc_rate * 4 * M_PI) / P.total_mass) * w[0];
    res[0] += dmdt;
    res[1] += dmdt * rxv.x;
    res[2] += dmdt * rxv.y;
    res[3] += dmdt * rxv.z;
    res[4] += dmdt * (gam / (gam - 1.f) * w[4] / w[0] + 0.5f * v2);
  }
  const float GM = 0.217909f;
  const float g_eff = GM - v2;
  // C = 12/5 k_m Sigma/Pi (3/4 c_sigma g_eff Sigma)^(1/4); constants folded
  // so that no intermediate leaves the FP32 range
  const float k1 = (float)(12. / 5 * 1.6e-13);
  const float q = (float)(3. / 4 * 4.85e36) * 1e-36f;  // scaled by 1e-36, undone by 10^9 below
  const float C = k1 * w[0] / w[4] * (sqrtf(sqrtf(q * g_eff * w[0])) * 1e9f);
  const float beta_switch = 0.736194670678821f;
  const float C_switch = -1.f - 1.f / (beta_switch - 1.f);
  float beta;
  if (C <= C_switch) {
    beta = 1.f - 1.f / (1.f + C);
  } else {
    const float x = 2.f / C;
    const float x2 = x * x;
    beta = 1.f - x2 * x2;
  }
  const float beta_ceil = 1.f - 1e-8f, beta_floor = 1e-8f;
  if (beta < beta_floor || isnan(beta)) beta = beta_floor;
  if (beta > beta_ceil) beta = beta_ceil;
  res[4] -= g_eff / 3.4e6f * (1.f - beta);
  if (P.friction_on) {
    const float gam3d = 1.f / (2.f - gam);
    const float rho = gam3d / (2.f * gam3d - 1.f) * g_eff * w[0] * w[0] / w[4];
    const F3 vel0 = cross3(f3(0.f, 0.f, (float)P.omega_ns), fcn);
    const F3 dv = sub(vel, vel0);
    const float dvn = norm3(dv);
    const float ar = (float)P.alpha * rho * dvn;
    const F3 wr = scal(dv, -ar);
    const F3 l_fr = cross3(fcn, wr);
    res[1] += l_fr.x;
    res[2] += l_fr.y;
    res[3] += l_fr.z;
    res[4] += dot3(wr, vel0);
    res[0] -= ar;
    res[1] -= ar / w[0] * w[1];
    res[2] -= ar / w[0] * w[2];
    res[3] -= ar / w[0] * w[3];
    res[4] -= ar * (0.5f * v2 + w[4] * gam / ((gam - 1.f) * w[0]));
  }
}

__global__ void __launch_bounds__(kBlock) prepare_kernel(DevGeomMixed G, DevState S, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) u[k] = S.U[k * G.fpad + f];
    const f64::D3 r = plane3d(G.fcn, G.fpad, f);
    double v2, inv_rho;
    const double p = pressure_recover(u, r, P.gam, v2, inv_rho);
    store_w32(S.W32, G.fpad, f, u, p);
    dt_candidates_sq(u, r, G.area[f], p, v2, inv_rho, P, vmax, dmin, sums);
  }
  red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

// find_U_edges (MUSCL_base.hpp:361-434) in FP32; edge field 4 stays Pi.
__global__ void __launch_bounds__(kBlock) reconstruct_kernel(DevGeomMixed G, DevState S, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= G.n_faces) return;
  const int fp = G.fpad;
  const int PS = G.max_slots * fp;
  const float* __restrict__ W = S.W32;
  const float dt = (float)S.scal[kScDt];
  const float gam = (float)P.gam;
  float w[kDim];
#pragma unroll
  for (int k = 0; k < kDim; ++k) w[k] = W[k * fp + f];
  const int n = G.nslots[f];
  const float twoN = (float)(2 * n);
  const float inv_rho = -1.0f / w[0];
  const float c = sqrtf(gam * w[4] / w[0]);
  for (int j = 0; j < n; ++j) {
    const int s = j * fp + f;
    const int ia = G.sten[s], ib = G.sten[PS + s], ic = G.sten[2 * PS + s], id = G.sten[3 * PS + s];
    const float bp0 = G.beta[s], bp1 = G.beta[PS + s], bm0 = G.beta[2 * PS + s], bm1 = G.beta[3 * PS + s];
    const float ihp = G.inv_h[s], ihm = G.inv_h[PS + s], bmd = G.bm[s];
    const F3 ec = plane3f(G.ec, PS, s);
    const F3 en = plane3f(G.en, PS, s);
    const F3 vel = scal(cross3(ec, f3(w[1], w[2], w[3])), inv_rho);
    const float nu_plus = (c + dot3(vel, en)) * dt * G.arc_a[s];
    const float eta_p = G.eta[s];
    const float sb_scale = G.eta[PS + s] / (twoN * nu_plus);
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      const float* Wk = W + k * fp;
      const float pp = (bp0 * Wk[ia] + bp1 * Wk[ib] - w[k]) * ihp;
      const float pm = (w[k] - (bm0 * Wk[ic] + bm1 * Wk[id])) * ihm;
      const float r = pm / pp;
      const float lim = limiter_field(r, nu_plus, eta_p, sb_scale);
      S.uplus32[k * PS + s] = w[k] + pp * lim * bmd;
    }
  }
}

template <int STAGE>
__global__ void __launch_bounds__(kBlock) flux_update_kernel(DevGeomMixed G, DevState S, PhysParams P) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < G.n_faces) {
    const int fp = G.fpad;
    const int PS = G.max_slots * fp;
    const double dt = S.scal[kScDt];
    const double dt_here = (STAGE == 1) ? dt / 2 : dt;
    const float dtf = (float)dt_here;
    const float gam = (float)P.gam;
    float w[kDim], src[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) w[k] = S.W32[k * fp + f];
    const F3 fcn32 = plane3f(G.fcn32, fp, f);
    const double acc0 = G.acc_src[f];
    source_f32(w, fcn32, (float)acc0, P, src);
    Acc acc[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      acc[k].hi = dtf * src[k];
      acc[k].lo = 0.f;
    }
    const int n = G.nslots[f];
    unsigned bits = 0;
    for (int j = 0; j < n; ++j) {
      const int s = j * fp + f;
      const int rv = G.rev[s];
      float uL[kDim], uR[kDim], F[kDim];
#pragma unroll
      for (int k = 0; k < kDim; ++k) {
        uL[k] = S.uplus32[k * PS + s];
        uR[k] = S.uplus32[k * PS + rv];
      }
      SlotGeomF g;
      g.ec = plane3f(G.ec, PS, s);
      g.en = plane3f(G.en, PS, s);
      g.nxr = plane3f(G.nxr, PS, s);
      bits |= flux_star(uL, uR, g, gam, P.solver, F);
      const float cf = dtf * G.coef[s];
#pragma unroll
      for (int k = 0; k < kDim; ++k) {
        if (isnan(F[k])) bits |= 1u;
        acc[k].add(-cf * F[k]);
      }
    }
    if (bits) atomicOr(S.err, bits);
    // the compensated FP32 sum is rounded once to FP32 (an increment of
    // dt * Phi, small against U) and added to the FP64 state; U0 stays in
    // S.U until stage 2 overwrites it
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) u[k] = S.U[k * fp + f] + (double)(acc[k].hi + acc[k].lo);
    if (P.accretion_on) u[0] += dt_here * acc0;  // accretion mass source in FP64
    if (u[0] < 1e-8) u[0] = 1e-8;
    const f64::D3 r = plane3d(G.fcn, fp, f);
    double v2, inv_rho;
    const double p = pressure_recover(u, r, P.gam, v2, inv_rho);
    store_w32(S.W32, fp, f, u, p);
    if (STAGE == 2) {
#pragma unroll
      for (int k = 0; k < kDim; ++k) S.U[k * fp + f] = u[k];
      dt_candidates_sq(u, r, G.area[f], p, v2, inv_rho, P, vmax, dmin, sums);
    }
  }
  if (STAGE == 2)
    red::block_partials<kBlock>(vmax, dmin, sums, S.partial + (size_t)blockIdx.x * kPartialStride);
}

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace
}  // namespace mx

int mixed_partial_blocks(int n_faces) { return mx::blocks_for(n_faces); }

cudaError_t mixed_prepare(const DevGeomMixed& G, const DevState& S, const PhysParams& P,
                          cudaStream_t st) {
  mx::prepare_kernel<<<mx::blocks_for(G.n_faces), mx::kBlock, 0, st>>>(G, S, P);
  return cudaGetLastError();
}

cudaError_t mixed_step(const DevGeomMixed& G, const DevState& S, const PhysParams& P,
                       cudaStream_t st, cudaEvent_t* ev) {
  const int nb = mx::blocks_for(G.n_faces);
  if (ev) cudaEventRecord(ev[0], st);
  cudaError_t e = dt_reduce(S, P, nb, st, /*squared_speeds=*/true);
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[1], st);
  mx::reconstruct_kernel<<<nb, mx::kBlock, 0, st>>>(G, S, P);
  if (ev) cudaEventRecord(ev[2], st);
  mx::flux_update_kernel<1><<<nb, mx::kBlock, 0, st>>>(G, S, P);
  if (ev) cudaEventRecord(ev[3], st);
  mx::reconstruct_kernel<<<nb, mx::kBlock, 0, st>>>(G, S, P);
  if (ev) cudaEventRecord(ev[4], st);
  mx::flux_update_kernel<2><<<nb, mx::kBlock, 0, st>>>(G, S, P);
  if (ev) cudaEventRecord(ev[5], st);
  return cudaGetLastError();
}

}  // namespace splash
