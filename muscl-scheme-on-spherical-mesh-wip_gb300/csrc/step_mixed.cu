// FP32/FP64 mixed-precision kernels of the MUSCL time step.
//
// One step is four launches: per stage an edge launch (reconstruction of
// both slots of every interior edge and one Riemann flux per edge; the
// stage-1 launch also clips the step's dt) and a per-face update launch.
// The batched (ensemble) launches add a dt finalize per step.  Work split:
//   FP32: slopes and limiter, edge states, Riemann fluxes, source terms,
//         the per-slot flux contributions, the dt candidates;
//   FP64: the conserved state U, the RK combine U0 + dt*Phi, the dt and
//         simulation time, and the accretion mass source;
//   double-word FP32 (FP32 pairs, dword.cuh): the pressure recovery
//         Pi = (E - |r x l|^2 / (2 Sigma)) (gam - 1);
//   compensated: the per-face sum of the FP32 contributions is carried as an
//         FP32 (hi, lo) pair and folded into FP64.
// W32 and W32b hold (Sigma, l, Pi) in FP32 of the stage-1 and stage-2 input
// states: the stage-1 update writes W32b, the stage-2 update W32, so the
// last stage-2 input survives the step (the writers recompute the edge
// states from it instead of every stage-2 launch storing them).
#include <cuda_runtime.h>

#include <cstdint>

#include "dword.cuh"
#include "fp_convert.cuh"
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
// slot bound of the mixed path: solvers and ensembles reject meshes with
// faces of more than 8 edges at creation
constexpr int kMaxFaceSlots = 8;

__device__ __forceinline__ F3 plane3f(const float* p, int stride, int i) {
  return F3{p[i], p[stride + i], p[2 * stride + i]};
}
// Programmatic dependent launch.  The step's kernels are launched with
// programmatic stream serialization: a kernel may start while its
// predecessor drains, loads what does not depend on it (stencil indices,
// geometry), then waits in griddep_wait() for the predecessor grid to
// complete and its writes to be visible.  Every read of state and every
// write comes after the wait, so no kernel overwrites what its predecessor
// is still reading.  Without a programmatic predecessor the wait returns at
// once.  launch_dependents lets the next kernel start as soon as every
// block of this one has begun.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }

// Two FP32 lanes per instruction (PTX .f32x2: round to nearest,
// flush-to-zero like the rest of this file); each lane rounds exactly as the
// scalar add / sub / mul.
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 A, B, D;\n\t"
      "mov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\t"
      "add.rn.ftz.f32x2 D, A, B;\n\tmov.b64 {%0, %1}, D;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 A, B, D;\n\t"
      "mov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\t"
      "sub.rn.ftz.f32x2 D, A, B;\n\tmov.b64 {%0, %1}, D;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 A, B, D;\n\t"
      "mov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\t"
      "mul.rn.ftz.f32x2 D, A, B;\n\tmov.b64 {%0, %1}, D;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

// Two compensated accumulators (Acc, physics_mixed.cuh) in the lanes of
// float2 values: the same TwoSum steps, one packed instruction for both.
struct Acc2 {
  float2 hi, lo;
  __device__ __forceinline__ void add(float2 x) {
    const float2 t = add2(hi, x);
    const float2 xx = sub2(t, hi);
    lo = add2(lo, add2(sub2(hi, sub2(t, xx)), sub2(x, xx)));
    hi = t;
  }
};

// Packed FP32 states (face states W32 and edge states uplus32): entry i of
// an n-entry array is a float4 (Sigma, l_x, l_y, l_z) at base + 4 i and Pi
// at base + 4 n + i, so a gather of one state is one 16-byte load (plus one
// for Pi; the isothermal solver needs none).
//
// State loads are ordinary (coherent) loads, never ld.global.nc: under
// programmatic dependent launch a kernel is resident while its predecessor
// still writes the state, and the non-coherent path is defined only for data
// that is read-only for the whole life of the kernel.  griddepcontrol.wait
// makes the predecessor's writes visible to ordinary loads.  (With __ldg
// here, batched runs of small meshes read stale face states.)  Only the
// geometry, which no kernel writes, goes through __ldg.
__device__ __forceinline__ float4 ld4(const float* base, int i) {
  return reinterpret_cast<const float4*>(base)[i];
}
__device__ __forceinline__ void ld5(const float* base, int n, int i, float* v) {
  const float4 a = ld4(base, i);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
  v[4] = base[4 * (size_t)n + i];
}
__device__ __forceinline__ void st5(float* base, int n, int i, const float* v) {
  reinterpret_cast<float4*>(base)[i] = make_float4(v[0], v[1], v[2], v[3]);
  base[4 * (size_t)n + i] = v[4];
}

// The min key holds the signed square of the extra dt; 1e40 = (1e20)^2 is
// the reference's initial extra dt (adiabatic.hpp:545) and the isothermal
// solver's only candidate (isothermal.hpp:262-267).
constexpr float kNoBound = __builtin_huge_valf();  // +inf: no extra-dt bound
// the initial max |v|^2, (1e-8)^2 (MUSCL_base.hpp:314) rounded to a float
constexpr float kMinVel2 = (float)1e-16;

// Order-preserving 32-bit keys of the FP32 dt candidates: unsigned
// comparison of the keys orders the values, so the dt clip's max and min
// are exact integer atomics (no FP64 work, independent of the reduction
// order).
__device__ __forceinline__ unsigned order_key(float x) {
  const unsigned b = __float_as_uint(x);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_value(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Warp-reduces the dt candidates (NaN ignored, like the reference's
// comparisons) and folds them into the global keys with one atomic each.
__device__ __forceinline__ void fold_candidates(float vmax2, float dmin, unsigned* keys) {
  unsigned kmax = isnan(vmax2) ? 0u : order_key(vmax2);
  unsigned kmin = isnan(dmin) ? ~0u : order_key(dmin);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned a = __shfl_down_sync(0xffffffffu, kmax, o);
    const unsigned b = __shfl_down_sync(0xffffffffu, kmin, o);
    kmax = a > kmax ? a : kmax;
    kmin = b < kmin ? b : kmin;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&keys[0], kmax);
    atomicMin(&keys[1], kmin);
  }
}

// The same for launches of kBlock threads: the warps' keys meet in shared
// memory and one atomic per key and block reaches the L2 (every warp folding
// into the same two addresses serialised at the L2: 2.2 us of the stage-2
// update on hex(7)).  All threads of the block must call it.  The batched
// launches keep the per-warp fold: their warps belong to different members,
// and a per-member fold within the block measured 1% slower.
__device__ __forceinline__ void fold_candidates_block(float vmax2, float dmin, unsigned* keys) {
  unsigned kmax = isnan(vmax2) ? 0u : order_key(vmax2);
  unsigned kmin = isnan(dmin) ? ~0u : order_key(dmin);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned a = __shfl_down_sync(0xffffffffu, kmax, o);
    const unsigned b = __shfl_down_sync(0xffffffffu, kmin, o);
    kmax = a > kmax ? a : kmax;
    kmin = b < kmin ? b : kmin;
  }
  __shared__ unsigned s_max[kBlock / 32], s_min[kBlock / 32];
  if ((threadIdx.x & 31) == 0) {
    s_max[threadIdx.x >> 5] = kmax;
    s_min[threadIdx.x >> 5] = kmin;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 1; w < kBlock / 32; ++w) {
      kmax = s_max[w] > kmax ? s_max[w] : kmax;
      kmin = s_min[w] < kmin ? s_min[w] : kmin;
    }
    atomicMax(&keys[0], kmax);
    atomicMin(&keys[1], kmin);
  }
}

// The FP32 face state (Sigma, l, Pi) of the FP64 state u of face f, stored
// to W32 and returned in w: (Sigma, l) rounded to the nearest float and the
// pressure recovery Pi = (E - |r x l|^2 / (2 Sigma)) (gam - 1), floored at
// 1e-16 (MUSCL_base.hpp:538).  Where the kinetic term cancels part of E
// (above E / 8: low density, fast flow) the recovery runs in double-word
// FP32 arithmetic (dword.cuh), accurate to the FP32 rounding of Pi down to
// kinetic energies within 1e-5 of E, instead of on the FP64 pipe (about 2
// lanes per SM per clock here); lo holds the FP32 residuals of the unit
// centre r32.  Below E / 8 the subtraction loses at most a factor 8/7, so
// plain FP32 gives Pi within about 2 units in the last place of its float
// (the rounding of E, a few ulp in the kinetic term, which enters at most
// 1/7 of the result, and two roundings; 2.1 ulp at worst on 10^6 states
// just below E / 8, 1.0 when the kinetic term is negligible): on hex(7) the
// same density L1 error against FP64 after 200 steps (6.0e-8) with both
// update launches at 12.3 us instead of 12.4 / 14.3 us.
__device__ __forceinline__ void store_face_state(float* W32, int fp, int f, const double* u, F3 r32, F3 lo,
                                                 const PhysParams& P, float* w) {
  w[0] = fpc::d2f(u[0]);
  w[1] = fpc::d2f(u[1]);
  w[2] = fpc::d2f(u[2]);
  w[3] = fpc::d2f(u[3]);
  const float E = fpc::d2f(u[4]);
  const F3 c = cross3(r32, f3(w[1], w[2], w[3]));
  const float ke = 0.5f * __fdividef(dot3(c, c), w[0]);
  if (ke <= 0.125f * E) {  // false for NaN operands (a zero density) and E < 0
    w[4] = fmaxf((E - ke) * P.gam_m1_h, 1e-16f);
  } else {
    const dw::DW r[3] = {{r32.x, lo.x}, {r32.y, lo.y}, {r32.z, lo.z}};
    dw::face_state_dw(u, r, dw::DW{P.gam_m1_h, P.gam_m1_l}, w);
  }
  st5(W32, fp, f, w);
}

// dt candidates in FP32 from the FP32 face state w = (Sigma, l, Pi) (the
// FP64 state and pressure rounded once) and the FP32 unit centre r: the CFL
// maximum over squared speeds max(|v|^2, gam Pi / Sigma), and
// extra_dt_constr (physics/adiabatic.hpp:543-580), d = A / (B |v - v0|) with
// A = 0.01 Pi, B = alpha k g_eff Sigma, k = gam3d / (2 gam3d - 1), reduced as
// the signed square sgn(B) A^2 / (B^2 |v - v0|^2) (x |x| is increasing, so
// the minimum is the same; the dt clip takes one square root).  The sign
// comes from B's sign bit, so zero denominators give the direct quotient's
// signed infinities; a bound past the FP32 range (d above ~1.8e19) reads as
// no bound, like the initial 1e20.  Both candidates carry FP32 rounding
// (~1e-7 relative), so the mixed path's dt follows the FP64 path's to that
// level when the clip is active.
__device__ __forceinline__ void dt_candidates_f32(const float* w, F3 r, const PhysParams& P, float& vmax2,
                                                  float& dmin_sq) {
  const float ir = __fdividef(1.0f, w[0]);
  const F3 c = cross3(r, f3(w[1], w[2], w[3]));
  const float v2 = dot3(c, c) * (ir * ir);
  const float vm = fmaxf(v2, P.gam_f * w[4] * ir);
  // v = (r x l) / (-Sigma) ; v0 = omega_ns z x r
  const float vx = -c.x * ir + P.omega_ns_f * r.y;
  const float vy = -c.y * ir - P.omega_ns_f * r.x;
  const float vz = -c.z * ir;
  const float d2 = vx * vx + vy * vy + vz * vz;
  const float g_eff = 0.217909f - v2;
  const float A = 0.01f * w[4];
  const float B = P.fric_ak_f * g_eff * w[0];
  const float q = (A * A) / ((B * B) * d2);
  vmax2 = vm;
  dmin_sq = signbit(B) ? -q : q;
}

// physics/adiabatic.hpp:396-541 in FP32, except the accretion mass source
// (a geometric constant kept in FP64 and added by the caller).  w[4] = Pi.
// Quotients are __fdividef like the edge path's (divisors: the floored
// Sigma and Pi, 1 + C with C >= 0, C above the switch value).
__device__ __forceinline__ void source_f32(const float* w, F3 fcn, float acc0, const PhysParams& P,
                                           float* res) {
#pragma unroll
  for (int i = 0; i < kDim; ++i) res[i] = 0.f;
  if (!P.accretion_on) return;
  const float gam = P.gam_f;
  const F3 vel = scal(cross3(fcn, f3(w[1], w[2], w[3])), __fdividef(-1.0f, w[0]));
  const F3 omega_acc = f3(P.omega_acc_f[0], P.omega_acc_f[1], P.omega_acc_f[2]);
  const F3 omxr = cross3(omega_acc, fcn);
  const F3 rxo = cross3(fcn, omxr);
  res[1] = acc0 * rxo.x;
  res[2] = acc0 * rxo.y;
  res[3] = acc0 * rxo.z;
  const F3 dvo = sub(omxr, vel);
  res[4] = acc0 * (P.e_acc_f + 0.5f * dot3(dvo, dvo));
  const F3 rxv = cross3(fcn, vel);
  const float v2 = dot3(vel, vel);
  if (!P.friction_on) {
    const float dmdt = P.depletion_f * w[0];
    res[0] += dmdt;
    res[1] += dmdt * rxv.x;
    res[2] += dmdt * rxv.y;
    res[3] += dmdt * rxv.z;
    res[4] += dmdt * (__fdividef(gam / (gam - 1.f) * w[4], w[0]) + 0.5f * v2);
  }
  const float GM = 0.217909f;
  const float g_eff = GM - v2;
  // C = 12/5 k_m Sigma/Pi (3/4 c_sigma g_eff Sigma)^(1/4); constants folded
  // so that no intermediate leaves the FP32 range
  const float k1 = (float)(12. / 5 * 1.6e-13);
  const float q = (float)(3. / 4 * 4.85e36) * 1e-36f;  // scaled by 1e-36, undone by 10^9 below
  const float C = __fdividef(k1 * w[0], w[4]) * (sqrtf(sqrtf(q * g_eff * w[0])) * 1e9f);
  const float beta_switch = 0.736194670678821f;
  const float C_switch = -1.f - 1.f / (beta_switch - 1.f);
  float beta;
  if (C <= C_switch) {
    beta = 1.f - __fdividef(1.f, 1.f + C);
  } else {
    const float x = __fdividef(2.f, C);
    const float x2 = x * x;
    beta = 1.f - x2 * x2;
  }
  const float beta_ceil = 1.f - 1e-8f, beta_floor = 1e-8f;
  if (beta < beta_floor || isnan(beta)) beta = beta_floor;
  if (beta > beta_ceil) beta = beta_ceil;
  res[4] -= g_eff / 3.4e6f * (1.f - beta);
  if (P.friction_on) {
    const float gam3d = 1.f / (2.f - gam);
    const float rho = __fdividef(gam3d / (2.f * gam3d - 1.f) * g_eff * w[0] * w[0], w[4]);
    const F3 vel0 = cross3(f3(0.f, 0.f, P.omega_ns_f), fcn);
    const F3 dv = sub(vel, vel0);
    const float dvn = norm3(dv);
    const float ar = P.alpha_f * rho * dvn;
    const F3 wr = scal(dv, -ar);
    const F3 l_fr = cross3(fcn, wr);
    res[1] += l_fr.x;
    res[2] += l_fr.y;
    res[3] += l_fr.z;
    res[4] += dot3(wr, vel0);
    res[0] -= ar;
    res[1] -= __fdividef(ar, w[0]) * w[1];
    res[2] -= __fdividef(ar, w[0]) * w[2];
    res[3] -= __fdividef(ar, w[0]) * w[3];
    res[4] -= ar * (0.5f * v2 + __fdividef(w[4] * gam, (gam - 1.f) * w[0]));
  }
}

// Isothermal state (4 fields): W32 is the state itself (field 4 unused) and
// the CFL candidate is max(|v|^2, a^2) with a = 1 (find_v_max with the
// isothermal sound speed); no extra constraint (isothermal.hpp:262-267).
__device__ __forceinline__ void iso_w32_candidates(const double* u, F3 r, float* W32, int fp, int f,
                                                   float& vmax2, float& dmin) {
  const float v[kDim] = {fpc::d2f(u[0]), fpc::d2f(u[1]), fpc::d2f(u[2]), fpc::d2f(u[3]), 0.f};
  st5(W32, fp, f, v);
  const float ir = 1.0f / v[0];
  const F3 c = cross3(r, f3(v[1], v[2], v[3]));
  vmax2 = fmaxf(dot3(c, c) * (ir * ir), 1.f);
  dmin = kNoBound;
}

// W32 and the dt candidates of the state u of internal face f
__device__ __forceinline__ void prepare_face(const DevGeomMixed& G, const DevState& S, const PhysParams& P, int f,
                                             const double* u, float& vmax, float& dmin) {
  const F3 r32 = plane3f(G.fcn32, G.fpad, f);
  if (P.solver == kSolverIsoHLLE) {
    iso_w32_candidates(u, r32, S.W32, G.fpad, f, vmax, dmin);
  } else {
    float w[kDim];
    store_face_state(S.W32, G.fpad, f, u, r32, plane3f(G.fcn_lo, G.fpad, f), P, w);
    dt_candidates_f32(w, r32, P, vmax, dmin);
  }
}

// W32 and the dt candidates of the current U for face f (all 32 lanes of a
// warp call it; lanes past the last face contribute neutral values).
__device__ __forceinline__ void prepare_body(const DevGeomMixed& G, const DevState& S,
                                             const PhysParams& P, int f) {
  float vmax = 0.f, dmin = kNoBound;
  if (f < G.n_faces) {
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) u[k] = S.U[k * G.fpad + f];
    prepare_face(G, S, P, f, u, vmax, dmin);
  }
  fold_candidates(vmax, dmin, S.keys);
}

// set_state of the mixed path in one pass: the block stages the caller's
// rows of kBlock consecutive reference faces (contiguous in the caller's
// [F][dim] array, possibly host memory read over the coherent link) through
// shared memory with one element per thread and load, so every warp load
// covers 256 contiguous bytes; then each thread stores its face's FP64
// state at the face's internal index and computes its W32 and dt candidates
// from registers (no second pass over U).
template <bool VEC>
__global__ void __launch_bounds__(kBlock) scatter_prepare_kernel(const double* __restrict__ aos,
                                                                 const int* __restrict__ iperm, DevGeomMixed G,
                                                                 DevState S, PhysParams P, int dim) {
  __shared__ __align__(16) double rows[kBlock * kDim];
  const int r0 = blockIdx.x * kBlock;
  const int nr = min(kBlock, G.n_faces - r0);
  const int ne = nr * dim;
  const double* src = aos + (size_t)r0 * dim;
  if (VEC) {
    // 16-byte accesses (the array and every block's first row are 16-byte
    // aligned: r0 * dim * 8 is a multiple of 16)
    for (int k = 2 * threadIdx.x; k + 1 < ne; k += 2 * kBlock)
      *reinterpret_cast<double2*>(rows + k) = *reinterpret_cast<const double2*>(src + k);
    if ((ne & 1) && threadIdx.x == 0) rows[ne - 1] = src[ne - 1];
  } else {
    for (int k = threadIdx.x; k < ne; k += kBlock) rows[k] = src[k];
  }
  __syncthreads();
  float vmax = 0.f, dmin = kNoBound;
  const int t = threadIdx.x;
  if (t < nr) {
    const int f = iperm[r0 + t];
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) {
      u[k] = (k < dim) ? rows[t * dim + k] : 0.0;
      S.U[(size_t)k * G.fpad + f] = u[k];
    }
    prepare_face(G, S, P, f, u, vmax, dmin);
  }
  fold_candidates_block(vmax, dmin, S.keys);
}

// initial keys: max |v|^2 starts at (1e-8)^2 (MUSCL_base.hpp:314) and the
// min extra-dt square at +inf, no bound, for which the clip takes the
// reference's initial 1e20 (adiabatic.hpp:545)
__global__ void reset_keys_kernel(unsigned* keys) {
  keys[0] = order_key(kMinVel2);
  keys[1] = order_key(kNoBound);
}

// dt = min(dt0, 0.1 h0 / max_vel, extra_dt) (MUSCL_base.hpp:100-115), time,
// and a fresh start for the keys the step's stage-2 launch will fold into.
// The step's dt from the two keys (the dt candidates folded by the previous
// stage-2 update or by set_state): dt = min(dt0, 0.1 h0 / max_vel, extra_dt)
// (MUSCL_base.hpp:100-115).  The candidates are FP32 values (see
// dt_candidates_f32), so the clip is evaluated in FP32 and only the chosen
// bound is widened to FP64.
struct StepDt {
  double dt, max_vel, extra;
  bool neg_extra;
};
__device__ __forceinline__ StepDt clip_dt(const unsigned* keys, const PhysParams& P, double dt0) {
  StepDt d;
  const float max_vel_f = sqrtf(key_value(keys[0]));
  d.max_vel = fpc::f2d(max_vel_f);
  d.extra = 1e20;
  if (keys[1] < order_key(kNoBound)) {
    const float xf = key_value(keys[1]);
    d.extra = fpc::f2d(xf < 0.f ? -sqrtf(-xf) : sqrtf(xf));
  }
  d.neg_extra = d.extra < 0;
  if (d.neg_extra) d.extra = 1e20;
  const double cfl = fpc::f2d(P.cfl_num_f / max_vel_f);
  d.dt = dt0;
  if (d.dt > cfl) d.dt = cfl;
  if (d.dt > d.extra) d.dt = d.extra;
  return d;
}

// (float) clip_dt(...).dt without FP64 instructions, for every thread of a
// launch, from dt0f = dt0 rounded to the nearest float (fpc::d2f): the
// bounds are FP32 values and rounding is monotone, so clipping the rounded
// dt0 by the FP32 bounds gives the rounded clipped dt (NaN bounds clip
// nothing in either form).
__device__ __forceinline__ float clip_dt_f32(const unsigned* keys, const PhysParams& P, float dt0f) {
  const unsigned k0 = keys[0], k1 = keys[1];
  const float max_vel_f = sqrtf(key_value(k0));
  float extra = 1e20f;
  if (k1 < order_key(kNoBound)) {
    const float xf = key_value(k1);
    extra = xf < 0.f ? -sqrtf(-xf) : sqrtf(xf);
    if (extra < 0.f) extra = 1e20f;
  }
  const float cfl = P.cfl_num_f / max_vel_f;
  float dt = dt0f;
  if (dt > cfl) dt = cfl;
  if (dt > extra) dt = extra;
  return dt;
}

// the step scalars of d: dt, dt/2 (FP64 and FP32), dt0, the bounds, time
__device__ __forceinline__ void publish_dt(const DevState& S, const StepDt& d, double dt0) {
  if (d.neg_extra) atomicOr(S.err, 8u);  // SPLASH_STOP_NEG_EXTRA_DT
  S.scal[kScDt] = d.dt;
  S.scal[kScDtHalf] = d.dt / 2;
  *reinterpret_cast<float2*>(S.scal + kScDtF) = make_float2((float)d.dt, (float)(d.dt / 2));
  S.scal[kScDt0] = dt0;
  S.scal[kScMaxVel] = d.max_vel;
  S.scal[kScExtraDt] = d.extra;
  S.scal[kScTime] = S.scal[kScTime] + d.dt;
}

// fresh keys for the next fold
__device__ __forceinline__ void restart_keys(unsigned* keys) {
  keys[0] = order_key(kMinVel2);
  keys[1] = order_key(kNoBound);
}

// One thread: dt, the scalars and fresh keys (the batched launches).
__device__ __forceinline__ void finalize_body(const DevState& S, const PhysParams& P, double dt0) {
  griddep_wait();
  publish_dt(S, clip_dt(S.keys, P, dt0), dt0);
  restart_keys(S.keys);
}

// find_U_edges (MUSCL_base.hpp:361-434) in FP32 for one slot: the edge
// state (Sigma, l, Pi) of face f (n edges) across the slot's edge, from the
// face, its four stencil faces and the slot's constants.  Edge field 4 stays
// Pi; the isothermal solver leaves it 0.
struct SlotConsts {
  int4 st;    // stencil faces: plus pair, minus pair
  float4 bt;  // beta_plus 0, 1, beta_minus 0, 1
  float4 hh;  // 1/H_plus, 1/H_minus, BM_dist, arc/area
  float eta_p, eta_m;
};

__device__ __forceinline__ void recon_slot(const float* W, int fp, int f, int n, const SlotConsts& sc, F3 ec,
                                           F3 en, float dt, const PhysParams& P, float* up) {
  const int ia = sc.st.x, ib = sc.st.y, ic = sc.st.z, id = sc.st.w;
  const float bp0 = sc.bt.x, bp1 = sc.bt.y, bm0 = sc.bt.z, bm1 = sc.bt.w;
  const float ihp = sc.hh.x, ihm = sc.hh.y, bmd = sc.hh.z, arc_a = sc.hh.w;
  // the face and its four stencil faces: one 16-byte gather each for
  // (Sigma, l), one more each for Pi (adiabatic only)
  const float4 w4 = ld4(W, f), a4 = ld4(W, ia), b4 = ld4(W, ib), c4 = ld4(W, ic), d4 = ld4(W, id);
  const float w[4] = {w4.x, w4.y, w4.z, w4.w};
  const float wa[4] = {a4.x, a4.y, a4.z, a4.w}, wb[4] = {b4.x, b4.y, b4.z, b4.w};
  const float wc[4] = {c4.x, c4.y, c4.z, c4.w}, wd[4] = {d4.x, d4.y, d4.z, d4.w};
  if (P.solver == kSolverIsoHLLE) {
    // isothermal: 4 fields, superbee limiter with the Courant factor
    // (a + v.n) dt arc / area (physics/isothermal.hpp:269-320)
    const F3 vel = scal(cross3(ec, f3(w[1], w[2], w[3])), __fdividef(-1.0f, w[0]));
    const float nu_plus = (1.f + dot3(vel, en)) * dt * arc_a;
    const float eta = sc.eta_m;
    const float sb_scale = __fdividef(eta * 2.f, (float)(2 * n) * nu_plus);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float pp = (bp0 * wa[k] + bp1 * wb[k] - w[k]) * ihp;
      const float pm = (w[k] - (bm0 * wc[k] + bm1 * wd[k])) * ihm;
      const float lim = iso_limiter_field(__fdividef(pm, pp), eta, sb_scale);
      up[k] = w[k] + pp * lim * bmd;
    }
    up[4] = 0.f;
    return;
  }
  const float* Wp = W + 4 * (size_t)fp;
  const float wp = Wp[f];
  const float gam = P.gam_f;
  const float inv_rho = __fdividef(-1.0f, w[0]);
  const float c = sqrtf(__fdividef(gam * wp, w[0]));
  const F3 vel = scal(cross3(ec, f3(w[1], w[2], w[3])), inv_rho);
  const float nu_plus = (c + dot3(vel, en)) * dt * arc_a;
  const float sb_scale = __fdividef(sc.eta_m, (float)(2 * n) * nu_plus);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float pp = (bp0 * wa[k] + bp1 * wb[k] - w[k]) * ihp;
    const float pm = (w[k] - (bm0 * wc[k] + bm1 * wd[k])) * ihm;
    const float lim = limiter_field(__fdividef(pm, pp), nu_plus, sc.eta_p, sb_scale);
    up[k] = w[k] + pp * lim * bmd;
  }
  {
    const float pp = (bp0 * Wp[ia] + bp1 * Wp[ib] - wp) * ihp;
    const float pm = (wp - (bm0 * Wp[ic] + bm1 * Wp[id])) * ihm;
    const float lim = limiter_field(__fdividef(pm, pp), nu_plus, sc.eta_p, sb_scale);
    up[4] = wp + pp * lim * bmd;
  }
}

// One stage's reconstruction and Riemann fluxes, one thread per interior
// edge (find_U_edges + find_flux_var, MUSCL_base.hpp:361-434, 345-359): the
// edge states of the owner slot (face f) and of the reverse slot (face g,
// same edge centre, negated normal), then the flux once in the owner's
// orientation (the reverse side takes it negated in the update).  The
// reference evaluates the flux from both faces; every solver here satisfies
// F(uR, uL, -n) = -F(uL, uR, n), so each edge moves exactly what it removes
// from its neighbour.  The edge states never go to memory, except in stage 2
// when the state has an edge-state buffer (edge-major, for the writers that
// read the last stage's edge states; batched instances have none).
// Stop bits are folded per warp.  With OWN_DT (the stage-1 launch of one
// solver) every thread clips its step's dt from the keys itself and the
// first thread publishes the step scalars; otherwise dt comes from the
// scalars.
// The record of interior edge e (edge centre, normal, n x R, both faces and
// both slots' stencils, weights and distances) and the slots' limiter
// constants H+/BM and H-/BM = 1 / ((1/H) BM).
struct EdgeRec {
  int4 ids;
  SlotGeomF g;
  SlotConsts so, sr;
};
// Edge-record loads: read-only for the life of the program (ld.global.nc)
// and not allocated in L1 (.L1::no_allocate).  Each record is read once per
// stage, so caching it only evicts the face states that neighbouring edges'
// stencil gathers reuse from L1: measured on hex(7), per step 0.0741 ->
// 0.0705 ms flushed (0.0733 with .nc alone; L2 eviction-priority hints
// keeping the records from stage 1 to stage 2 gave 0.0716).
__device__ __forceinline__ int4 ld_rec_i4(const int* base, size_t i) {
  int4 v;
  asm("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(base + 4 * i));
  return v;
}
__device__ __forceinline__ float4 ld_rec_f4(const float* base, size_t i) {
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(base + 4 * i));
  return v;
}
__device__ __forceinline__ void load_edge(const DevGeomMixed& G, int e, bool live, EdgeRec& r) {
  float4 ce = make_float4(0.f, 0.f, 0.f, 0.f), ne = ce;
  r.ids = make_int4(0, 0, 0, 0);
  r.so = SlotConsts{};
  r.sr = SlotConsts{};
  if (live) {
    const size_t ep = (size_t)G.epad;
    r.ids = ld_rec_i4(G.e_ids, e);
    ce = ld_rec_f4(G.e_ec, e);
    ne = ld_rec_f4(G.e_en, e);
    r.so.st = ld_rec_i4(G.e_sten, e);
    r.so.bt = ld_rec_f4(G.e_beta, e);
    r.so.hh = ld_rec_f4(G.e_h, e);
    // the reverse slot's constants are loaded once the owner slot's edge
    // state is done (recon_edge); their lines are fetched into L2 now
    asm volatile("prefetch.global.L2 [%0];" ::"l"(G.e_sten + 4 * (ep + e)));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(G.e_beta + 4 * (ep + e)));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(G.e_h + 4 * (ep + e)));
  }
  r.so.eta_p = __fdividef(1.0f, r.so.hh.x * r.so.hh.z);
  r.so.eta_m = __fdividef(1.0f, r.so.hh.y * r.so.hh.z);
  r.g.ec = f3(ce.x, ce.y, ce.z);
  r.g.en = f3(ne.x, ne.y, ne.z);
  r.g.nxr = f3(ce.w, ne.w, __int_as_float(r.ids.z));
}

// The reverse slot's record entries, loaded after the owner slot's edge
// state: volatile with a memory clobber, so that neither the compiler nor
// the barrier before them moves them up into the owner slot, where they
// would hold 14 registers through its reconstruction (measured on hex(7):
// 72 registers with a 16-byte spill at 7 blocks per SM before; 64 without
// a spill at 8 blocks per SM after, 0.0704 -> 0.0667 ms per step flushed).
__device__ __forceinline__ int4 ld_rec_i4_late(const int* base, size_t i) {
  int4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(base + 4 * i)
               : "memory");
  return v;
}
__device__ __forceinline__ float4 ld_rec_f4_late(const float* base, size_t i) {
  float4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(base + 4 * i)
               : "memory");
  return v;
}

// the edge states of both slots of edge e from the face states W: the
// owner slot (face f) and the reverse slot (face g, negated normal).  PARK
// (blocks of at most kBlock threads): the owner slot's edge state waits in
// shared memory while the reverse slot is reconstructed (5 registers fewer
// at the peak: on hex(7) 0.0672 -> 0.0665 ms per step flushed)
template <bool PARK = false>
__device__ __forceinline__ void recon_edge(const float* W, const DevGeomMixed& G, const PhysParams& P, EdgeRec& r,
                                           int e, float dt, float* uL, float* uR) {
  recon_slot(W, G.fpad, r.ids.x & 0x0fffffff, r.ids.x >> 28, r.so, r.g.ec, r.g.en, dt, P, uL);
  __shared__ float park[PARK ? kDim : 1][PARK ? kBlock : 1];
  if (PARK) {
#pragma unroll
    for (int k = 0; k < kDim; ++k) park[k][threadIdx.x] = uL[k];
  }
  asm volatile("" ::: "memory");
  const size_t ep = (size_t)G.epad;
  r.sr.st = ld_rec_i4_late(G.e_sten, ep + e);
  r.sr.bt = ld_rec_f4_late(G.e_beta, ep + e);
  r.sr.hh = ld_rec_f4_late(G.e_h, ep + e);
  r.sr.eta_p = __fdividef(1.0f, r.sr.hh.x * r.sr.hh.z);
  r.sr.eta_m = __fdividef(1.0f, r.sr.hh.y * r.sr.hh.z);
  recon_slot(W, G.fpad, r.ids.y & 0x0fffffff, r.ids.y >> 28, r.sr, r.g.ec, f3(-r.g.en.x, -r.g.en.y, -r.g.en.z),
             dt, P, uR);
  if (PARK) {
    asm volatile("" ::: "memory");
#pragma unroll
    for (int k = 0; k < kDim; ++k) uL[k] = park[k][threadIdx.x];
  }
}

// The stage's input face states: W32 in stage 1 (written by set_state and
// the stage-2 update), W32b in stage 2 (written by the stage-1 update).
// Two buffers keep the stage-2 input until the next step's stage-1 update,
// so the last stage's edge states can be recomputed for the writers instead
// of being stored by every stage-2 edge launch.
template <int STAGE>
__device__ __forceinline__ const float* stage_input(const DevState& S) {
  return STAGE == 1 ? S.W32 : S.W32b;
}
// the next stage's input face states, written by the stage's update
template <int STAGE>
__device__ __forceinline__ float* stage_output(const DevState& S) {
  return STAGE == 1 ? S.W32b : S.W32;
}

// PARK: recon_edge parks the owner slot's edge state in shared memory (the
// single-solver edge launches; the batched ones measured 3% slower with it)
template <int STAGE, bool OWN_DT, bool PARK = false>
__device__ __forceinline__ void edge_body(const DevGeomMixed& G, const DevState& S, const PhysParams& P, int e,
                                          double dt0, float dt0f) {
  const bool live = e < G.n_edges;
  EdgeRec r;
  load_edge(G, e, live, r);
  griddep_wait();
  float dt;
  if (OWN_DT) {
    dt = clip_dt_f32(S.keys, P, dt0f);
    if (e == 0) publish_dt(S, clip_dt(S.keys, P, dt0), dt0);
  } else {
    dt = reinterpret_cast<const float2*>(S.scal + kScDtF)->x;
  }
  unsigned bits = 0;
  if (live) {
    float uL[kDim], uR[kDim], F[kDim] = {0.f, 0.f, 0.f, 0.f, 0.f};
    recon_edge<PARK>(stage_input<STAGE>(S), G, P, r, e, dt, uL, uR);
    bits = (P.solver == kSolverIsoHLLE) ? iso_flux_star(uL, uR, r.g, F)
                                        : flux_star(uL, uR, r.g, P.gam_f, P.solver, F);
#pragma unroll
    for (int k = 0; k < kDim; ++k)
      if (isnan(F[k])) bits |= 1u;
    st5(S.fe32, G.epad, e, F);
  }
  bits = __reduce_or_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && bits) atomicOr(S.err, bits);
}

// The last step's stage-2 edge states for the writers (write_t_curl): the
// stage-2 reconstruction of edge_body, from the stage-2 input W32b and the
// step's dt, into uplus32 (edge-major: the owner side of edge e at e, the
// reverse side at epad + e).
__global__ void __launch_bounds__(kBlock) edge_states_kernel(DevGeomMixed G, DevState S, PhysParams P) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= G.n_edges) return;
  EdgeRec r;
  load_edge(G, e, true, r);
  const float dt = reinterpret_cast<const float2*>(S.scal + kScDtF)->x;
  float uL[kDim], uR[kDim];
  recon_edge(stage_input<2>(S), G, P, r, e, dt, uL, uR);
  st5(S.uplus32, 2 * G.epad, e, uL);
  st5(S.uplus32, 2 * G.epad, G.epad + e, uR);
}

// at most 64 registers (8 blocks of 128 per SM, no spill; measured best of
// 7 to 9 blocks)
template <int STAGE>
__global__ void __launch_bounds__(kBlock, 8) edge_kernel(DevGeomMixed G, DevState S, PhysParams P, double dt0,
                                                         float dt0f) {
  griddep_launch_dependents();
  edge_body<STAGE, STAGE == 1, true>(G, S, P, blockIdx.x * blockDim.x + threadIdx.x, dt0, dt0f);
}

// res2d + RK combine (MUSCL_base.hpp:238-276, 124-161) of face f: the
// slot contributions -dt_here coef F (F the edge flux, negated on the
// reverse side) summed in slot order (Neumaier-compensated FP32), plus
// dt_here times the source in FP32 from the face state
// (physics/adiabatic.hpp:396-541), rounded once and added to the FP64 U0;
// the accretion mass source in FP64; the density floor, the pressure
// recovery (double-word FP32), the FP32 face state of the next stage, and in
// stage 2 the new U and the dt candidates.  Every lane of the calling warp
// must call it (the candidates fold per warp).
// BLOCK_FOLD: kBlock-thread launches of one solver; RESTART_KEYS: the
// stage-1 update of one solver gives the keys a fresh start (the stage-1
// edge launch that read them has completed); EARLY_STATE: the face's own
// FP32 and FP64 states are loaded right after the dependency wait, in
// flight with the flux gathers (one memory round trip less per thread, at
// more registers: for the one-wave launches of one solver)
template <int STAGE, int MAXS = kMaxFaceSlots, bool BLOCK_FOLD = false, bool RESTART_KEYS = false,
          bool EARLY_STATE = false>
__device__ __forceinline__ void update_body(const DevGeomMixed& G, const DevState& S, const PhysParams& P,
                                            int f) {
  const int fp = G.fpad;
  const bool live = f < G.n_faces;
  F3 fcn32 = f3(0.f, 0.f, 0.f), fcn_lo = f3(0.f, 0.f, 0.f);
  double acc0 = 0.0;
  int n = 0;
  // the slots' edges and flux coefficients: geometry, loaded before the wait
  int se[MAXS];
  float co[MAXS];
  if (live) {
    fcn32 = plane3f(G.fcn32, fp, f);
    acc0 = G.acc_src[f];
    if (P.solver != kSolverIsoHLLE) fcn_lo = plane3f(G.fcn_lo, fp, f);
    n = G.nslots[f];
  }
#pragma unroll
  for (int j = 0; j < MAXS; ++j) {
    se[j] = (j < n) ? G.slot_edge[j * fp + f] : 0;
    co[j] = (j < n) ? G.coef[j * fp + f] : 0.f;
  }
  griddep_wait();
  if (RESTART_KEYS && f == 0) restart_keys(S.keys);
  float vmax = 0.f, dmin = kNoBound;
  if (live) {
    float w[kDim];
    double u0[kDim];
    if (EARLY_STATE) {
      ld5(stage_input<STAGE>(S), fp, f, w);
#pragma unroll
      for (int k = 0; k < kDim; ++k) u0[k] = S.U[k * fp + f];
    }
    const float2 dtf2 = *reinterpret_cast<const float2*>(S.scal + kScDtF);
    const float dtf = (STAGE == 1) ? dtf2.y : dtf2.x;
    // fields 0-1 and 2-3 accumulate in packed pairs, field 4 alone
    Acc2 a01{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}, a23 = a01;
    Acc a4{0.f, 0.f};
    // unrolled over the slot bound so that every slot's gather is in flight
    // before the first is summed; the sum stays in slot order
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      if (j < n) {
        const float cf = dtf * co[j];
        // -cf F with F = Fe on the owner side and -Fe on the reverse side
        const float c = (se[j] < 0) ? cf : -cf;
        const int e = se[j] & 0x7fffffff;
        const float4 fe = ld4(S.fe32, e);
        const float fe4 = S.fe32[4 * (size_t)G.epad + e];
        const float2 c2 = make_float2(c, c);
        a01.add(mul2(c2, make_float2(fe.x, fe.y)));
        a23.add(mul2(c2, make_float2(fe.z, fe.w)));
        a4.add(c * fe4);
      }
    }
    const Acc acc[kDim] = {{a01.hi.x, a01.lo.x}, {a01.hi.y, a01.lo.y}, {a23.hi.x, a23.lo.x},
                           {a23.hi.y, a23.lo.y}, a4};
    float src[kDim];
    if (!EARLY_STATE) ld5(stage_input<STAGE>(S), fp, f, w);
    source_f32(w, fcn32, fpc::d2f(acc0), P, src);
    // the FP32 increment (flux sum + dt source, one rounding) is added to
    // the FP64 state; U0 stays in S.U until stage 2 overwrites it
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k)
      u[k] = (EARLY_STATE ? u0[k] : S.U[k * fp + f]) + fpc::f2d((acc[k].hi + acc[k].lo) + dtf * src[k]);
    if (P.accretion_on) {  // accretion mass source in FP64
      const double dt_here = S.scal[(STAGE == 1) ? kScDtHalf : kScDt];
      u[0] += dt_here * acc0;
    }
    if (u[0] < 1e-8) u[0] = 1e-8;
    if (P.solver == kSolverIsoHLLE) {
      u[4] = 0.0;
      float vm, dm;
      iso_w32_candidates(u, fcn32, stage_output<STAGE>(S), fp, f, vm, dm);
      if (STAGE == 2) {
#pragma unroll
        for (int k = 0; k < kDim; ++k) S.U[k * fp + f] = u[k];
        vmax = vm;
        dmin = dm;
      }
    } else {
      float w32[kDim];
      store_face_state(stage_output<STAGE>(S), fp, f, u, fcn32, fcn_lo, P, w32);
      if (STAGE == 2) {
#pragma unroll
        for (int k = 0; k < kDim; ++k) S.U[k * fp + f] = u[k];
        dt_candidates_f32(w32, fcn32, P, vmax, dmin);
      }
    }
  }
  if (STAGE == 2) {
    if (BLOCK_FOLD)
      fold_candidates_block(vmax, dmin, S.keys);
    else
      fold_candidates(vmax, dmin, S.keys);
  }
}

// MAXS: the mesh's largest face degree rounded up to 4, 6 or 8 (the slot
// loop is unrolled to it; slots past a face's own count are predicated off
// but still issued)
template <int STAGE, int MAXS>
__global__ void __launch_bounds__(kBlock) update_kernel(DevGeomMixed G, DevState S, PhysParams P) {
  griddep_launch_dependents();
  update_body<STAGE, MAXS, true, STAGE == 1>(G, S, P, blockIdx.x * blockDim.x + threadIdx.x);
}
// the same with the early state loads of update_body, at most 56 registers
// (9 blocks of 128 per SM; uncapped they take 63-72 registers and the
// hex(7) grid two waves, 1-4 us slower per launch)
template <int STAGE, int MAXS>
__global__ void __launch_bounds__(kBlock, 9) update_early_kernel(DevGeomMixed G, DevState S, PhysParams P) {
  griddep_launch_dependents();
  update_body<STAGE, MAXS, true, STAGE == 1, true>(G, S, P, blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------- ensemble
// Batched launches over many independent instances: every block looks up
// its (instance, first face) tile and runs the same bodies as a single
// solver, so each instance's arithmetic is exactly that of a standalone run.
__global__ void __launch_bounds__(32) ens_prepare_kernel(const EnsInstance* __restrict__ inst,
                                                         const int2* __restrict__ tiles) {
  const int2 t = tiles[blockIdx.x];
  const EnsInstance& I = inst[t.x];
  prepare_body(I.G, I.S, I.P, t.y + threadIdx.x);
}

__global__ void ens_reset_keys_kernel(const EnsInstance* __restrict__ inst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    inst[i].S.keys[0] = order_key(kMinVel2);
    inst[i].S.keys[1] = order_key(kNoBound);
  }
}

__global__ void ens_finalize_kernel(const EnsInstance* __restrict__ inst, int n, double dt0) {
  griddep_launch_dependents();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) finalize_body(inst[i].S, inst[i].P, dt0);
}

// reconstruction + edge fluxes: one 32-edge tile per warp (tiles hold
// (instance, first edge))
constexpr int kWarpTiles = kBlock / 32;
// at most 64 registers like the single-solver edge launch (blocks of at
// most 128 threads; 1% faster per ensemble step than 72 registers)
template <int STAGE>
__global__ void __launch_bounds__(kBlock, 8) ens_edge_kernel(const EnsInstance* __restrict__ inst,
                                                       const int2* __restrict__ tiles, int n_tiles) {
  griddep_launch_dependents();
  const int tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (tile >= n_tiles) return;  // whole warps: stop bits fold per warp
  const int2 t = tiles[tile];
  const EnsInstance& I = inst[t.x];
  edge_body<STAGE, false>(I.G, I.S, I.P, t.y + (threadIdx.x & 31), 0.0, 0.f);
}

// update: one 32-face tile per warp; MAXS as update_kernel, over every
// member's mesh
template <int STAGE, int MAXS>
__global__ void __launch_bounds__(kBlock) ens_update_kernel(const EnsInstance* __restrict__ inst,
                                                            const int2* __restrict__ tiles, int n_tiles) {
  griddep_launch_dependents();
  const int tile = blockIdx.x * kWarpTiles + (threadIdx.x >> 5);
  if (tile >= n_tiles) return;  // whole warps: the candidates fold per warp
  const int2 t = tiles[tile];
  const EnsInstance& I = inst[t.x];
  update_body<STAGE, MAXS>(I.G, I.S, I.P, t.y + (threadIdx.x & 31));
}

// ---- the ensemble as one persistent launch
// One cooperative launch runs n_steps steps of every member: per step the
// per-member dt clip, then edge and update of each stage, the phases
// separated by a grid-wide barrier instead of launch boundaries.  Every
// block is resident (the grid is sized to the occupancy), warps take the
// same (member, tile) pairs in the same order as the five-launch schedule
// and call the same bodies, so each member's arithmetic is that of a
// standalone solver.

// ld.acquire at GPU scope (the barrier's generation word)
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier: thread 0 of every block adds itself to bar[0]; the
// last to arrive restarts the count and advances the generation bar[1]; the
// others wait for the generation to move, at most kBarrierSpins polls of
// ~64 ns (about a quarter of a second, against phases of well under a
// millisecond), after which they set kEnsBarrierTimeout in *status and the
// launch returns early.  The GPU-scope fences around the arrival make every
// write of a phase visible to the loads of the next one, like a launch
// boundary.  All threads of the block call it; false when the wait ran out.
constexpr long long kBarrierSpins = 1ll << 22;
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned* status) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned gen = ld_acquire_gpu(bar + 1);
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (ld_acquire_gpu(bar + 1) == gen) {
        if (++spins > kBarrierSpins) {
          atomicOr(status, kEnsBarrierTimeout);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// at most 72 registers (7 blocks of 128 per SM)
__global__ void __launch_bounds__(kBlock, 7)
    ens_persistent_kernel(const EnsInstance* __restrict__ inst, int n_inst, const int2* __restrict__ ftiles,
                          int n_ftiles, const int2* __restrict__ etiles, int n_etiles, double dt0, int n_steps,
                          unsigned* bar, unsigned* status) {
  const int warps = gridDim.x * kWarpTiles;
  const int wid = blockIdx.x * kWarpTiles + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  for (int s = 0; s < n_steps; ++s) {
    // each member's dt from its keys, then fresh keys (the finalize launch)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += gridDim.x * blockDim.x) {
      publish_dt(inst[i].S, clip_dt(inst[i].S.keys, inst[i].P, dt0), dt0);
      restart_keys(inst[i].S.keys);
    }
    if (!grid_barrier(bar, status)) return;
    for (int t = wid; t < n_etiles; t += warps) {
      const int2 tt = etiles[t];
      const EnsInstance& I = inst[tt.x];
      edge_body<1, false>(I.G, I.S, I.P, tt.y + lane, 0.0, 0.f);
    }
    if (!grid_barrier(bar, status)) return;
    for (int t = wid; t < n_ftiles; t += warps) {
      const int2 tt = ftiles[t];
      const EnsInstance& I = inst[tt.x];
      update_body<1>(I.G, I.S, I.P, tt.y + lane);
    }
    if (!grid_barrier(bar, status)) return;
    for (int t = wid; t < n_etiles; t += warps) {
      const int2 tt = etiles[t];
      const EnsInstance& I = inst[tt.x];
      edge_body<2, false>(I.G, I.S, I.P, tt.y + lane, 0.0, 0.f);
    }
    if (!grid_barrier(bar, status)) return;
    for (int t = wid; t < n_ftiles; t += warps) {
      const int2 tt = ftiles[t];
      const EnsInstance& I = inst[tt.x];
      update_body<2>(I.G, I.S, I.P, tt.y + lane);
    }
    if (s + 1 < n_steps && !grid_barrier(bar, status)) return;
  }
}

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace
}  // namespace mx

const void* mixed_dt0_kernel_ptr() { return (const void*)mx::edge_kernel<1>; }

cudaError_t mixed_scatter_prepare(const double* aos, const int* iperm, const DevGeomMixed& G, const DevState& S,
                                  const PhysParams& P, int dim, cudaStream_t st) {
  mx::reset_keys_kernel<<<1, 1, 0, st>>>(S.keys);
  if (((uintptr_t)aos & 15) == 0)
    mx::scatter_prepare_kernel<true><<<mx::blocks_for(G.n_faces), mx::kBlock, 0, st>>>(aos, iperm, G, S, P, dim);
  else
    mx::scatter_prepare_kernel<false><<<mx::blocks_for(G.n_faces), mx::kBlock, 0, st>>>(aos, iperm, G, S, P, dim);
  return cudaGetLastError();
}

namespace {
// A launch with programmatic stream serialization (see griddep_wait).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
}  // namespace

cudaError_t mixed_step(const DevGeomMixed& G, const DevState& S, const PhysParams& P, double dt0,
                       cudaStream_t st, cudaEvent_t* ev, bool /*per_launch: four launches, same layout*/) {
  const dim3 egrid(mx::blocks_for(G.n_edges));
  const dim3 ugrid(mx::blocks_for(G.n_faces));
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  // ev[0]..ev[1] is the (empty) slot of the dt clip, which the stage-1 edge
  // launch evaluates itself
  if (ev) cudaEventRecord(ev[0], st);
  if (ev) cudaEventRecord(ev[1], st);
  const float dt0f = fpc::d2f(dt0);
  // The update variant: the early state loads for meshes of at most 6-gons
  // whose update grid nearly fills the GPU in one wave at 9 blocks per SM
  // (more than 6, at most 9 blocks per SM).  Measured per step against the
  // plain update: hex(7) (8.4 blocks per SM) 1.2% faster; hex(5) (0.5 per
  // SM) 2.5% slower back to back; hex(8) (34 per SM) 0.8% slower; hex(9)
  // equal; quad(7) with the 4-slot copy 3% slower (a larger spill).
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 0;
  const bool early = G.max_slots > 4 && G.max_slots <= 6 && (int)ugrid.x > 6 * sms && (int)ugrid.x <= 9 * sms;
  void (*upd1)(DevGeomMixed, DevState, PhysParams) = mx::update_kernel<1, 8>;
  void (*upd2)(DevGeomMixed, DevState, PhysParams) = mx::update_kernel<2, 8>;
  if (G.max_slots <= 4) {
    upd1 = mx::update_kernel<1, 4>;
    upd2 = mx::update_kernel<2, 4>;
  } else if (G.max_slots <= 6) {
    upd1 = early ? mx::update_early_kernel<1, 6> : mx::update_kernel<1, 6>;
    upd2 = early ? mx::update_early_kernel<2, 6> : mx::update_kernel<2, 6>;
  }
  chk(launch_pdl(mx::edge_kernel<1>, egrid, dim3(mx::kBlock), st, G, S, P, dt0, dt0f));
  if (ev) cudaEventRecord(ev[2], st);
  chk(launch_pdl(upd1, ugrid, dim3(mx::kBlock), st, G, S, P));
  if (ev) cudaEventRecord(ev[3], st);
  chk(launch_pdl(mx::edge_kernel<2>, egrid, dim3(mx::kBlock), st, G, S, P, dt0, dt0f));
  if (ev) cudaEventRecord(ev[4], st);
  chk(launch_pdl(upd2, ugrid, dim3(mx::kBlock), st, G, S, P));
  if (ev) cudaEventRecord(ev[5], st);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t ensemble_prepare(const EnsInstance* inst, int n_inst, const int2* ftiles, int n_ftiles,
                             cudaStream_t st) {
  mx::ens_reset_keys_kernel<<<(n_inst + 127) / 128, 128, 0, st>>>(inst, n_inst);
  mx::ens_prepare_kernel<<<n_ftiles, 32, 0, st>>>(inst, ftiles);
  return cudaGetLastError();
}

cudaError_t ensemble_step(const EnsInstance* inst, int n_inst, const int2* ftiles, int n_ftiles,
                          const int2* etiles, int n_etiles, int edge_block, int max_slots, double dt0,
                          cudaStream_t st) {
  const int wpb = edge_block / 32;
  const dim3 egrid((n_etiles + wpb - 1) / wpb);
  const dim3 ugrid((n_ftiles + mx::kWarpTiles - 1) / mx::kWarpTiles);
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  void (*upd1)(const EnsInstance*, const int2*, int) = mx::ens_update_kernel<1, 8>;
  void (*upd2)(const EnsInstance*, const int2*, int) = mx::ens_update_kernel<2, 8>;
  if (max_slots <= 4) {
    upd1 = mx::ens_update_kernel<1, 4>;
    upd2 = mx::ens_update_kernel<2, 4>;
  } else if (max_slots <= 6) {
    upd1 = mx::ens_update_kernel<1, 6>;
    upd2 = mx::ens_update_kernel<2, 6>;
  }
  chk(launch_pdl(mx::ens_finalize_kernel, dim3((n_inst + 127) / 128), dim3(128), st, inst, n_inst, dt0));
  chk(launch_pdl(mx::ens_edge_kernel<1>, egrid, dim3(edge_block), st, inst, etiles, n_etiles));
  chk(launch_pdl(upd1, ugrid, dim3(mx::kBlock), st, inst, ftiles, n_ftiles));
  chk(launch_pdl(mx::ens_edge_kernel<2>, egrid, dim3(edge_block), st, inst, etiles, n_etiles));
  chk(launch_pdl(upd2, ugrid, dim3(mx::kBlock), st, inst, ftiles, n_ftiles));
  return e != cudaSuccess ? e : cudaGetLastError();
}

const void* ensemble_finalize_kernel_ptr() { return (const void*)mx::ens_finalize_kernel; }

cudaError_t mixed_edge_states(const DevGeomMixed& G, const DevState& S, const PhysParams& P, cudaStream_t st) {
  mx::edge_states_kernel<<<mx::blocks_for(G.n_edges), mx::kBlock, 0, st>>>(G, S, P);
  return cudaGetLastError();
}

int ensemble_persistent_grid(int device) {
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mx::ens_persistent_kernel, mx::kBlock, 0) !=
      cudaSuccess)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  return per_sm * sms;
}

cudaError_t ensemble_persistent(const EnsInstance* inst, int n_inst, const int2* ftiles, int n_ftiles,
                                const int2* etiles, int n_etiles, double dt0, int n_steps, unsigned* bar,
                                unsigned* status, int grid, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(mx::kBlock);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, mx::ens_persistent_kernel, inst, n_inst, ftiles, n_ftiles, etiles, n_etiles,
                            dt0, n_steps, bar, status);
}

const void* ensemble_persistent_kernel_ptr() { return (const void*)mx::ens_persistent_kernel; }

}  // namespace splash
