// Device-side diagnostics of a solver state: the per-step sums of
// MUSCL_base.hpp:187-214 (mass, angular momentum, energy, each weighted by
// the face area) and the light curves of physics/adiabatic.hpp:228-333, in
// one pass over the conserved state, so that a caller gets 9 numbers back
// instead of downloading the state.
//
// Light curves: for four observers (x axis, 45 degrees, +z, -z) the sum over
// the faces the observer sees of Pi * cos(alpha) * area.  Visibility and
// cos(alpha) depend on the geometry only and are precomputed on the host with
// the reference's expressions (one plane per observer, 0 where not visible);
// the device evaluates Pi per face and the products in the reference order
// (Pi * cos) * area.  The sums are reduced in a fixed tree order (per-block
// partials, then one block), so the result is deterministic; it differs from
// the reference's serial sum only by summation order.
//
// Compiled with -fmad=false like the FP64 step.
#include <cuda_runtime.h>

#include "diagnostics.hpp"
#include "physics_fp64.cuh"

namespace splash {
namespace diag {
namespace {

constexpr int kBlock = 256;
constexpr int kVals = 9;

__device__ __forceinline__ double pressure_of(const double* u, double rx, double ry, double rz, double gam) {
  // vel = cross(r, l) / (-Sigma) ; Pi = max(1e-16, (E - Sigma |v|^2 / 2)(gam - 1))
  const double cx = ry * u[3] - rz * u[2], cy = rz * u[1] - rx * u[3], cz = rx * u[2] - ry * u[1];
  const double vx = cx / (-u[0]), vy = cy / (-u[0]), vz = cz / (-u[0]);
  double s = vx * vx;
  s = s + vy * vy;
  s = s + vz * vz;
  const double n = sqrt(s);
  return f64::smax(1e-16, (u[4] - u[0] * (n * n) / 2) * (gam - 1));
}

__global__ void __launch_bounds__(kBlock) partials_kernel(DiagInput in, double* __restrict__ partial) {
  __shared__ double sm[kVals][kBlock];
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double v[kVals] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (f < in.n_faces) {
    const int fp = in.fpad;
    double u[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) u[k] = (k < in.dim) ? in.U[(size_t)k * fp + f] : 0.0;
    const double a = in.area[f];
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = u[k] * a;
    if (in.light_curves) {
      const double PI = pressure_of(u, in.fcn[f], in.fcn[fp + f], in.fcn[2 * (size_t)fp + f], in.gam);
#pragma unroll
      for (int o = 0; o < 4; ++o) {
        const double c = in.cos_obs[(size_t)o * fp + f];
        if (c != 0.0) v[5 + o] = PI * c * a;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kVals; ++k) sm[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int h = kBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
#pragma unroll
      for (int k = 0; k < kVals; ++k) sm[k][threadIdx.x] = sm[k][threadIdx.x] + sm[k][threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x < kVals) partial[(size_t)blockIdx.x * kVals + threadIdx.x] = sm[threadIdx.x][0];
}

__global__ void __launch_bounds__(kBlock) final_kernel(const double* __restrict__ partial, int nblocks,
                                                       double* __restrict__ out) {
  __shared__ double sm[kVals][kBlock];
  double v[kVals] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += kBlock) {
#pragma unroll
    for (int k = 0; k < kVals; ++k) v[k] = v[k] + partial[(size_t)b * kVals + k];
  }
#pragma unroll
  for (int k = 0; k < kVals; ++k) sm[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int h = kBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
#pragma unroll
      for (int k = 0; k < kVals; ++k) sm[k][threadIdx.x] = sm[k][threadIdx.x] + sm[k][threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x < kVals) out[threadIdx.x] = sm[threadIdx.x][0];
}

}  // namespace
}  // namespace diag

int diag_partial_blocks(int n_faces) { return (n_faces + diag::kBlock - 1) / diag::kBlock; }

cudaError_t diag_launch(const DiagInput& in, double* partial, double* out, cudaStream_t st) {
  const int nb = diag_partial_blocks(in.n_faces);
  diag::partials_kernel<<<nb, diag::kBlock, 0, st>>>(in, partial);
  diag::final_kernel<<<1, diag::kBlock, 0, st>>>(partial, nb, out);
  return cudaGetLastError();
}

}  // namespace splash
