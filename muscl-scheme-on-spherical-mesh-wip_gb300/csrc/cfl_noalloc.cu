// CFL time-step clip on caller-owned device buffers, without allocating.
//
// Some callers cannot allocate device memory at the point where they need
// the time step: a coupling code that owns every device allocation through
// its own pool (an allocation inside the library would bypass its
// accounting and its out-of-memory handling), or a caller that is about to
// capture its own stream into a CUDA graph and must not see a cudaMalloc
// inside the captured region.  splash_cfl_dt_noalloc serves them: it reads
// a conserved state that already lives on the device and writes the clipped
// dt, with the per-block partial records of the reduction kept in a
// file-scope __device__ array instead of a cudaMalloc'ed buffer.
//
// The array (kMaxBlocks records of kPartialStride doubles, 1 MiB) is
// part of the library image: every GPU that loads the library holds it until
// the process exits.  All calls share it, so calls that overlap on the GPU
// (different streams, different host threads) race on it.  Every call
// writes each record it later reads, so nothing needs clearing between
// calls.
//
// The kernels are the FP64 path's own per-face candidates and reduction
// (physics_fp64.cuh, reduce.cuh), and this file is compiled with the same
// -fmad=false as step_fp64.cu.  dt, max_vel and extra_dt are maxima and
// minima, exact in any order, so they equal what an FP64 adiabatic (dim 5)
// solver's splash_do_step computes for the same state; the five sums are
// reduced over 256-face blocks here and 64-face blocks in the solver, so
// they agree to rounding, not bit for bit.  A mixed-precision solver clips
// dt from FP32 candidates of its FP32 face state (within ~1e-7 relative of
// this value), and the isothermal (dim 4) state layout is not accepted.
#include <cuda_runtime.h>

#include <mutex>

#include "physics_fp64.cuh"
#include "reduce.cuh"
#include "solver.hpp"
#include "splash_gb300.h"

namespace splash {
namespace noalloc {
namespace {

constexpr int kBlock = 256;
constexpr int kMaxFaces = 4194304;  // 2^22 faces (icosphere_hex(10) would not fit)
constexpr int kMaxBlocks = kMaxFaces / kBlock;
constexpr int kMaxDevices = 64;

// the scratch: one partial record per block of the candidate kernel
__device__ __align__(256) double g_scratch[kMaxBlocks * kPartialStride];

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

__global__ void __launch_bounds__(kBlock) candidates_kernel(const double* __restrict__ U,
                                                            const double* __restrict__ r,
                                                            const double* __restrict__ area,
                                                            int n_faces, PhysParams P,
                                                            double* __restrict__ scratch) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0, dmin = 1e20, sums[5] = {0, 0, 0, 0, 0};
  if (f < n_faces) {
    double u[kDim];
#pragma unroll
    for (int k = 0; k < kDim; ++k) u[k] = U[(size_t)f * kDim + k];
    const f64::D3 rf{r[3 * (size_t)f], r[3 * (size_t)f + 1], r[3 * (size_t)f + 2]};
    f64::dt_candidates(u, rf, area[f], P, vmax, dmin, sums);
  }
  red::block_partials<kBlock>(vmax, dmin, sums, scratch + (size_t)blockIdx.x * kPartialStride);
}

// MUSCL_base.hpp:100-115 and physics/adiabatic.hpp:573-577
__global__ void __launch_bounds__(256) finalize_kernel(const double* __restrict__ scratch,
                                                       int nblocks, PhysParams P, double dt0,
                                                       double* __restrict__ out) {
  __shared__ double sm[256][7];
  double v[7] = {1e-8, 1e20, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double* p = scratch + (size_t)b * kPartialStride;
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
    double stop = 0.0;
    if (extra < 0) {
      stop = 1.0;
      extra = 1e20;
    }
    double dt = dt0;
    if (dt > P.h0 * 0.1 / max_vel) dt = P.h0 * 0.1 / max_vel;
    if (dt > extra) dt = extra;
    out[0] = dt;
    out[1] = max_vel;
    out[2] = extra;
    out[3] = stop;
#pragma unroll
    for (int k = 0; k < 5; ++k) out[4 + k] = sm[0][2 + k];
  }
}

}  // namespace
}  // namespace noalloc
}  // namespace splash

extern "C" int splash_cfl_dt_noalloc(const double* U, const double* unit_centres,
                                     const double* area, int n_faces, double gam, double omega_ns,
                                     double alpha, double h0, double dt0, double* out,
                                     void* stream) {
  using namespace splash;
  using namespace splash::noalloc;
  if (!U || !unit_centres || !area || !out)
    return set_error(SPLASH_E_INVALID, "splash_cfl_dt_noalloc: NULL device pointer");
  if (n_faces < 1 || n_faces > kMaxFaces)
    return set_error(SPLASH_E_INVALID,
                     "splash_cfl_dt_noalloc: n_faces=%d outside [1, %d] (the static scratch "
                     "holds %d block records)",
                     n_faces, kMaxFaces, kMaxBlocks);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_error(SPLASH_E_CUDA, "splash_cfl_dt_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(SPLASH_E_INVALID, "splash_cfl_dt_noalloc: device %d beyond %d", dev, kMaxDevices);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess)
    return set_error(SPLASH_E_CUDA, "splash_cfl_dt_noalloc: cudaStreamIsCapturing: %s",
                     cudaGetErrorString(e));
  double* scratch = nullptr;
  {
    // the device address of the static array (its host-side name is only a
    // stand-in), with this device current: looked up on every call made
    // outside stream capture (so that a context torn down and recreated,
    // e.g. by cudaDeviceReset, gets the reloaded image's address), and kept
    // per device for calls inside a capture, which reuse the last one
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || p == nullptr)
        return set_error(SPLASH_E_CUDA, "splash_cfl_dt_noalloc: cudaGetSymbolAddress: %s",
                         cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  PhysParams P{};
  P.gam = gam;
  P.omega_ns = omega_ns;
  P.alpha = alpha;
  P.h0 = h0;
  derive_params(P);
  const int nb = (n_faces + kBlock - 1) / kBlock;
  candidates_kernel<<<nb, kBlock, 0, st>>>(U, unit_centres, area, n_faces, P, scratch);
  finalize_kernel<<<1, 256, 0, st>>>(scratch, nb, P, dt0, out);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(SPLASH_E_CUDA, "splash_cfl_dt_noalloc: launch: %s", cudaGetErrorString(e));
  return SPLASH_OK;
}
