// Deterministic block reduction of the per-block partial records used by
// the dt clip and the diagnostics sums (shared by both precision paths).
#pragma once

#include "layout.hpp"

namespace splash {
namespace red {

// Warp + block reduction of one partial record; thread 0 of the block
// writes it.  Fixed tree order, so the result is deterministic.
template <int kBlock>
__device__ void block_partials(double vmax, double dmin, const double sums[5], double* out) {
  __shared__ double sm[kBlock / 32][7];
  double v[7] = {vmax, dmin, sums[0], sums[1], sums[2], sums[3], sums[4]};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double a = __shfl_down_sync(0xffffffffu, v[0], o);
    const double b = __shfl_down_sync(0xffffffffu, v[1], o);
    v[0] = fmax(v[0], a);
    v[1] = fmin(v[1], b);
#pragma unroll
    for (int k = 2; k < 7; ++k) v[k] = v[k] + __shfl_down_sync(0xffffffffu, v[k], o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 7; ++k) sm[warp][k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) r[k] = sm[0][k];
    for (int w = 1; w < kBlock / 32; ++w) {
      r[0] = fmax(r[0], sm[w][0]);
      r[1] = fmin(r[1], sm[w][1]);
#pragma unroll
      for (int k = 2; k < 7; ++k) r[k] = r[k] + sm[w][k];
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) out[k] = r[k];
  }
}

}  // namespace red
}  // namespace splash
