// Device-side diagnostics of a solver state (diagnostics.cu).
#pragma once

#include <cuda_runtime.h>

namespace splash {

struct DiagInput {
  int n_faces;
  int fpad;
  int dim;                // 5 (adiabatic) or 4 (isothermal: no energy, no light curves)
  const double* U;        // dim planes of fpad
  const double* fcn;      // unit face centres, 3 planes of fpad
  const double* area;     // [fpad]
  const double* cos_obs;  // 4 planes of fpad: cos(alpha) of each observer, 0 where not visible
  double gam;
  int light_curves;       // evaluate the light curves (adiabatic only)
};

// Per-block partial records needed by diag_launch.
int diag_partial_blocks(int n_faces);
// out (device, 9 doubles): sum Sigma A, sum l_x A, sum l_y A, sum l_z A,
// sum E A, then the light curves (observer 0, 45, 90, 180 degrees).
cudaError_t diag_launch(const DiagInput& in, double* partial, double* out, cudaStream_t st);

}  // namespace splash
