// Host build of the integer FP32 <-> FP64 conversions of the mixed update
// (csrc/fp_convert.cuh) for the CPU test suite.
#include <cstdint>

#include "fp_convert.cuh"

extern "C" {
void conv_d2f(const double* x, float* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] = splash::fpc::d2f(x[i]);
}
void conv_f2d(const float* x, double* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] = splash::fpc::f2d(x[i]);
}
void conv_isnan(const double* x, int* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] = splash::fpc::is_nan_bits(x[i]) ? 1 : 0;
}
}
