// Host build of the double-word arithmetic of the mixed update
// (csrc/dword.cuh) for the CPU test suite.
#include <cstdint>

#include "dword.cuh"

namespace {
splash::dw::DW to_dw(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
}  // namespace

extern "C" {
void dw_split(const double* x, float* h, float* l, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    const splash::dw::DW d = splash::dw::split(x[i]);
    h[i] = d.h;
    l[i] = d.l;
  }
}
// u [n][5] FP64 states, r [n][3] FP64 unit centres, w [n][5] FP32 face states
void dw_face_state(const double* u, const double* r, double gam_m1, float* w, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    const splash::dw::DW rd[3] = {to_dw(r[3 * i]), to_dw(r[3 * i + 1]), to_dw(r[3 * i + 2])};
    splash::dw::face_state_dw(u + 5 * i, rd, to_dw(gam_m1), w + 5 * i);
  }
}
}
