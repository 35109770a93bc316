// Host build of the Hilbert face ordering (csrc/hilbert.cpp) for the CPU
// test suite: the order it returns and the keys it sorts by.
#include <cstdint>
#include <vector>

#include "hilbert.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
void ho_order(const double* xyz, int n, int threads, int* out) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  const std::vector<int> o = splash::hilbert_order(xyz, n);
  for (int i = 0; i < n; ++i) out[i] = o[i];
}
uint64_t ho_key(double x, double y, double z, int bits) { return splash::hilbert_key3(x, y, z, bits); }
}
