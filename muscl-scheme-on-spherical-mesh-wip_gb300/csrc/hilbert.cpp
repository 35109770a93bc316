#include "hilbert.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <parallel/algorithm>
#endif

namespace splash {

uint64_t hilbert_key3(double x, double y, double z, int bits) {
  const double scale = (double)((1u << bits) - 1);
  uint32_t X[3];
  const double c[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    double t = (c[a] + 1.0) * 0.5;
    t = std::min(1.0, std::max(0.0, t));
    X[a] = (uint32_t)std::lround(t * scale);
  }
  // inverse undo of excess work (Skilling's AxestoTranspose)
  const uint32_t M = 1u << (bits - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;  // invert low bits of the first axis
      } else {
        const uint32_t t = (X[0] ^ X[i]) & P;  // exchange low bits
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  // Gray encode
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  // interleave the transposed index, most significant bit first
  uint64_t key = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> b) & 1u);
  return key;
}

std::vector<int> hilbert_order(const double* xyz, int n) {
  std::vector<uint64_t> key(n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const double* p = xyz + 3 * (size_t)i;
    const double r = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    key[i] = hilbert_key3(p[0] / r, p[1] / r, p[2] / r, 21);
  }
  // (key, index) pairs are distinct, so any sort of them gives the order of a
  // stable sort by key; the parallel sort of libstdc++ when OpenMP is on
  std::vector<std::pair<uint64_t, int>> kv(n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) kv[i] = {key[i], i};
#ifdef _OPENMP
  __gnu_parallel::sort(kv.begin(), kv.end());
#else
  std::sort(kv.begin(), kv.end());
#endif
  std::vector<int> order(n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) order[i] = kv[i].second;
  return order;
}

}  // namespace splash
