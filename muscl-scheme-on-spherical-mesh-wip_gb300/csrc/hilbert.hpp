// Space-filling-curve renumbering of faces.
#pragma once

#include <cstdint>
#include <vector>

namespace splash {

// 3-D Hilbert index of a point of [-1, 1]^3 at `bits` bits per axis
// (bits <= 21), after J. Skilling, "Programming the Hilbert curve",
// AIP Conf. Proc. 707 (2004): axes -> transposed index -> interleave.
uint64_t hilbert_key3(double x, double y, double z, int bits);

// Order of `n` points (xyz interleaved) along the Hilbert curve, ties broken
// by index.  Returns order[new] = old.
std::vector<int> hilbert_order(const double* xyz, int n);

}  // namespace splash
