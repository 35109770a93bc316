// FP32/FP64 mixed-precision kernels (not built yet).
#include "solver.hpp"

namespace splash {
bool mixed_available() { return false; }
}  // namespace splash
