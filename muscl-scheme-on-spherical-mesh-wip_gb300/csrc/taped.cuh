// A scalar that records or replays the outcomes of its comparisons.
//
// The discrete adjoint differentiates the FP64 step with every branch fixed
// at the one the forward run took (limiter cases and min/max arguments,
// Riemann-solver sides, wave-speed fallbacks, floors).  Central differences
// of the step itself cross those branches wherever a perturbation moves a
// limiter ratio or a wave speed across a switch, so they measure the
// kinks as well as the derivative.  Taped evaluates the same per-face
// bodies (step_body_fp64.cuh) with plain double arithmetic, but every
// comparison, is_nan and is_inf of a Taped value goes through a tape:
//   record  the outcome is computed from the values and appended;
//   replay  the outcome is read back from the tape of a recorded run.
// A forward run recorded at x and replayed at x +- h d evaluates the
// branch-frozen map whose derivative the adjoint computes, so its central
// differences converge to the adjoint's directional derivative.
//
// Each thread of a launch (one face) owns a slice of kTapeWords 32-bit
// words of the launch's tape region (outcome bits, the last word holds how
// many were recorded) and a bit position in pos[face]; the region, the
// position array and the mode are in the __constant__ TapeCfg that the host
// updates before every launch (stream-ordered; a recorded region starts
// zeroed).  A thread whose comparisons would run past its slice sets
// kTapeOverflow in err and compares on values from then on; a replay that
// asks for more outcomes than were recorded sets kTapeMismatch.  A replay
// also counts in *flips the outcomes whose own values would have decided
// otherwise: the branch switches (limiter kinks, wave-speed sides, floors)
// that the perturbation crossed and the frozen map ignores; once a replayed
// branch leads a formula outside its domain (NaN) every later comparison
// involving it counts too.  The compare mode runs the plain step and counts
// the faces per launch whose branch path departs from the recording: the
// kink crossings between the recorded point and the compared one.  Validation
// only: every comparison is a read-modify-write of the thread's own global
// words.
#pragma once

#include <cmath>
#include <cstdint>

#include "dual.cuh"

namespace splash {
namespace tape {

constexpr int kTapeWords = 16;                      // per face and launch
constexpr uint32_t kCapacity = 32 * (kTapeWords - 1);  // 480 outcomes
constexpr unsigned kTapeOverflow = 1u;
constexpr unsigned kTapeMismatch = 2u;

// mode: kRecord appends the outcomes; kReplay takes them from the tape and
// counts in *flips the outcomes whose own values would have decided
// otherwise; kCompare decides on the values (the plain step) and counts in
// *flips the faces whose sequence of outcomes in this launch departs from
// the recorded one (the first departure of a face ends its comparison: the
// branch taken there changes which decisions follow).
constexpr int kRecord = 0, kReplay = 1, kCompare = 2;
constexpr uint32_t kDeparted = 0x80000000u;  // pos[] flag of a face that departed (kCompare)

struct TapeCfg {
  uint32_t* words;  // this launch's region: [n_faces][kTapeWords]
  uint32_t* pos;    // [n_faces] next outcome index, zeroed before the launch
  unsigned* err;
  unsigned long long* flips;
  int mode;
};

}  // namespace tape
}  // namespace splash

#if defined(__CUDACC__)
namespace splash {
namespace tape {
__constant__ TapeCfg g_tape;

__device__ __forceinline__ bool outcome(bool value_outcome) {
  const TapeCfg& c = g_tape;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t* slice = c.words + (size_t)f * kTapeWords;
  const uint32_t p = c.pos[f];
  if (c.mode == kCompare) {
    if (p & kDeparted) return value_outcome;
    const bool recorded = p < slice[kTapeWords - 1] && p < kCapacity && (slice[p >> 5] & (1u << (p & 31))) != 0;
    if (p >= slice[kTapeWords - 1] || recorded != value_outcome) {
      c.pos[f] = kDeparted;
      atomicAdd(c.flips, 1ull);
    } else {
      c.pos[f] = p + 1;
    }
    return value_outcome;
  }
  if (p >= kCapacity) {
    atomicOr(c.err, kTapeOverflow);
    return value_outcome;
  }
  c.pos[f] = p + 1;
  uint32_t* w = slice + (p >> 5);
  const uint32_t bit = 1u << (p & 31);
  if (c.mode == kReplay) {
    if (p >= slice[kTapeWords - 1]) atomicOr(c.err, kTapeMismatch);
    const bool recorded = (*w & bit) != 0;
    if (recorded != value_outcome) atomicAdd(c.flips, 1ull);
    return recorded;
  }
  if (value_outcome) *w |= bit;
  slice[kTapeWords - 1] = p + 1;
  return value_outcome;
}
}  // namespace tape

struct Taped {
  double v;
  SPLASH_HD Taped() : v(0.0) {}
  SPLASH_HD Taped(double x) : v(x) {}  // NOLINT: constants promote
};

SPLASH_HD double val(const Taped& x) { return x.v; }

#define SPLASH_TAPED_BIN(op)                                                                  \
  SPLASH_HD Taped operator op(const Taped& a, const Taped& b) { return Taped(a.v op b.v); } \
  SPLASH_HD Taped operator op(const Taped& a, double b) { return Taped(a.v op b); }         \
  SPLASH_HD Taped operator op(double a, const Taped& b) { return Taped(a op b.v); }
SPLASH_TAPED_BIN(+)
SPLASH_TAPED_BIN(-)
SPLASH_TAPED_BIN(*)
SPLASH_TAPED_BIN(/)
#undef SPLASH_TAPED_BIN
SPLASH_HD Taped operator-(const Taped& a) { return Taped(-a.v); }
SPLASH_HD Taped& operator+=(Taped& a, const Taped& b) { return a = a + b; }
SPLASH_HD Taped& operator-=(Taped& a, const Taped& b) { return a = a - b; }

#define SPLASH_TAPED_CMP(op)                                                                                     \
  __device__ __forceinline__ bool operator op(const Taped& a, const Taped& b) { return tape::outcome(a.v op b.v); } \
  __device__ __forceinline__ bool operator op(const Taped& a, double b) { return tape::outcome(a.v op b); }         \
  __device__ __forceinline__ bool operator op(double a, const Taped& b) { return tape::outcome(a op b.v); }
SPLASH_TAPED_CMP(<)
SPLASH_TAPED_CMP(>)
SPLASH_TAPED_CMP(<=)
SPLASH_TAPED_CMP(>=)
#undef SPLASH_TAPED_CMP

__device__ __forceinline__ bool is_nan(const Taped& a) { return tape::outcome(::isnan(a.v)); }
__device__ __forceinline__ bool is_inf(const Taped& a) { return tape::outcome(::isinf(a.v)); }

__device__ __forceinline__ Taped sqrt(const Taped& a) { return Taped(::sqrt(a.v)); }
__device__ __forceinline__ Taped exp(const Taped& a) { return Taped(::exp(a.v)); }
__device__ __forceinline__ Taped expm1(const Taped& a) { return Taped(::expm1(a.v)); }
__device__ __forceinline__ Taped log(const Taped& a) { return Taped(::log(a.v)); }

}  // namespace splash
#endif
