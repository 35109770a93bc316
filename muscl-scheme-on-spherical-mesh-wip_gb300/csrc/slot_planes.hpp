// Host-side preparation of the device layout (see layout.hpp): the Hilbert
// renumbering and every per-face / per-slot constant of the time step,
// evaluated once with the reference's own expressions.
#pragma once

#include <cstdint>
#include <vector>

#include "geometry.hpp"
#include "splash_gb300.h"

namespace splash {

struct SlotPlanes {
  int n_faces = 0, fpad = 0, max_slots = 0;
  std::vector<int> perm, iperm;  // perm[internal] = reference face
  // per face [fpad]
  std::vector<int8_t> nslots;
  std::vector<double> fcn;   // 3 planes
  std::vector<double> area;
  // per slot [max_slots * fpad] (x planes)
  std::vector<int> sten;     // 4 planes, internal ids
  std::vector<int> rev;      // slot-plane index of the reverse slot
  std::vector<double> beta;  // 4 planes
  std::vector<double> hpm;   // 2 planes
  std::vector<double> bm, eta /*2 planes*/, arc, ec /*3*/, ecn, en /*3*/, nxr /*3*/, chord;
  double round_diff = 0.0;
  size_t PS() const { return (size_t)max_slots * fpad; }
};

SlotPlanes make_slot_planes(const RefGeometry& g);

// area_coeff of physics/adiabatic.hpp:70-84 (loop counter starting at 0)
double area_coefficient(const RefGeometry& g, double acc_width);

// Accretion mass source res[0] of physics/adiabatic.hpp:428-436 per internal
// face (zeros when accretion is off): a function of geometry and parameters
// only, so it is evaluated once on the host.
std::vector<double> accretion_source(const SlotPlanes& sp, const splash_params& par,
                                     double area_coeff, bool accretion_on);

// The same profile from the unit face centres alone (3 planes of fpad),
// and its partial derivatives with respect to accretion_rate and
// tilt_angle (d_rate, d_tilt; the adjoint's parameter gradients).
std::vector<double> accretion_source_fcn(const std::vector<double>& fcn, int n_faces, int fpad,
                                         const splash_params& par, double area_coeff, bool accretion_on,
                                         std::vector<double>* d_rate = nullptr,
                                         std::vector<double>* d_tilt = nullptr);

// FP32 planes of the mixed path.  The mixed step works per interior edge:
// one thread reconstructs the edge states of the edge's two slots (owner:
// the slot with the smaller slot-plane index; reverse: the other) and
// evaluates the Riemann flux once, in the owner's orientation.  Edges are
// numbered face-major; slot_edge maps every slot to its edge, with bit
// 31 set on the reverse side, whose flux is the owner's with the sign
// flipped (every Riemann solver here satisfies F(uR, uL, -n) = -F(uL, uR, n)).
// The two sides share the edge centre (the same two vertices) and have
// opposite normals (exactly, in the reference geometry), so the reverse
// slot is reconstructed with the owner's centre and the negated normal.
// Per-edge records hold four interleaved values (one 16-byte load each).
struct MixedPlanes {
  std::vector<float> fcn32, fcn_lo, coef;  // per face (nearest float, residual); per slot (slot planes)
  int n_edges = 0, epad = 0;           // epad: n_edges rounded up to 32
  std::vector<int> slot_edge;          // [max_slots * fpad]
  std::vector<int> e_ids;              // [epad][4]: f | n_f << 28, g | n_g << 28, bits of (n x R).z, 0
  std::vector<float> e_ec, e_en;       // [epad][4]: owner's unit edge centre | (n x R).x, normal | (n x R).y
  std::vector<int> e_sten;             // [2][epad][4]: stencil faces (plus pair, minus pair), owner then reverse
  std::vector<float> e_beta;           // [2][epad][4]: beta_plus 0, 1, beta_minus 0, 1
  std::vector<float> e_h;              // [2][epad][4]: 1/H_plus, 1/H_minus, BM_dist, arc/area
};
MixedPlanes make_mixed_planes(const SlotPlanes& sp);

}  // namespace splash
