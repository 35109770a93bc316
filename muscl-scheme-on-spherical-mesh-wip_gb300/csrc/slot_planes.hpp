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

// FP32 planes of the mixed path.  The Riemann flux of an interior edge is
// evaluated once, in the orientation of its owner: of the edge's two slots
// the one with the smaller slot-plane index.  Edges are numbered in owner
// order; slot_edge maps every slot to its edge, with bit 31 set on the
// reverse (non-owner) side, whose flux is the owner's with the sign flipped
// (every Riemann solver here satisfies F(uR, uL, -n) = -F(uL, uR, n)).
struct MixedPlanes {
  std::vector<float> fcn32, beta, inv_h, bm, eta, arc, ec, en, coef;
  // the reconstruction's constants of slot s as four interleaved values
  // (one 16-byte load each): stencil faces (a, b, c, d); (beta_plus 0, 1,
  // beta_minus 0, 1); (1/H_plus, 1/H_minus, BM_dist, arc/area);
  // (unit edge centre, H_plus/BM_dist); (edge normal, H_minus/BM_dist)
  std::vector<int> rc_sten;
  std::vector<float> rc_beta, rc_h, rc_ec, rc_en;
  int n_edges = 0, epad = 0;           // epad: n_edges rounded up to 32
  std::vector<int> e_own, e_nbr;       // [epad] slot-plane indices of the two sides
  std::vector<float> e_ec, e_en, e_nxr;  // 3 planes of epad: the owner slot's geometry
  std::vector<int> slot_edge;          // [max_slots * fpad]
};
MixedPlanes make_mixed_planes(const SlotPlanes& sp);

}  // namespace splash
