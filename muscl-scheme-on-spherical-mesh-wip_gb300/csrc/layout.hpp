// Device-resident data layout of one solver instance.
//
// Faces are stored in an internal order (a Hilbert curve through the unit
// face centres) so that the neighbour gathers of a warp touch nearby memory.
// Per-face arrays have length `fpad` (n_faces rounded up to a multiple of 32).
// Per-slot arrays (one value per face edge) use "slot planes": the value of
// slot j of internal face f lives at index j * fpad + f, so a warp of
// consecutive faces reading slot j issues one coalesced access.  Faces with
// fewer than max_slots edges (the 12 pentagons of an icosphere_hex mesh)
// leave their last plane entries unused.
//
// Every geometric constant the time step needs is precomputed on the host
// with the reference's own expression (so the device never re-derives a
// transcendental of the geometry), converted to the slot-plane layout and
// uploaded once.
#pragma once

#include <cstdint>

namespace splash {

constexpr int kDim = 5;          // conserved fields: Sigma, l_x, l_y, l_z, E
constexpr int kMaxSlots = 6;     // hexagons (pentagons and quads use fewer)
constexpr int kPartialStride = 8;  // doubles per block partial record

// Physics constants of the adiabatic model (physics/adiabatic.hpp).
struct PhysParams {
  double gam;            // 2D adiabatic index (2 - 1/gam3d)
  double omega_ns;       // star rotation, z axis
  double e_acc;          // accreted specific energy
  double omega_acc_x, omega_acc_y, omega_acc_z;  // (0, sin(tilt), cos(tilt)) * omega_acc_abs
  double alpha;          // friction coefficient
  double acc_rate;       // accretion rate (depletion without friction)
  double total_mass;     // initial mass (depletion without friction)
  double h0;             // minimum edge arc length
  double round_diff;     // arc/chord of face 0 edge (1,2)
  int accretion_on;
  int friction_on;
  int solver;            // 1 HLLE_p, 2 HLLC, 3 HLLC+, 4 HLLE (isothermal)
  // derived once on the host (derive_params) so that no thread re-derives a
  // uniform constant: gam3d / (2 gam3d - 1) with gam3d = 1 / (2 - gam)
  // (physics/adiabatic.hpp:563-566), and FP32 copies for the mixed path
  double fric_k;
  double gam_m1, fric_ak;  // gam - 1 and alpha * fric_k (mixed-path update)
  float gam_f, e_acc_f, alpha_f, omega_ns_f, fric_ak_f;
  float gam_m1_h, gam_m1_l;  // gam - 1 as a double-word (nearest float + residual)
  float cfl_num_f;           // h0 * 0.1 rounded to a float (numerator of the CFL bound)
  float omega_acc_f[3];
  float depletion_f;     // -(acc_rate 4 pi) / total_mass (adiabatic.hpp:430-436)
};

// Fills the derived fields of P from its primary ones.
inline void derive_params(PhysParams& P) {
  const double gam3d = 1 / (2 - P.gam);
  P.fric_k = gam3d / (2 * gam3d - 1);
  P.gam_m1 = P.gam - 1.0;
  P.fric_ak = P.alpha * P.fric_k;
  P.fric_ak_f = (float)P.fric_ak;
  P.gam_m1_h = (float)P.gam_m1;
  P.gam_m1_l = (float)(P.gam_m1 - (double)P.gam_m1_h);
  P.cfl_num_f = (float)(P.h0 * 0.1);
  P.gam_f = (float)P.gam;
  P.e_acc_f = (float)P.e_acc;
  P.alpha_f = (float)P.alpha;
  P.omega_ns_f = (float)P.omega_ns;
  P.omega_acc_f[0] = (float)P.omega_acc_x;
  P.omega_acc_f[1] = (float)P.omega_acc_y;
  P.omega_acc_f[2] = (float)P.omega_acc_z;
  P.depletion_f = (P.total_mass != 0) ? (float)(-(P.acc_rate * 4 * 3.14159265358979323846) / P.total_mass) : 0.f;
}

constexpr int kSolverIsoHLLE = 4;  // the isothermal solver (4 state fields)

// FP64 geometry, slot planes of length max_slots * fpad unless noted.
struct DevGeom {
  int n_faces;
  int fpad;
  int max_slots;
  // per face [fpad]
  const int8_t* nslots;   // number of edges
  const double* fcn;      // unit face centre, 3 planes of fpad (x | y | z)
  const double* area;     // spherical excess
  const double* acc_src;  // accretion mass source res[0] (0 when accretion is off)
  // per slot
  const int* sten;        // 4 planes: flux_faces_plus[0..1], flux_faces_minus[0..1] (internal ids)
  const double* beta;     // 4 planes: betas_plus[0..1], betas_minus[0..1]
  const double* hpm;      // 2 planes: H_plus, H_minus
  const double* bm;       // BM_dist
  const double* eta;      // 2 planes: H_plus/BM, H_minus/BM
  const double* arc_a;    // great-circle edge length / face area (limiter Courant factor)
  const double* ec;       // 3 planes: unit edge centre
  const double* ecn;      // |ec| as evaluated in double
  const double* en;       // 3 planes: outward edge normal
  const double* nxr;      // 3 planes: cross(en, ec/|ec|)
  const double* chord;    // straight edge length
  const int* rev;         // slot-plane index of the same edge seen from the neighbour
};

// Geometry of the FP32/FP64 mixed path: FP32 slot planes, FP64 where the
// value feeds an FP64 step (unit centre for pressure recovery and the dt
// clip, area, accretion mass source, flux coefficient).
struct DevGeomMixed {
  int n_faces;
  int fpad;
  int max_slots;
  const int8_t* nslots;
  const double* fcn;      // 3 planes, FP64 unit face centre
  const float* fcn32;     // 3 planes, FP32 copy (source term), the nearest float
  const float* fcn_lo;    // 3 planes, fcn - fcn32 rounded to a float (fcn as a double-word)
  const double* area;
  const double* acc_src;  // accretion mass source, FP64
  const float* coef;      // per slot: round_diff * chord / area
  const int* slot_edge;   // per slot: its edge, bit 31 set on the edge's reverse side
  // interior edges, each once, face-major (owner face, then slot); records of four interleaved
  // values (read as one int4 / float4 each), see MixedPlanes
  int n_edges;
  int epad;               // n_edges rounded up to 32
  const int* e_ids;       // f | n_f << 28, g | n_g << 28, bits of (n x R).z, 0
  const float* e_ec;      // owner's unit edge centre, (n x R).x
  const float* e_en;      // owner's edge normal, (n x R).y
  const int* e_sten;      // [2][epad]: stencil faces, owner then reverse slot
  const float* e_beta;    // [2][epad]: beta_plus 0, 1, beta_minus 0, 1
  const float* e_h;       // [2][epad]: 1/H_plus, 1/H_minus, BM_dist, arc/area
};

// Solver state on the device.
struct DevState {
  double* U;      // conserved state, kDim planes of fpad
  double* W0;     // (Sigma, l, Pi) of U, kDim planes
  double* W1;     // (Sigma, l, Pi) after stage 1, kDim planes
  double* uplus;  // reconstructed edge states, kDim * max_slots planes of fpad
  float* W32;     // mixed path: stage-1 input (Sigma, l, Pi) in FP32: [fpad] float4 (Sigma, l), then a Pi plane
  float* W32b;    // mixed path: stage-2 input, the same layout (written by the stage-1 update)
  float* uplus32; // mixed path: the last stage-2 edge states, packed like W32 over 2 * epad entries
                  // (owner side of edge e at e, reverse side at epad + e), recomputed for the
                  // writers (mixed_edge_states); may be null
  float* fe32;    // mixed path: FP32 Riemann flux of every edge, packed like W32 over epad edges
  double* partial;  // per-block partial records (kPartialStride doubles)
  double* scal;   // device scalars, see ScalarSlot
  unsigned int* err;  // stop bits
  unsigned* keys;  // mixed path: [0] max |v|^2 key, [1] min signed-square extra-dt key (FP32 order keys)
};

// One member of an ensemble: its mesh level's geometry (shared between
// members on the same mesh, except the per-member accretion source), its own
// state buffers and its own physics parameters.
struct EnsInstance {
  DevGeomMixed G;
  DevState S;
  PhysParams P;
};

enum ScalarSlot : int {
  kScDt = 0,       // dt of the current step (clipped)
  kScTime = 1,     // simulation time after the current step
  kScMaxVel = 2,   // max_vel of the step's input state
  kScExtraDt = 3,  // extra_dt_constr of the step's input state
  kScMass = 4,     // 4..8: sum Sigma A, l_x A, l_y A, l_z A, E A of the step's input state
  kScDt0 = 9,      // dt0 requested by the caller
  kScDtF = 10,     // mixed path: (float dt, float dt/2) packed in one slot
  kScDtHalf = 11,  // mixed path: dt / 2 (FP64)
  kScCount = 16
};

}  // namespace splash
