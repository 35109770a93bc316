// Once-per-run finite-volume geometry in the reference numbering.
//
// Restates the reference precompute of geometry/MUSCL_geometry.hpp:43-575
// and :981-1030 (vertex/face extraction, vertex-ring and edge neighbours,
// polyhedral face centres, face normals, spherical-excess areas, edge normals,
// the two-face reconstruction stencils with their barycentric weights and the
// distances H+, H-, BM) plus h0 of MUSCL_base/MUSCL_base.hpp:63-91 and the
// res2d chord factor of :242.  Arrays are flattened: faces use CSR offsets
// `face_off`, and every per-(face, edge) quantity is stored per "slot"
// s = face_off[i] + j.
#pragma once

#include <cstdint>
#include <vector>

#include "mesh.hpp"

namespace splash {

struct RefGeometry {
  int n_vertices = 0;
  int n_faces = 0;
  int n_slots = 0;
  int max_slots = 0;  // largest face valence (N in MUSCL_base.hpp:63-70)

  std::vector<double> vertices;  // [nv][3]
  std::vector<int> face_off;     // [nf+1]
  std::vector<int> face_vtx;     // [ns]    faces[i][j]
  std::vector<int> nbr_off;      // [nf+1]
  std::vector<int> nbr;          // sorted vertex-ring neighbours (neighbors[i])
  std::vector<int> nbr_edge;     // [ns]    neighbors_edge[i][j]
  std::vector<double> face_centers;  // [nf][3] polyhedral centroid, |c| < 1
  std::vector<double> normals;       // [nf][3]
  std::vector<double> area;          // [nf]   spherical excess

  std::vector<double> edge_normals;  // [ns][3]
  std::vector<double> bm_dist;       // [ns]
  std::vector<double> h_plus;        // [ns]
  std::vector<double> h_minus;       // [ns]
  std::vector<int> ff_plus;          // [ns][2] flux_faces_plus
  std::vector<int> ff_minus;         // [ns][2] flux_faces_minus
  std::vector<double> beta_plus;     // [ns][2]
  std::vector<double> beta_minus;    // [ns][2]

  double h0 = 0.0;          // minimum great-circle edge length
  double round_diff = 0.0;  // arc / chord of face 0, edge (1, 2)
};

// A polygon mesh as plain arrays: the input of the geometry precompute.
struct MeshArrays {
  std::vector<double> vertices;  // [nv][3]
  std::vector<int> face_off;     // [nf+1]
  std::vector<int> face_vtx;     // corner ids in circulation order
};

// Face corner lists in pmp's circulation order (MUSCL_geometry.hpp:79-88).
MeshArrays mesh_arrays(const HalfedgeMesh& mesh);

// Builds the reference geometry of a mesh.  The vertex-ring neighbour sets
// only depend on which faces share a vertex, so plain arrays suffice.
// `threads` <= 0 uses the OpenMP default.  Throws std::runtime_error if the
// mesh is malformed or violates an assumption of the reference (an edge
// without exactly one edge-neighbour).
RefGeometry build_ref_geometry(const MeshArrays& mesh, int threads);

// Great-circle distance of geometry/MUSCL_geometry.hpp:981-987.
double great_circle(const double* a, const double* b);

}  // namespace splash
