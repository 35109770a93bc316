// Spherical mesh construction with the reference's element numbering.
//
// The reference builds its meshes with the vendored pmp-library
// (pmp/surface_mesh.cpp, pmp/algorithms/subdivision.cpp) driven by
// geometry/sph_gen.h.  The solver numbers faces, vertices and the vertex
// order inside each face exactly as pmp's iterators and circulators visit
// them, and several floating-point sums (subdivision stencils, centroids)
// depend on that visiting order.  This file is an independent half-edge mesh
// that reproduces the same element order and the same arithmetic order:
//
//   * element creation order of add_face / insert_vertex / insert_edge
//     (pmp/surface_mesh.cpp:244-420, 598-690);
//   * circulation direction: around a vertex counter-clockwise starting at the
//     vertex's outgoing half-edge, around a face following next()
//     (pmp/surface_mesh.h:602-1090);
//   * Loop and Catmull-Clark subdivision (pmp/algorithms/subdivision.cpp:9-331)
//     and the face-vertex dual (geometry/sph_gen.h:72-96).
//
// Only what closed manifold sphere meshes need is implemented: no boundary
// feature rules, no deletion / garbage collection.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

namespace splash {

using Vec3 = std::array<double, 3>;

class HalfedgeMesh {
 public:
  static constexpr int kInvalid = -1;

  int add_vertex(const Vec3& p);
  // Adds a face over the given vertex loop.  Throws std::runtime_error on a
  // non-manifold configuration (the cases pmp reports as TopologyException).
  int add_face(const std::vector<int>& loop);
  // Splits the edge of half-edge h0 by vertex v; returns the new half-edge
  // that starts at v on the opposite side (pmp insert_vertex(Halfedge, Vertex)).
  int insert_vertex(int h0, int v);
  // Splits the face of h0/h1 by a new edge from to(h0) to to(h1); returns the
  // new half-edge from to(h0) (pmp insert_edge).
  int insert_edge(int h0, int h1);

  int n_vertices() const { return (int)pos_.size(); }
  int n_faces() const { return (int)face_he_.size(); }
  int n_edges() const { return (int)(he_to_.size() / 2); }

  const Vec3& position(int v) const { return pos_[v]; }
  Vec3& position(int v) { return pos_[v]; }

  int to_vertex(int h) const { return he_to_[h]; }
  int next(int h) const { return he_next_[h]; }
  int prev(int h) const { return he_prev_[h]; }
  int face(int h) const { return he_face_[h]; }
  static int opposite(int h) { return h ^ 1; }
  int vertex_halfedge(int v) const { return vert_he_[v]; }
  int face_halfedge(int f) const { return face_he_[f]; }
  bool is_boundary_he(int h) const { return he_face_[h] == kInvalid; }
  bool is_boundary_vertex(int v) const {
    const int h = vert_he_[v];
    return !(h != kInvalid && he_face_[h] != kInvalid);
  }
  // Rotations about the start vertex of h.
  int ccw(int h) const { return opposite(he_prev_[h]); }
  int cw(int h) const { return he_next_[opposite(h)]; }

  // Visiting orders identical to pmp's range-based circulators.
  void face_vertices(int f, std::vector<int>& out) const;
  void vertex_vertices(int v, std::vector<int>& out) const;
  void vertex_faces(int v, std::vector<int>& out) const;

  void reserve(size_t nv, size_t ne, size_t nf);

 private:
  int new_edge(int from, int to);
  int new_face();
  int find_halfedge(int from, int to) const;
  void adjust_outgoing(int v);
  void link(int h, int nh) {
    he_next_[h] = nh;
    he_prev_[nh] = h;
  }

  std::vector<Vec3> pos_;
  std::vector<int> vert_he_;
  std::vector<int> he_to_, he_next_, he_prev_, he_face_;
  std::vector<int> face_he_;
};

// Generators with the reference numbering (geometry/sph_gen.h:31-57,
// 140-148, 158-205, 267-295).
HalfedgeMesh make_icosahedron();
HalfedgeMesh make_hexahedron();
void loop_subdivide(HalfedgeMesh& m);
void catmull_clark_subdivide(HalfedgeMesh& m);
void project_to_unit_sphere(HalfedgeMesh& m);
HalfedgeMesh face_vertex_dual(const HalfedgeMesh& m);

HalfedgeMesh icosphere(int levels);
HalfedgeMesh icosphere_hex(int levels);
HalfedgeMesh quad_sphere(int levels);

enum MeshKind : int { kMeshIcosphereHex = 0, kMeshQuadSphere = 1, kMeshIcosphere = 2 };
HalfedgeMesh build_mesh(int kind, int levels);

}  // namespace splash
