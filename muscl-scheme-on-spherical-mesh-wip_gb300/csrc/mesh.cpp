// Half-edge mesh and sphere generators reproducing the reference numbering.
// See mesh.hpp for the contract.  Floating-point expressions are written in
// the exact evaluation order of the reference so that vertex positions come
// out bit-identical (the library is compiled without FMA contraction).
#include "mesh.hpp"

#include <cmath>
#include <stdexcept>
#include <utility>

namespace splash {

namespace {

inline Vec3 add(const Vec3& a, const Vec3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline void add_to(Vec3& a, const Vec3& b) {
  a[0] += b[0];
  a[1] += b[1];
  a[2] += b[2];
}
inline void scale(Vec3& a, double s) {
  a[0] *= s;
  a[1] *= s;
  a[2] *= s;
}
inline void divide(Vec3& a, double s) {
  a[0] /= s;
  a[1] /= s;
  a[2] /= s;
}
// pmp sqrnorm accumulates from 0 in index order (pmp/mat_vec.h:518-524).
inline double norm(const Vec3& a) {
  double s = 0.0;
  s += a[0] * a[0];
  s += a[1] * a[1];
  s += a[2] * a[2];
  return std::sqrt(s);
}

// Arithmetic mean of a face's corner positions in face-circulation order
// (pmp/algorithms/differential_geometry.cpp:150-161, geometry/sph_gen.h:59-70).
Vec3 face_centroid(const HalfedgeMesh& m, int f, std::vector<int>& scratch) {
  m.face_vertices(f, scratch);
  Vec3 c{0.0, 0.0, 0.0};
  double n = 0.0;
  for (int v : scratch) {
    add_to(c, m.position(v));
    n += 1.0;
  }
  divide(c, n);
  return c;
}

}  // namespace

void HalfedgeMesh::reserve(size_t nv, size_t ne, size_t nf) {
  pos_.reserve(nv);
  vert_he_.reserve(nv);
  he_to_.reserve(2 * ne);
  he_next_.reserve(2 * ne);
  he_prev_.reserve(2 * ne);
  he_face_.reserve(2 * ne);
  face_he_.reserve(nf);
}

int HalfedgeMesh::add_vertex(const Vec3& p) {
  pos_.push_back(p);
  vert_he_.push_back(kInvalid);
  return (int)pos_.size() - 1;
}

int HalfedgeMesh::new_edge(int from, int to) {
  const int h = (int)he_to_.size();
  // h points to `to`; its opposite h+1 points back to `from`.
  he_to_.push_back(to);
  he_to_.push_back(from);
  for (int k = 0; k < 2; ++k) {
    he_next_.push_back(kInvalid);
    he_prev_.push_back(kInvalid);
    he_face_.push_back(kInvalid);
  }
  return h;
}

int HalfedgeMesh::new_face() {
  face_he_.push_back(kInvalid);
  return (int)face_he_.size() - 1;
}

int HalfedgeMesh::find_halfedge(int from, int to) const {
  const int start = vert_he_[from];
  if (start == kInvalid) return kInvalid;
  int h = start;
  do {
    if (he_to_[h] == to) return h;
    h = cw(h);
  } while (h != start);
  return kInvalid;
}

void HalfedgeMesh::adjust_outgoing(int v) {
  const int start = vert_he_[v];
  if (start == kInvalid) return;
  int h = start;
  do {
    if (is_boundary_he(h)) {
      vert_he_[v] = h;
      return;
    }
    h = cw(h);
  } while (h != start);
}

int HalfedgeMesh::add_face(const std::vector<int>& loop) {
  const size_t n = loop.size();
  if (n < 3) throw std::runtime_error("add_face: fewer than three vertices");
  // per-thread scratch, reused across calls (a mesh build adds millions of
  // faces; the algorithm and the resulting numbering are unchanged)
  thread_local std::vector<int> he;
  thread_local std::vector<char> fresh, adjust;
  thread_local std::vector<std::pair<int, int>> links;
  he.assign(n, kInvalid);
  fresh.assign(n, 0);
  adjust.assign(n, 0);
  links.clear();
  links.reserve(3 * n);

  // Existing half-edges along the loop; every corner must lie on the
  // current boundary and every existing edge must still be open.
  for (size_t i = 0; i < n; ++i) {
    const size_t ii = (i + 1) % n;
    if (!is_boundary_vertex(loop[i])) throw std::runtime_error("add_face: complex vertex");
    he[i] = find_halfedge(loop[i], loop[ii]);
    fresh[i] = (he[i] == kInvalid);
    if (!fresh[i] && !is_boundary_he(he[i])) throw std::runtime_error("add_face: complex edge");
  }

  // Two consecutive existing half-edges that are not yet consecutive on the
  // boundary: move the patch between them to another boundary gap.
  for (size_t i = 0; i < n; ++i) {
    const size_t ii = (i + 1) % n;
    if (fresh[i] || fresh[ii]) continue;
    const int in_prev = he[i];
    const int in_next = he[ii];
    if (he_next_[in_prev] == in_next) continue;
    int gap_prev = opposite(in_next);
    do {
      gap_prev = opposite(he_next_[gap_prev]);
    } while (!is_boundary_he(gap_prev) || gap_prev == in_prev);
    const int gap_next = he_next_[gap_prev];
    if (gap_next == in_next) throw std::runtime_error("add_face: patch re-linking failed");
    const int patch_first = he_next_[in_prev];
    const int patch_last = he_prev_[in_next];
    links.emplace_back(gap_prev, patch_first);
    links.emplace_back(patch_last, gap_next);
    links.emplace_back(in_prev, in_next);
  }

  for (size_t i = 0; i < n; ++i) {
    if (fresh[i]) he[i] = new_edge(loop[i], loop[(i + 1) % n]);
  }

  const int f = new_face();
  face_he_[f] = he[n - 1];

  for (size_t i = 0; i < n; ++i) {
    const size_t ii = (i + 1) % n;
    const int v = loop[ii];
    const int in_prev = he[i];
    const int in_next = he[ii];
    const int kind = (fresh[i] ? 1 : 0) | (fresh[ii] ? 2 : 0);
    if (kind != 0) {
      const int out_prev = opposite(in_next);
      const int out_next = opposite(in_prev);
      if (kind == 1) {
        // incoming edge is new, outgoing edge existed
        links.emplace_back(he_prev_[in_next], out_next);
        vert_he_[v] = out_next;
      } else if (kind == 2) {
        // incoming edge existed, outgoing edge is new
        const int bnext = he_next_[in_prev];
        links.emplace_back(out_prev, bnext);
        vert_he_[v] = bnext;
      } else {
        // both new
        if (vert_he_[v] == kInvalid) {
          vert_he_[v] = out_next;
          links.emplace_back(out_prev, out_next);
        } else {
          const int bnext = vert_he_[v];
          const int bprev = he_prev_[bnext];
          links.emplace_back(bprev, out_next);
          links.emplace_back(out_prev, bnext);
        }
      }
      links.emplace_back(in_prev, in_next);
    } else {
      adjust[ii] = (vert_he_[v] == in_next);
    }
    he_face_[he[i]] = f;
  }

  for (const auto& l : links) link(l.first, l.second);
  for (size_t i = 0; i < n; ++i)
    if (adjust[i]) adjust_outgoing(loop[i]);
  return f;
}

int HalfedgeMesh::insert_vertex(int h0, int v) {
  const int h2 = he_next_[h0];
  const int o0 = opposite(h0);
  const int o2 = he_prev_[o0];
  const int v2 = he_to_[h0];
  const int fh = he_face_[h0];
  const int fo = he_face_[o0];

  const int h1 = new_edge(v, v2);
  const int o1 = opposite(h1);

  link(h1, h2);
  link(h0, h1);
  he_to_[h0] = v;
  he_to_[h1] = v2;
  he_face_[h1] = fh;

  link(o1, o0);
  link(o2, o1);
  he_to_[o1] = v;
  he_face_[o1] = fo;

  vert_he_[v2] = o1;
  adjust_outgoing(v2);
  vert_he_[v] = h1;
  adjust_outgoing(v);

  if (fh != kInvalid) face_he_[fh] = h0;
  if (fo != kInvalid) face_he_[fo] = o1;
  return o1;
}

int HalfedgeMesh::insert_edge(int h0, int h1) {
  const int v0 = he_to_[h0];
  const int v1 = he_to_[h1];
  const int h2 = he_next_[h0];
  const int h3 = he_next_[h1];

  const int h4 = new_edge(v0, v1);
  const int h5 = opposite(h4);

  const int f0 = he_face_[h0];
  const int f1 = new_face();

  face_he_[f0] = h0;
  face_he_[f1] = h1;

  link(h0, h4);
  link(h4, h3);
  he_face_[h4] = f0;

  link(h1, h5);
  link(h5, h2);
  int h = h2;
  do {
    he_face_[h] = f1;
    h = he_next_[h];
  } while (h != h2);
  return h4;
}

void HalfedgeMesh::face_vertices(int f, std::vector<int>& out) const {
  out.clear();
  const int start = face_he_[f];
  int h = start;
  do {
    out.push_back(he_to_[h]);
    h = he_next_[h];
  } while (h != start);
}

void HalfedgeMesh::vertex_vertices(int v, std::vector<int>& out) const {
  out.clear();
  const int start = vert_he_[v];
  if (start == kInvalid) return;
  int h = start;
  do {
    out.push_back(he_to_[h]);
    h = ccw(h);
  } while (h != start);
}

void HalfedgeMesh::vertex_faces(int v, std::vector<int>& out) const {
  out.clear();
  int start = vert_he_[v];
  if (start == kInvalid) return;
  // The face circulator skips boundary half-edges, starting with the first.
  if (is_boundary_he(start)) {
    do {
      start = ccw(start);
    } while (is_boundary_he(start));
  }
  int h = start;
  do {
    out.push_back(he_face_[h]);
    do {
      h = ccw(h);
    } while (is_boundary_he(h));
  } while (h != start);
}

void project_to_unit_sphere(HalfedgeMesh& m) {
  // p <- (1/|p|) * p   (geometry/sph_gen.h:140-148)
  for (int v = 0; v < m.n_vertices(); ++v) {
    Vec3& p = m.position(v);
    const double n = norm(p);
    scale(p, 1.0 / n);
  }
}

HalfedgeMesh make_icosahedron() {
  HalfedgeMesh m;
  const double phi = (1.0 + std::sqrt(5.0)) * 0.5;
  const double a = 1.0;
  const double b = 1.0 / phi;
  // corner order and coordinates of geometry/sph_gen.h:167-178
  const Vec3 corners[12] = {{0, b, -a}, {b, a, 0},  {-b, a, 0},  {0, b, a},
                            {0, -b, a}, {-a, 0, b}, {0, -b, -a}, {a, 0, -b},
                            {a, 0, b},  {-a, 0, -b}, {b, -a, 0}, {-b, -a, 0}};
  for (const auto& c : corners) m.add_vertex(c);
  project_to_unit_sphere(m);
  // triangles of geometry/sph_gen.h:183-202, 1-based corner labels
  static const int tri[20][3] = {{3, 2, 1},   {2, 3, 4},   {6, 5, 4},  {5, 9, 4},  {8, 7, 1},
                                 {7, 10, 1},  {12, 11, 5}, {11, 12, 7}, {10, 6, 3}, {6, 10, 12},
                                 {9, 8, 2},   {8, 9, 11},  {3, 6, 4},  {9, 2, 4},  {10, 3, 1},
                                 {2, 8, 1},   {12, 10, 7}, {8, 11, 7}, {6, 12, 5}, {11, 9, 5}};
  for (const auto& t : tri) m.add_face({t[0] - 1, t[1] - 1, t[2] - 1});
  return m;
}

HalfedgeMesh make_hexahedron() {
  HalfedgeMesh m;
  const double a = 1.0 / std::sqrt(3.0);
  // corner order of geometry/sph_gen.h:39-46
  const Vec3 corners[8] = {{-a, -a, -a}, {a, -a, -a}, {a, a, -a}, {-a, a, -a},
                           {-a, -a, a},  {a, -a, a},  {a, a, a},  {-a, a, a}};
  for (const auto& c : corners) m.add_vertex(c);
  // quads of geometry/sph_gen.h:49-54
  static const int quad[6][4] = {{3, 2, 1, 0}, {2, 6, 5, 1}, {5, 6, 7, 4},
                                 {0, 4, 7, 3}, {3, 7, 6, 2}, {1, 5, 4, 0}};
  for (const auto& q : quad) m.add_face({q[0], q[1], q[2], q[3]});
  return m;
}

void loop_subdivide(HalfedgeMesh& m) {
  const int nv = m.n_vertices();
  const int ne = m.n_edges();
  const int nf = m.n_faces();
  m.reserve((size_t)(nv + ne), (size_t)(2 * ne + 3 * nf), (size_t)(4 * nf));
  std::vector<int> ring;
  std::vector<Vec3> vpoint(nv), epoint(ne);

  // even (old) vertices: (1-beta) p + beta * mean(ring)
  // (pmp/algorithms/subdivision.cpp:251-265)
  for (int v = 0; v < nv; ++v) {
    if (m.vertex_halfedge(v) == HalfedgeMesh::kInvalid) {
      vpoint[v] = m.position(v);
      continue;
    }
    m.vertex_vertices(v, ring);
    Vec3 p{0.0, 0.0, 0.0};
    double k = 0.0;
    for (int w : ring) {
      add_to(p, m.position(w));
      k += 1.0;
    }
    divide(p, k);
    const double s = 0.375 + 0.25 * std::cos(2.0 * M_PI / k);
    const double beta = 0.625 - s * s;
    Vec3 q = m.position(v);
    scale(q, 1.0 - beta);
    Vec3 r = p;
    scale(r, beta);
    vpoint[v] = add(q, r);
  }

  // odd (edge) vertices: (3 (a + b) + c + d) / 8 with the stencil order of
  // pmp/algorithms/subdivision.cpp:281-289
  for (int e = 0; e < ne; ++e) {
    const int h0 = 2 * e;
    const int h1 = 2 * e + 1;
    Vec3 p = m.position(m.to_vertex(h0));
    add_to(p, m.position(m.to_vertex(h1)));
    scale(p, 3.0);
    add_to(p, m.position(m.to_vertex(m.next(h0))));
    add_to(p, m.position(m.to_vertex(m.next(h1))));
    scale(p, 0.125);
    epoint[e] = p;
  }

  for (int v = 0; v < nv; ++v) m.position(v) = vpoint[v];

  // split every original edge, then cut each original triangle into four
  for (int e = 0; e < ne; ++e) m.insert_vertex(2 * e, m.add_vertex(epoint[e]));
  for (int f = 0; f < nf; ++f) {
    int h = m.face_halfedge(f);
    m.insert_edge(h, m.next(m.next(h)));
    h = m.next(h);
    m.insert_edge(h, m.next(m.next(h)));
    h = m.next(h);
    m.insert_edge(h, m.next(m.next(h)));
  }
}

void catmull_clark_subdivide(HalfedgeMesh& m) {
  const int nv = m.n_vertices();
  const int ne = m.n_edges();
  const int nf = m.n_faces();
  m.reserve((size_t)(nv + ne + nf), (size_t)(2 * ne + 4 * nf), (size_t)(4 * nf));
  std::vector<int> scratch, ring, fring;
  std::vector<Vec3> vpoint(nv), epoint(ne), fpoint(nf);

  for (int f = 0; f < nf; ++f) fpoint[f] = face_centroid(m, f, scratch);

  // edge points: (a + b + fa + fb) / 4  (pmp/algorithms/subdivision.cpp:42-50)
  for (int e = 0; e < ne; ++e) {
    Vec3 p{0.0, 0.0, 0.0};
    add_to(p, m.position(m.to_vertex(2 * e)));
    add_to(p, m.position(m.to_vertex(2 * e + 1)));
    add_to(p, fpoint[m.face(2 * e)]);
    add_to(p, fpoint[m.face(2 * e + 1)]);
    scale(p, 0.25);
    epoint[e] = p;
  }

  // vertex points: (sum ring + sum faces) / k^2 + (k-2)/k p
  // (pmp/algorithms/subdivision.cpp:103-119)
  for (int v = 0; v < nv; ++v) {
    if (m.vertex_halfedge(v) == HalfedgeMesh::kInvalid) {
      vpoint[v] = m.position(v);
      continue;
    }
    m.vertex_vertices(v, ring);
    m.vertex_faces(v, fring);
    const double k = (double)ring.size();
    Vec3 p{0.0, 0.0, 0.0};
    for (int w : ring) add_to(p, m.position(w));
    for (int f : fring) add_to(p, fpoint[f]);
    divide(p, k * k);
    Vec3 q = m.position(v);
    scale(q, (k - 2.0) / k);
    add_to(p, q);
    vpoint[v] = p;
  }

  for (int v = 0; v < nv; ++v) m.position(v) = vpoint[v];

  for (int e = 0; e < ne; ++e) m.insert_vertex(2 * e, m.add_vertex(epoint[e]));

  for (int f = 0; f < nf; ++f) {
    const int h0 = m.face_halfedge(f);
    m.insert_edge(h0, m.next(m.next(h0)));
    const int h1 = m.next(h0);
    // insert the face point on the new diagonal (edge(h1)'s first half-edge)
    m.insert_vertex(h1 & ~1, m.add_vertex(fpoint[f]));
    int h = m.next(m.next(m.next(h1)));
    while (h != h0) {
      m.insert_edge(h1, h);
      h = m.next(m.next(m.next(h1)));
    }
  }
}

HalfedgeMesh face_vertex_dual(const HalfedgeMesh& m) {
  HalfedgeMesh d;
  const int nf = m.n_faces();
  const int nv = m.n_vertices();
  d.reserve((size_t)nf, (size_t)m.n_edges(), (size_t)nv);
  std::vector<int> scratch, fring;
  for (int f = 0; f < nf; ++f) d.add_vertex(face_centroid(m, f, scratch));
  for (int v = 0; v < nv; ++v) {
    m.vertex_faces(v, fring);
    d.add_face(fring);  // dual vertex id == primal face id
  }
  return d;
}

HalfedgeMesh icosphere(int levels) {
  HalfedgeMesh m = make_icosahedron();
  for (int i = 0; i < levels; ++i) {
    loop_subdivide(m);
    project_to_unit_sphere(m);
  }
  return m;
}

HalfedgeMesh icosphere_hex(int levels) {
  HalfedgeMesh m = face_vertex_dual(icosphere(levels));
  project_to_unit_sphere(m);
  return m;
}

HalfedgeMesh quad_sphere(int levels) {
  HalfedgeMesh m = make_hexahedron();
  for (int i = 0; i < levels; ++i) {
    catmull_clark_subdivide(m);
    project_to_unit_sphere(m);
  }
  return m;
}

HalfedgeMesh build_mesh(int kind, int levels) {
  if (levels < 0 || levels > 11) throw std::runtime_error("mesh level out of range [0, 11]");
  switch (kind) {
    case kMeshIcosphereHex:
      return icosphere_hex(levels);
    case kMeshQuadSphere:
      return quad_sphere(levels);
    case kMeshIcosphere:
      return icosphere(levels);
    default:
      throw std::runtime_error("unknown mesh kind");
  }
}

}  // namespace splash
