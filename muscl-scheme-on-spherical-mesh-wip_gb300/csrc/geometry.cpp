// Reference-numbered geometry precompute.  Every floating-point expression is
// written in the evaluation order of geometry/MUSCL_geometry.hpp so that the
// arrays are bit-identical to the reference's members when both are compiled
// without FMA contraction.  Per-face work is independent and runs in an
// OpenMP loop; results do not depend on the thread count.
#include "geometry.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace splash {

namespace {

struct V {
  double x, y, z;
};

inline V mk(const double* p) { return {p[0], p[1], p[2]}; }
inline V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V operator*(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V operator/(V a, double s) { return {a.x / s, a.y / s, a.z / s}; }
// vector3d::norm: sqrt of an in-order sum starting at 0 (vec3d.hpp:56-64)
inline double norm(V a) {
  double s = 0.0;
  s += a.x * a.x;
  s += a.y * a.y;
  s += a.z * a.z;
  return std::sqrt(s);
}
inline V cross(V a, V b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// geometry/MUSCL_geometry.hpp:981-987
inline double gc_distance(V a, V b) {
  a = a / norm(a);
  b = b / norm(b);
  const double d = norm(a - b);
  return 2 * std::asin(d / 2);
}

// geometry/MUSCL_geometry.hpp:846-870: point where the line xl + t nl meets
// the plane through xs spanned by vs1, vs2.
inline V line_plane(V xl, V nl, V xs, V vs1, V vs2) {
  const double A = vs1.y * vs2.z - vs1.z * vs2.y;
  const double B = vs1.z * vs2.x - vs1.x * vs2.z;
  const double C = vs1.x * vs2.y - vs1.y * vs2.x;
  const double D = -xs.x * A - xs.y * B - xs.z * C;
  const double t = -(D + A * xl.x + B * xl.y + C * xl.z) / (A * nl.x + B * nl.y + C * nl.z);
  return xl + nl * t;
}

}  // namespace

double great_circle(const double* a, const double* b) { return gc_distance(mk(a), mk(b)); }

MeshArrays mesh_arrays(const HalfedgeMesh& mesh) {
  MeshArrays a;
  const int nv = mesh.n_vertices();
  const int nf = mesh.n_faces();
  a.vertices.resize(3 * (size_t)nv);
  for (int v = 0; v < nv; ++v) {
    const Vec3& p = mesh.position(v);
    a.vertices[3 * (size_t)v + 0] = p[0];
    a.vertices[3 * (size_t)v + 1] = p[1];
    a.vertices[3 * (size_t)v + 2] = p[2];
  }
  a.face_off.assign(nf + 1, 0);
  a.face_vtx.reserve(6 * (size_t)nf);
  std::vector<int> loop;
  for (int f = 0; f < nf; ++f) {
    mesh.face_vertices(f, loop);
    a.face_off[f] = (int)a.face_vtx.size();
    a.face_vtx.insert(a.face_vtx.end(), loop.begin(), loop.end());
  }
  a.face_off[nf] = (int)a.face_vtx.size();
  return a;
}

RefGeometry build_ref_geometry(const MeshArrays& mesh, int threads) {
  RefGeometry g;
  const int nv = (int)(mesh.vertices.size() / 3);
  const int nf = (int)mesh.face_off.size() - 1;
  if (nv < 4 || nf < 4) throw std::runtime_error("mesh needs at least 4 vertices and 4 faces");
  if (mesh.face_off[0] != 0 || mesh.face_off[nf] != (int)mesh.face_vtx.size())
    throw std::runtime_error("face offsets do not cover the corner list");
  for (int f = 0; f < nf; ++f) {
    const int n = mesh.face_off[f + 1] - mesh.face_off[f];
    if (n < 3 || n > 64) throw std::runtime_error("face " + std::to_string(f) + " has " + std::to_string(n) + " corners");
  }
  for (int v : mesh.face_vtx)
    if (v < 0 || v >= nv) throw std::runtime_error("corner index out of range");
  g.n_vertices = nv;
  g.n_faces = nf;
  g.vertices = mesh.vertices;
  g.face_off = mesh.face_off;
  g.face_vtx = mesh.face_vtx;
  for (int f = 0; f < nf; ++f) g.max_slots = std::max(g.max_slots, g.face_off[f + 1] - g.face_off[f]);
  const int ns = g.face_off[nf];
  g.n_slots = ns;
  const std::vector<int>& off = g.face_off;
  const std::vector<int>& fv = g.face_vtx;
  auto vtx = [&](int v) { return mk(&g.vertices[3 * (size_t)v]); };

  // faces incident to each vertex (a set: the neighbour lists below are
  // sorted and de-duplicated, so the visiting order is irrelevant)
  std::vector<int> vf_off(nv + 1, 0), vf(ns);
  for (int s = 0; s < ns; ++s) vf_off[fv[s] + 1]++;
  for (int v = 0; v < nv; ++v) vf_off[v + 1] += vf_off[v];
  {
    std::vector<int> fill(vf_off.begin(), vf_off.end() - 1);
    for (int f = 0; f < nf; ++f)
      for (int s = off[f]; s < off[f + 1]; ++s) vf[fill[fv[s]]++] = f;
  }

  if (threads > 0) {
#ifdef _OPENMP
    omp_set_num_threads(threads);
#endif
  }

  // vertex-ring neighbours: sorted, unique, without the face itself
  // (MUSCL_geometry.hpp:91-118)
  std::vector<std::vector<int>> nb(nf);
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    std::vector<int>& l = nb[f];
    for (int s = off[f]; s < off[f + 1]; ++s) {
      const int v = fv[s];
      l.insert(l.end(), vf.begin() + vf_off[v], vf.begin() + vf_off[v + 1]);
    }
    std::sort(l.begin(), l.end());
    l.erase(std::unique(l.begin(), l.end()), l.end());
    l.erase(std::remove(l.begin(), l.end(), f), l.end());
  }
  g.nbr_off.assign(nf + 1, 0);
  for (int f = 0; f < nf; ++f) g.nbr_off[f + 1] = g.nbr_off[f] + (int)nb[f].size();
  g.nbr.resize(g.nbr_off[nf]);
  for (int f = 0; f < nf; ++f) std::copy(nb[f].begin(), nb[f].end(), g.nbr.begin() + g.nbr_off[f]);
  std::vector<std::vector<int>>().swap(nb);

  // edge neighbours in edge order (MUSCL_geometry.hpp:145-174): the
  // neighbour containing both end vertices of the edge
  g.nbr_edge.assign(ns, -1);
  int bad_edges = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad_edges)
  for (int f = 0; f < nf; ++f) {
    const int n = off[f + 1] - off[f];
    for (int j = 0; j < n; ++j) {
      const int f1 = fv[off[f] + j];
      const int f2 = fv[off[f] + (j + 1) % n];
      int found = 0;
      for (int k = g.nbr_off[f]; k < g.nbr_off[f + 1]; ++k) {
        const int c = g.nbr[k];
        bool h1 = false, h2 = false;
        for (int s = off[c]; s < off[c + 1]; ++s) {
          h1 = h1 || fv[s] == f1;
          h2 = h2 || fv[s] == f2;
        }
        if (h1 && h2) {
          if (found == 0) g.nbr_edge[off[f] + j] = c;
          ++found;
        }
      }
      if (found != 1) ++bad_edges;
    }
  }
  if (bad_edges != 0)
    throw std::runtime_error("mesh has " + std::to_string(bad_edges) +
                             " edges without exactly one edge-neighbour");

  // polyhedral face centres (MUSCL_geometry.hpp:176-187)
  g.face_centers.resize(3 * (size_t)nf);
  g.normals.resize(3 * (size_t)nf);
  g.area.resize(nf);
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    V c{0, 0, 0};
    const int n = off[f + 1] - off[f];
    for (int k = 0; k < n; ++k) c = c + vtx(fv[off[f] + k]);
    c = c / (double)n;
    g.face_centers[3 * f + 0] = c.x;
    g.face_centers[3 * f + 1] = c.y;
    g.face_centers[3 * f + 2] = c.z;

    // face normal: sum of consecutive edge cross products (:189-218)
    V nrm{0, 0, 0};
    const int* p = &fv[off[f]];
    for (int j = 0; j < n; ++j) {
      V r1, r2;
      if (j + 2 == n) {
        r2 = vtx(p[0]) - vtx(p[j + 1]);
        r1 = vtx(p[j + 1]) - vtx(p[j]);
      } else if (j + 1 == n) {
        r1 = vtx(p[0]) - vtx(p[j]);
        r2 = vtx(p[1]) - vtx(p[0]);
      } else {
        r2 = vtx(p[j + 2]) - vtx(p[j + 1]);
        r1 = vtx(p[j + 1]) - vtx(p[j]);
      }
      nrm = nrm + cross(r1, r2);
    }
    nrm = nrm / norm(nrm);
    g.normals[3 * f + 0] = nrm.x;
    g.normals[3 * f + 1] = nrm.y;
    g.normals[3 * f + 2] = nrm.z;

    // spherical excess of the fan of triangles (centre, v_j, v_j+1)
    // (:989-1030)
    double a_sum = 0;
    const V cn = c / norm(c);
    for (int j = 0; j < n; ++j) {
      const int j1 = (j != n - 1) ? j + 1 : 0;
      const double a = gc_distance(cn, vtx(p[j]));
      const double b = gc_distance(cn, vtx(p[j1]));
      const double cc = gc_distance(vtx(p[j]), vtx(p[j1]));
      const double A = std::acos((std::cos(a) - std::cos(b) * std::cos(cc)) / (std::sin(b) * std::sin(cc)));
      const double B = std::acos((std::cos(b) - std::cos(a) * std::cos(cc)) / (std::sin(a) * std::sin(cc)));
      const double C = std::acos((std::cos(cc) - std::cos(b) * std::cos(a)) / (std::sin(b) * std::sin(a)));
      a_sum += A + B + C - M_PI;
    }
    g.area[f] = a_sum;
  }

  // per-slot stencils (MUSCL_geometry.hpp:227-575)
  g.edge_normals.resize(3 * (size_t)ns);
  g.bm_dist.resize(ns);
  g.h_plus.resize(ns);
  g.h_minus.resize(ns);
  g.ff_plus.resize(2 * (size_t)ns);
  g.ff_minus.resize(2 * (size_t)ns);
  g.beta_plus.resize(2 * (size_t)ns);
  g.beta_minus.resize(2 * (size_t)ns);
  auto fc = [&](int f) { return mk(&g.face_centers[3 * (size_t)f]); };
  auto nr = [&](int f) { return mk(&g.normals[3 * (size_t)f]); };

#pragma omp parallel for schedule(dynamic, 256)
  for (int f = 0; f < nf; ++f) {
    const int n = off[f + 1] - off[f];
    const int* p = &fv[off[f]];
    const V c0 = fc(f);
    const V nf_ = nr(f);
    const int* nb_begin = &g.nbr[g.nbr_off[f]];
    const int* nb_end = nb_begin + (g.nbr_off[f + 1] - g.nbr_off[f]);
    for (int i = 0; i < n; ++i) {
      const int s = off[f] + i;
      const int vb = (i == n - 1) ? p[0] : p[i + 1];
      const V BM = (vtx(p[i]) + vtx(vb)) / 2 - c0;
      const V r = vtx(p[i]) - vtx(vb);
      V r1 = vtx(p[i]) + vtx(vb);
      r1 = r1 / norm(r1);

      V en = cross(r1, r);
      en = en / norm(en);
      if (norm(BM + en * 0.01) < norm(BM)) en = en * -1;
      g.edge_normals[3 * (size_t)s + 0] = en.x;
      g.edge_normals[3 * (size_t)s + 1] = en.y;
      g.edge_normals[3 * (size_t)s + 2] = en.z;
      g.bm_dist[s] = gc_distance(c0, r1);

      // first pass: the neighbours most aligned with -BM (left) and +BM
      // (right) after projection onto the face plane
      double max_left = -1, max_right = -1;
      int left1 = -1, right1 = -1;
      for (const int* q = nb_begin; q != nb_end; ++q) {
        const int o = *q;
        V d = c0 - fc(o);
        V dp = d - nf_ * dot(d, nf_);
        double ce = dot(BM, dp) / (norm(BM) * norm(dp));
        if (ce > max_left) {
          max_left = ce;
          left1 = o;
        }
        d = fc(o) - c0;
        dp = d - nf_ * dot(d, nf_);
        ce = dot(BM, dp) / (norm(BM) * norm(dp));
        if (ce > max_right) {
          max_right = ce;
          right1 = o;
        }
      }

      if (left1 < 0 || right1 < 0)
        throw std::runtime_error("face " + std::to_string(f) + " has no usable stencil neighbour");

      // second pass: the best neighbour on the other side of the BM line
      max_left = -1;
      max_right = -1;
      int left2 = left1, right2 = right1;
      const V B_left = c0 - fc(left1);
      const V B_right = fc(right1) - c0;
      const V B_right_face = B_right - nf_ * dot(B_right, nf_);
      const V side = cross(c0, r1 / 2);
      for (const int* q = nb_begin; q != nb_end; ++q) {
        const int o = *q;
        V d = c0 - fc(o);
        V dp = d - nf_ * dot(d, nf_);
        double ce = dot(BM, dp) / (norm(BM) * norm(dp));
        double lcc = dot(side, d) * dot(side, B_left);
        if ((ce > max_left) && (o != left1) && (lcc <= 0)) {
          max_left = ce;
          left2 = o;
        }
        d = fc(o) - c0;
        dp = d - nf_ * dot(d, nf_);
        ce = dot(BM, dp) / (norm(BM) * norm(dp));
        lcc = dot(nf_, cross(dp, BM)) * dot(nf_, cross(B_right_face, BM));
        if ((ce > max_right) && (o != right1) && (lcc <= 0)) {
          max_right = ce;
          right2 = o;
        }
      }

      V p3 = line_plane(fc(left1), fc(left2) - fc(left1), c0, BM, c0);
      const V Hm = p3 / norm(p3);
      p3 = line_plane(fc(right1), fc(right2) - fc(right1), c0, BM, c0);
      const V Hp = p3 / norm(p3);

      const double hm_dist = gc_distance(c0, Hm);
      const double b12m = gc_distance(fc(left1), fc(left2));
      const double hm2 = gc_distance(fc(left2), Hm);
      const double hm1 = gc_distance(fc(left1), Hm);
      g.h_minus[s] = hm_dist;
      g.ff_minus[2 * (size_t)s + 0] = left1;
      g.ff_minus[2 * (size_t)s + 1] = left2;
      g.beta_minus[2 * (size_t)s + 0] = hm2 / b12m;
      g.beta_minus[2 * (size_t)s + 1] = hm1 / b12m;

      const double hp_dist = gc_distance(c0, Hp);
      const double b12p = gc_distance(fc(right1), fc(right2));
      const double hp2 = gc_distance(fc(right2), Hp);
      const double hp1 = gc_distance(fc(right1), Hp);
      g.h_plus[s] = hp_dist;
      g.ff_plus[2 * (size_t)s + 0] = right1;
      g.ff_plus[2 * (size_t)s + 1] = right2;
      g.beta_plus[2 * (size_t)s + 0] = hp2 / b12p;
      g.beta_plus[2 * (size_t)s + 1] = hp1 / b12p;
    }
  }

  // h0: minimum great-circle edge length (MUSCL_base.hpp:63-91); the
  // minimum is exact in any order
  double h0 = 10;
#pragma omp parallel for schedule(static) reduction(min : h0)
  for (int f = 0; f < nf; ++f) {
    const int n = off[f + 1] - off[f];
    for (int j = 0; j < n; ++j) {
      const int a = fv[off[f] + j];
      const int b = fv[off[f] + ((j < n - 1) ? j + 1 : 0)];
      const double d = gc_distance(vtx(a), vtx(b));
      if (d < h0) h0 = d;
    }
  }
  g.h0 = h0;
  // arc / chord ratio of face 0's edge (1, 2) used by res2d
  // (MUSCL_base.hpp:242)
  {
    const V a = vtx(fv[off[0] + 1]);
    const V b = vtx(fv[off[0] + 2]);
    g.round_diff = gc_distance(a, b) / norm(a - b);
  }
  return g;
}

}  // namespace splash
