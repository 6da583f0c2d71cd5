// ref_recover.cpp -- TEST INFRASTRUCTURE ONLY (built into oracle/_ref/ by
// build_oracle.py where the reference checkout exists; never shipped).
//
// Compiles the reference's own source/recover.h (barycentric, locate,
// recover) and source/weighting.h (weighting_vertices_with_area) from the
// reference checkout, unchanged, against minimal stand-ins for the CGAL and
// Boost names those templates use, so their arithmetic and loop order run
// here as written.  The stand-ins model one indexed triangle mesh: face f
// lists vertices tri[3f..3f+2] in the order vertices_around_face(halfedge(f))
// visits them; vertex v has parameter-space point uv[v] and surface point
// xyz[v].  CGAL itself is not in the reference checkout; the two CGAL
// computations the headers call are restated from CGAL's published kernel
// (CGAL 5.x, Simple_cartesian<double> as main.cpp:75 uses):
//   * centroid(p, q, r) = ((p.x + q.x + r.x) / 3, (p.y + q.y + r.y) / 3);
//   * PMP::face_area(f) = sqrt(squared_area(source(h), target(h),
//     target(next(h)))) for h = halfedge(f), squared_area = |cross(q - p,
//     r - p)|^2 / 4; with vertices_around_face(h) starting at target(h) the
//     three points are (tri[3f+2], tri[3f], tri[3f+1]).
#include <math.h>
#include <array>
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

namespace boost {
template <class G> struct graph_traits {
  typedef typename G::vertex_descriptor vertex_descriptor;
  typedef typename G::halfedge_descriptor halfedge_descriptor;
  typedef typename G::face_descriptor face_descriptor;
  typedef typename G::edge_descriptor edge_descriptor;
};
template <class K, class V> using unordered_map = std::unordered_map<K, V>;
}  // namespace boost

struct Kernel {
  typedef double FT;
  struct Point_2 {
    double px = 0, py = 0;
    Point_2() {}
    Point_2(double x, double y) : px(x), py(y) {}
    double x() const { return px; }
    double y() const { return py; }
  };
  struct Point_3 {
    double px = 0, py = 0, pz = 0;
    Point_3() {}
    Point_3(double x, double y, double z) : px(x), py(y), pz(z) {}
    double x() const { return px; }
    double y() const { return py; }
    double z() const { return pz; }
  };
};
typedef Kernel::Point_2 Point_2;
typedef Kernel::Point_3 Point_3;

struct FaceD {
  int i = -1;  // -1: no face (a location that never succeeded)
};
struct HalfD {
  int f;
};

struct IdxMesh {
  typedef int vertex_descriptor;
  typedef HalfD halfedge_descriptor;
  typedef FaceD face_descriptor;
  typedef int edge_descriptor;
  const double *uv, *xyz;
  int nv;
  const int *tri;
  int nt;
  std::vector<FaceD> faces() const {
    std::vector<FaceD> r(nt);
    for (int i = 0; i < nt; ++i) r[i].i = i;
    return r;
  }
  std::vector<int> vertices() const {
    std::vector<int> r(nv);
    for (int i = 0; i < nv; ++i) r[i] = i;
    return r;
  }
  // vertex nv stands for the vertices of "no face": NaN coordinates
  Point_2 point(int v) const {
    return v < nv ? Point_2(uv[2 * v], uv[2 * v + 1]) : Point_2(NAN, NAN);
  }
};
typedef IdxMesh Mesh2D;

inline HalfD halfedge(FaceD f, const IdxMesh &) { return HalfD{f.i}; }
inline std::vector<int> vertices_around_face(HalfD h, const IdxMesh &m) {
  if (h.f < 0) return {m.nv, m.nv, m.nv};
  return {m.tri[3 * h.f], m.tri[3 * h.f + 1], m.tri[3 * h.f + 2]};
}

struct IdMap {  // vertex_3d_to_2d / vertex_2d_to_3d: the identity
  int operator[](int v) const { return v; }
};
inline int get(const IdMap &, int v) { return v; }

struct PointMap {
  const IdxMesh *m;
};
inline Point_3 get(const PointMap &pm, int v) {
  const IdxMesh &m = *pm.m;
  return v < m.nv ? Point_3(m.xyz[3 * v], m.xyz[3 * v + 1], m.xyz[3 * v + 2])
                  : Point_3(NAN, NAN, NAN);
}

struct WeightMap {
  std::vector<double> w;
  double &operator[](int v) { return w[v]; }
};
inline void put(WeightMap &m, int v, double x) { m.w[v] = x; }

struct ResultMesh {
  std::vector<Point_3> v;
  std::vector<std::array<int, 3>> f;
  int add_vertex(const Point_3 &p) {
    v.push_back(p);
    return (int)v.size() - 1;
  }
  int add_face(const std::vector<int> &vs) {
    f.push_back({vs[0], vs[1], vs[2]});
    return (int)f.size() - 1;
  }
};

namespace CGAL {
struct vertex_point_t {};
static const vertex_point_t vertex_point{};
inline PointMap get(vertex_point_t, const IdxMesh &m) { return PointMap{&m}; }

inline Point_2 centroid(const Point_2 &p, const Point_2 &q, const Point_2 &r) {
  return Point_2((p.x() + q.x() + r.x()) / 3, (p.y() + q.y() + r.y()) / 3);
}

namespace Polygon_mesh_processing {
inline double face_area(FaceD f, const IdxMesh &m) {
  const int *t = m.tri + 3 * f.i;
  const double *p = m.xyz + 3 * t[2], *q = m.xyz + 3 * t[0], *r = m.xyz + 3 * t[1];
  const double dqx = q[0] - p[0], dqy = q[1] - p[1], dqz = q[2] - p[2];
  const double drx = r[0] - p[0], dry = r[1] - p[1], drz = r[2] - p[2];
  const double vx = dqy * drz - dqz * dry;
  const double vy = dqz * drx - dqx * drz;
  const double vz = dqx * dry - dqy * drx;
  return std::sqrt((vx * vx + vy * vy + vz * vz) / 4);
}
template <class V, class M> Point_3 compute_vertex_normal(V, const M &);  // not used
}  // namespace Polygon_mesh_processing
namespace Surface_mesh_parameterization {}
}  // namespace CGAL

using CGAL::get;

#include "weighting.h"
#include "recover.h"

struct CdtPoint {
  double _p[2];
};
struct CdtTri {
  int _v[3];
};

extern "C" int refr_recover(const double *uv, const double *xyz, int nv, const int *tri, int nt,
                            const double *pts, int np, const int *fixed, int nfixed,
                            const int *cdt, int nc, double *out_xyz, unsigned char *keep) {
  IdxMesh m{uv, xyz, nv, tri, nt};
  std::vector<CdtPoint> point(np);
  for (int i = 0; i < np; ++i) point[i] = CdtPoint{{pts[2 * i], pts[2 * i + 1]}};
  std::vector<CdtTri> triangle(nc);
  for (int t = 0; t < nc; ++t) triangle[t] = CdtTri{{cdt[3 * t], cdt[3 * t + 1], cdt[3 * t + 2]}};
  std::vector<int> c_points(fixed, fixed + nfixed);
  ResultMesh res;
  recover(m, m, IdMap{}, point, triangle, c_points, res);
  if ((int)res.v.size() != np) return -1;
  for (int i = 0; i < np; ++i) {
    out_xyz[3 * i] = res.v[i].x();
    out_xyz[3 * i + 1] = res.v[i].y();
    out_xyz[3 * i + 2] = res.v[i].z();
  }
  // the faces were added in triangle order, vertex ids = point indices
  size_t k = 0;
  for (int t = 0; t < nc; ++t) {
    const bool hit = k < res.f.size() && res.f[k][0] == cdt[3 * t] &&
                     res.f[k][1] == cdt[3 * t + 1] && res.f[k][2] == cdt[3 * t + 2];
    keep[t] = hit ? 1 : 0;
    k += hit;
  }
  return k == res.f.size() ? 0 : -2;
}

extern "C" int refr_weights(const double *uv, const double *xyz, int nv, const int *tri, int nt,
                            double *weight) {
  IdxMesh m{uv, xyz, nv, tri, nt};
  WeightMap w;
  w.w.assign(nv, 0.0);
  weighting_vertices_with_area(m, m, IdMap{}, w);
  for (int v = 0; v < nv; ++v) weight[v] = w.w[v];
  return 0;
}
