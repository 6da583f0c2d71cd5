// lift.cu -- from parameter space back to the surface: the reference's
// recover() (recover.h:98-157) and weighting_vertices_with_area()
// (weighting.h:38-97) on the GPU, with the reference's results.
//
// Point location.  The reference's locate() (recover.h:64-85) tests a 2D
// point against every parameter-space face in index order with the FP64
// barycentric of recover.h:30-52 and takes the first face whose three weights
// are all >= 0: O(points x faces) on one core.  Here each face is classified
// once:
//   * skip   -- denominator exactly 0: the reference returns weights -1, so
//               the face never matches;
//   * local  -- finite, denominator > 0 and conditioning
//               kappa = d00*d11/denom <= 2^40: binned by its bounding box
//               enlarged by max(1e-6, kappa 2^-45) of its width + height into
//               a uniform grid over the faces;
//   * global -- everything else (non-finite coordinates, negative
//               denominator, kappa above 2^40, boxes over more than 1024
//               cells): tested by every point.
// A point scans its grid cell's list (sorted, so the first face that passes
// ends the scan) and the global list, keeps the smallest face index whose
// test passes -- the reference's first hit -- and a point with a non-finite
// coordinate tests every face in order.  The test is the
// reference's arithmetic with every product, sum and quotient rounded once
// (the reference's host build has no fused multiply-add), so the weights are
// bit-identical.  Why the enlarged box cannot drop a match for a local face:
// for a point at distance D outside the face, the rounding error of each
// computed weight is at most about 32 u kappa |p - p1| / h (u = 2^-53, h the
// face's height over the weight's edge) while the exact weight is -D / h, so
// a false "inside" needs D < 32 u kappa (D + L), L the face's size, i.e.
// D < 2^-48 kappa L / (1 - 2^-48 kappa): at kappa <= 2^20 below 4e-9 L, far
// inside the 1e-6 margin, and below the kappa 2^-45 margin by a factor 8 up
// to kappa = 2^40.
//
// Points whose location fails keep the previous point's face and weights in
// the reference (f_loc is not reset between calls, recover.h:120-134): such a
// point gets the lifted position of the nearest earlier located point, found
// by a prefix maximum; with none (no earlier located point, where the
// reference reads an uninitialised location) it gets NaN.
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace cvtgb {

namespace {

constexpr double kMaxCond = 1099511627776.0;  // 2^40
constexpr double kMargin = 1e-6;
constexpr int kMaxCellsPerFace = 1024;
constexpr int kMaxGrid = 4096;
constexpr int kLocal = 1, kGlobal = 2;

// recover.h:30-52 on a face whose point-independent terms are precomputed
// (the same expressions, so the same values).
struct LiftFace {
  double x1, y1, v0x, v0y, v1x, v1y, d00, d01, d11, denom;
};

struct __align__(32) Box {
  double x, y, z, w;  // min x, min y, max x, max y
};

struct Grid {
  double x0, y0, x1, y1, ix, iy;  // covered box and cells per unit
  int gx, gy;
};

__device__ __forceinline__ double dot_rn(double ax, double ay, double bx, double by) {
  return __dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by));
}

// barycentric(x1, y1, x2, y2, x3, y3, x0, y0, _w[0], _w[1], _w[2]): the
// reference's output slots are (w3, w1, w2), so _w = (1 - w1 - w2, w1, w2).
__device__ __forceinline__ bool face_test(const LiftFace &f, double px, double py, double &c,
                                          double &a, double &b) {
  if (f.denom == 0) return false;  // all weights -1
  const double v2x = __dsub_rn(px, f.x1), v2y = __dsub_rn(py, f.y1);
  const double d20 = dot_rn(v2x, v2y, f.v0x, f.v0y);
  const double d21 = dot_rn(v2x, v2y, f.v1x, f.v1y);
  a = __ddiv_rn(__dsub_rn(__dmul_rn(f.d11, d20), __dmul_rn(f.d01, d21)), f.denom);
  b = __ddiv_rn(__dsub_rn(__dmul_rn(f.d00, d21), __dmul_rn(f.d01, d20)), f.denom);
  c = __dsub_rn(__dsub_rn(1.0, a), b);
  return !(c < 0 || a < 0 || b < 0);
}

// RN(num / denom) < 0 for denom > 0, decided without dividing: num < 0 and
// the quotient too large to round to -0 (|q| >= 2^-1074 when denom <= 1;
// otherwise |num| >= denom 2^-1000 keeps it far from underflow).  False
// means "divide to know".
__device__ __forceinline__ bool quot_negative(double num, double denom) {
  return num < 0 && (denom <= 1.0 || -num >= __dmul_rn(denom, 0x1p-1000));
}

// face_test for a face with a finite denominator > 0 and a finite point: the
// same results, but a weight whose numerator already shows it negative
// rejects the face before the two divisions (FP64 issue is scarce on GB300).
__device__ __forceinline__ bool face_test_local(const LiftFace &f, double px, double py,
                                                double &c, double &a, double &b) {
  const double v2x = __dsub_rn(px, f.x1), v2y = __dsub_rn(py, f.y1);
  const double d20 = dot_rn(v2x, v2y, f.v0x, f.v0y);
  const double d21 = dot_rn(v2x, v2y, f.v1x, f.v1y);
  const double na = __dsub_rn(__dmul_rn(f.d11, d20), __dmul_rn(f.d01, d21));
  if (quot_negative(na, f.denom)) return false;
  const double nb = __dsub_rn(__dmul_rn(f.d00, d21), __dmul_rn(f.d01, d20));
  if (quot_negative(nb, f.denom)) return false;
  a = __ddiv_rn(na, f.denom);
  b = __ddiv_rn(nb, f.denom);
  c = __dsub_rn(__dsub_rn(1.0, a), b);
  return !(c < 0 || a < 0 || b < 0);
}

// Order-preserving 64-bit keys of doubles for atomic min / max.
__device__ __forceinline__ long long dkey(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : b ^ 0x7fffffffffffffffLL;
}
__host__ __device__ inline double dunkey(long long k) {
  const long long b = k >= 0 ? k : k ^ 0x7fffffffffffffffLL;
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
}

__device__ __forceinline__ int cell_x(const Grid &g, double x) {
  return min(g.gx - 1, (int)__dmul_rn(__dsub_rn(x, g.x0), g.ix));
}
__device__ __forceinline__ int cell_y(const Grid &g, double y) {
  return min(g.gy - 1, (int)__dmul_rn(__dsub_rn(y, g.y0), g.iy));
}

// Face i: its precomputed test terms, class and enlarged box; true (with the
// box in e) for a local face.
__device__ __forceinline__ bool classify_face(const double *__restrict__ uv, int nv,
                                              const int *__restrict__ tri, int i,
                                              LiftFace *faces, Box *ebox, unsigned char *kind,
                                              int *err, Box &e) {
  const int t0 = tri[3 * i], t1 = tri[3 * i + 1], t2 = tri[3 * i + 2];
  LiftFace f{};
  if (t0 < 0 || t1 < 0 || t2 < 0 || t0 >= nv || t1 >= nv || t2 >= nv) {
    atomicOr(err, 1);
    faces[i] = f;  // denom 0: never matches
    kind[i] = 0;
    return false;
  }
  const double x1 = uv[2 * t0], y1 = uv[2 * t0 + 1];
  const double x2 = uv[2 * t1], y2 = uv[2 * t1 + 1];
  const double x3 = uv[2 * t2], y3 = uv[2 * t2 + 1];
  f.x1 = x1;
  f.y1 = y1;
  f.v0x = __dsub_rn(x2, x1);
  f.v0y = __dsub_rn(y2, y1);
  f.v1x = __dsub_rn(x3, x1);
  f.v1y = __dsub_rn(y3, y1);
  f.d00 = dot_rn(f.v0x, f.v0y, f.v0x, f.v0y);
  f.d01 = dot_rn(f.v0x, f.v0y, f.v1x, f.v1y);
  f.d11 = dot_rn(f.v1x, f.v1y, f.v1x, f.v1y);
  f.denom = __dsub_rn(__dmul_rn(f.d00, f.d11), __dmul_rn(f.d01, f.d01));
  faces[i] = f;
  if (f.denom == 0) {
    kind[i] = 0;
    return false;
  }
  const double xmin = fmin(x1, fmin(x2, x3)), xmax = fmax(x1, fmax(x2, x3));
  const double ymin = fmin(y1, fmin(y2, y3)), ymax = fmax(y1, fmax(y2, y3));
  const bool finite = isfinite(x1) && isfinite(y1) && isfinite(x2) && isfinite(y2) &&
                      isfinite(x3) && isfinite(y3) && isfinite(f.denom);
  const double cond = f.d00 * f.d11 / f.denom;
  if (!finite || !(f.denom > 0) || !(cond <= kMaxCond)) {
    kind[i] = kGlobal;
    ebox[i] = Box{-INFINITY, -INFINITY, INFINITY, INFINITY};
    return false;
  }
  const double m = fmax(kMargin, cond * 0x1p-45) * ((xmax - xmin) + (ymax - ymin));
  e = Box{xmin - m, ymin - m, xmax + m, ymax + m};
  if (!(isfinite(e.x) && isfinite(e.y) && isfinite(e.z) && isfinite(e.w))) {
    kind[i] = kGlobal;
    ebox[i] = Box{-INFINITY, -INFINITY, INFINITY, INFINITY};
    return false;
  }
  kind[i] = kLocal;
  ebox[i] = e;
  return true;
}

__device__ __forceinline__ long long warp_min64(long long v) {
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ long long warp_max64(long long v) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Per face: the precomputed test terms, the class, the enlarged box and the
// union of the local faces' boxes (keys[0..3] = min x, min y, max x, max y;
// one atomic per warp).
__global__ void __launch_bounds__(256) k_lift_faces(const double *__restrict__ uv, int nv,
                                                    const int *__restrict__ tri, int nt,
                                                    LiftFace *faces, Box *ebox,
                                                    unsigned char *kind, long long *keys,
                                                    int *nlocal, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool local = false;
  Box e{0, 0, 0, 0};
  if (i < nt) local = classify_face(uv, nv, tri, i, faces, ebox, kind, err, e);
  const unsigned lanes = __ballot_sync(0xffffffffu, local);
  if (!lanes) return;
  const long long k0 = warp_min64(local ? dkey(e.x) : LLONG_MAX);
  const long long k1 = warp_min64(local ? dkey(e.y) : LLONG_MAX);
  const long long k2 = warp_max64(local ? dkey(e.z) : LLONG_MIN);
  const long long k3 = warp_max64(local ? dkey(e.w) : LLONG_MIN);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&keys[0], k0);
    atomicMin(&keys[1], k1);
    atomicMax(&keys[2], k2);
    atomicMax(&keys[3], k3);
    atomicAdd(nlocal, __popc(lanes));
  }
}

// Local faces: count their cells, or move them to the global list when their
// box covers more than kMaxCellsPerFace cells; global faces join the list.
__global__ void k_lift_count(const Box *__restrict__ ebox, unsigned char *kind, int nt, Grid g,
                             int *cell_count, int *glist, int *gcount,
                             unsigned long long *entries) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  int k = kind[i];
  if (k == kLocal) {
    const Box e = ebox[i];
    const int cx0 = cell_x(g, e.x), cx1 = cell_x(g, e.z);
    const int cy0 = cell_y(g, e.y), cy1 = cell_y(g, e.w);
    if ((long long)(cx1 - cx0 + 1) * (cy1 - cy0 + 1) > kMaxCellsPerFace) {
      kind[i] = k = kGlobal;
    } else {
      atomicAdd(entries, (unsigned long long)((cx1 - cx0 + 1) * (cy1 - cy0 + 1)));
      for (int cy = cy0; cy <= cy1; ++cy)
        for (int cx = cx0; cx <= cx1; ++cx) atomicAdd(&cell_count[cy * g.gx + cx], 1);
      return;
    }
  }
  if (k == kGlobal) glist[atomicAdd(gcount, 1)] = i;
}

__global__ void k_lift_scatter(const Box *__restrict__ ebox,
                               const unsigned char *__restrict__ kind, int nt, Grid g,
                               int *cursor, int *list) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt || kind[i] != kLocal) return;
  const Box e = ebox[i];
  const int cx0 = cell_x(g, e.x), cx1 = cell_x(g, e.z);
  const int cy0 = cell_y(g, e.y), cy1 = cell_y(g, e.w);
  for (int cy = cy0; cy <= cy1; ++cy)
    for (int cx = cx0; cx <= cx1; ++cx) list[atomicAdd(&cursor[cy * g.gx + cx], 1)] = i;
}

// Each cell's list in ascending face order (one thread per cell; lists are
// a few faces long).
__global__ void k_lift_sort(const int *__restrict__ offset, int ncell, int *list) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int l0 = offset[c], l1 = offset[c + 1];
  for (int k = l0 + 1; k < l1; ++k) {
    const int x = list[k];
    int j = k - 1;
    while (j >= l0 && list[j] > x) {
      list[j + 1] = list[j];
      --j;
    }
    list[j + 1] = x;
  }
}

struct Locator {
  const LiftFace *faces;
  const Box *ebox;
  const int *offset, *list, *glist;
  int ngl, nt;
  Grid g;

  // locate() (recover.h:64-85): the first face in index order whose weights
  // are all >= 0, or -1.
  __device__ int find(double px, double py, double &c, double &a, double &b) const {
    double wc, wa, wb;
    if (!isfinite(px) || !isfinite(py)) {
      for (int i = 0; i < nt; ++i)
        if (face_test(faces[i], px, py, wc, wa, wb)) {
          c = wc, a = wa, b = wb;
          return i;
        }
      return -1;
    }
    int best = INT_MAX;
    if (g.gx > 0 && px >= g.x0 && px <= g.x1 && py >= g.y0 && py <= g.y1) {
      // the cell's faces in ascending order: the first that passes is the answer
      const int cell = cell_y(g, py) * g.gx + cell_x(g, px);
      const int l1 = offset[cell + 1];
      for (int k = offset[cell]; k < l1; ++k) {
        const int i = list[k];
        const Box e = ebox[i];
        if (px < e.x || px > e.z || py < e.y || py > e.w) continue;
        if (face_test_local(faces[i], px, py, wc, wa, wb)) {
          best = i, c = wc, a = wa, b = wb;
          break;
        }
      }
    }
    for (int k = 0; k < ngl; ++k) {
      const int i = glist[k];
      if (i >= best) continue;
      const Box e = ebox[i];
      if (px < e.x || px > e.z || py < e.y || py > e.w) continue;
      if (face_test(faces[i], px, py, wc, wa, wb)) best = i, c = wc, a = wa, b = wb;
    }
    return best == INT_MAX ? -1 : best;
  }
};

// One thread per query: the np - nfixed free points (locate + lift,
// recover.h:120-134), the nfixed constraint points (their mesh vertex,
// recover.h:137-139), then the nc triangles (keep when the centroid
// locates, recover.h:141-156).
__global__ void k_lift_locate(Locator L, const double *__restrict__ xyz, int nv,
                              const int *__restrict__ tri, const double *__restrict__ pts, int np,
                              const int *__restrict__ fixed_vertex, int nfixed,
                              const int *__restrict__ cdt, int nc, double *out_xyz, int *out_face,
                              unsigned char *keep, int *err) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nfree = np - nfixed;
  if (q < nfree) {
    const int i = (int)q;
    double c = 0, a = 0, b = 0;
    const int f = L.find(pts[2 * i], pts[2 * i + 1], c, a, b);
    out_face[i] = f;
    if (f < 0) return;  // filled by k_lift_stale
    const int v[3] = {tri[3 * f], tri[3 * f + 1], tri[3 * f + 2]};
    const double w[3] = {c, a, b};
    for (int d = 0; d < 3; ++d) {
      double s = 0.0;
      for (int j = 0; j < 3; ++j) s = __dadd_rn(s, __dmul_rn(xyz[3 * v[j] + d], w[j]));
      out_xyz[3 * i + d] = s;
    }
  } else if (q < np) {
    const int i = (int)q;
    const int v = fixed_vertex[i - nfree];
    out_face[i] = -1;
    if (v < 0 || v >= nv) {
      atomicOr(err, 1);
      for (int d = 0; d < 3; ++d) out_xyz[3 * i + d] = NAN;
      return;
    }
    for (int d = 0; d < 3; ++d) out_xyz[3 * i + d] = xyz[3 * v + d];
  } else if (q < (long long)np + nc) {
    const int t = (int)(q - np);
    const int p0 = cdt[3 * t], p1 = cdt[3 * t + 1], p2 = cdt[3 * t + 2];
    if (p0 < 0 || p1 < 0 || p2 < 0 || p0 >= np || p1 >= np || p2 >= np) {
      atomicOr(err, 1);
      keep[t] = 0;
      return;
    }
    // CGAL::centroid of three Point_2: ((p + q + r) / 3) per coordinate
    const double cx = __ddiv_rn(__dadd_rn(__dadd_rn(pts[2 * p0], pts[2 * p1]), pts[2 * p2]), 3.0);
    const double cy =
        __ddiv_rn(__dadd_rn(__dadd_rn(pts[2 * p0 + 1], pts[2 * p1 + 1]), pts[2 * p2 + 1]), 3.0);
    double c, a, b;
    keep[t] = L.find(cx, cy, c, a, b) >= 0 ? 1 : 0;
  }
}

constexpr int kScanBlock = 1024;

__device__ __forceinline__ int block_max_scan(int v, int *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = max(v, u);
  }
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    int s = sh[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s = max(s, u);
    }
    sh[lane] = s;
  }
  __syncthreads();
  return w > 0 ? max(v, sh[w - 1]) : v;
}

// Last located free point of each block of kScanBlock points.
__global__ void __launch_bounds__(kScanBlock) k_lift_last(const int *__restrict__ face, int nfree,
                                                          int *block_last) {
  __shared__ int sh[32];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int v = (i < nfree && face[i] >= 0) ? i : -1;
  const int s = block_max_scan(v, sh);
  if (threadIdx.x == kScanBlock - 1) block_last[blockIdx.x] = s;
}

// Unlocated free points copy the nearest earlier located point's result.
__global__ void __launch_bounds__(kScanBlock) k_lift_stale(const int *__restrict__ face, int nfree,
                                                           const int *__restrict__ block_last,
                                                           double *out_xyz) {
  __shared__ int sh[32];
  __shared__ int prev;
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const bool miss = i < nfree && face[i] < 0;
  if (!__syncthreads_or(miss)) return;
  int p = -1;
  for (int k = threadIdx.x; k < (int)blockIdx.x; k += kScanBlock) p = max(p, block_last[k]);
  for (int o = 16; o > 0; o >>= 1) p = max(p, __shfl_xor_sync(0xffffffffu, p, o));
  if (threadIdx.x == 0) prev = -1;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) atomicMax(&prev, p);
  __syncthreads();
  const int v = (i < nfree && face[i] >= 0) ? i : -1;
  const int src = max(prev, block_max_scan(v, sh));
  if (!miss) return;
  for (int d = 0; d < 3; ++d) out_xyz[3 * i + d] = src >= 0 ? out_xyz[3 * src + d] : NAN;
}

// weighting_vertices_with_area (weighting.h:38-97).
// Per face: its 3D area as CGAL's PMP::face_area computes it -- the squared
// area of (source(h), target(h), target(next(h))) for h = halfedge(f), i.e.
// (t2, t0, t1) when the face lists its vertices as vertices_around_face(h)
// does, as |cross(q - p, r - p)|^2 / 4, then its square root -- and its
// parameter-space area get_area (weighting.h:34-36).
__global__ void k_face_areas(const double *__restrict__ uv, const double *__restrict__ xyz,
                             int nv, const int *__restrict__ tri, int nt, double2 *area,
                             int *vcount, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const int t0 = tri[3 * i], t1 = tri[3 * i + 1], t2 = tri[3 * i + 2];
  if (t0 < 0 || t1 < 0 || t2 < 0 || t0 >= nv || t1 >= nv || t2 >= nv) {
    atomicOr(err, 1);
    area[i] = make_double2(0, 0);
    return;
  }
  const double *p = xyz + 3 * t2, *q = xyz + 3 * t0, *r = xyz + 3 * t1;
  const double dqx = __dsub_rn(q[0], p[0]), dqy = __dsub_rn(q[1], p[1]),
               dqz = __dsub_rn(q[2], p[2]);
  const double drx = __dsub_rn(r[0], p[0]), dry = __dsub_rn(r[1], p[1]),
               drz = __dsub_rn(r[2], p[2]);
  const double vx = __dsub_rn(__dmul_rn(dqy, drz), __dmul_rn(dqz, dry));
  const double vy = __dsub_rn(__dmul_rn(dqz, drx), __dmul_rn(dqx, drz));
  const double vz = __dsub_rn(__dmul_rn(dqx, dry), __dmul_rn(dqy, drx));
  const double sq = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
  const double a3 = __dsqrt_rn(__ddiv_rn(sq, 4.0));
  // get_area(A, B, C) = |cross(B - A, C - A)| / 2, cross(P, Q) = P.x Q.y - Q.x P.y
  const double ax = uv[2 * t0], ay = uv[2 * t0 + 1];
  const double bx = __dsub_rn(uv[2 * t1], ax), by = __dsub_rn(uv[2 * t1 + 1], ay);
  const double cx = __dsub_rn(uv[2 * t2], ax), cy = __dsub_rn(uv[2 * t2 + 1], ay);
  const double a2 = __ddiv_rn(fabs(__dsub_rn(__dmul_rn(bx, cy), __dmul_rn(cx, by))), 2.0);
  area[i] = make_double2(a3, a2);
  atomicAdd(&vcount[t0], 1);
  atomicAdd(&vcount[t1], 1);
  atomicAdd(&vcount[t2], 1);
}

__global__ void k_vertex_faces(const int *__restrict__ tri, int nt, int nv, int *cursor,
                               int *inc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const int t0 = tri[3 * i], t1 = tri[3 * i + 1], t2 = tri[3 * i + 2];
  if (t0 < 0 || t1 < 0 || t2 < 0 || t0 >= nv || t1 >= nv || t2 >= nv) return;
  inc[atomicAdd(&cursor[t0], 1)] = i;
  inc[atomicAdd(&cursor[t1], 1)] = i;
  inc[atomicAdd(&cursor[t2], 1)] = i;
}

// Per vertex: the incident faces' areas summed in face order (the order the
// reference's face loops add them), the ratio, and the running maximum of
// the ratios that are at most 1e10.
__global__ void k_vertex_weight(const int *__restrict__ offset, int *inc,
                                const double2 *__restrict__ area, int nv, double *weight,
                                unsigned char *over, unsigned long long *mx_bits) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int l0 = offset[v], l1 = offset[v + 1];
  for (int k = l0 + 1; k < l1; ++k) {  // this vertex's segment, sorted in place
    const int x = inc[k];
    int j = k - 1;
    while (j >= l0 && inc[j] > x) {
      inc[j + 1] = inc[j];
      --j;
    }
    inc[j + 1] = x;
  }
  double s3 = 0.0, s2 = 0.0;
  for (int k = l0; k < l1; ++k) {
    const double2 a = area[inc[k]];
    s3 = __dadd_rn(s3, a.x);
    s2 = __dadd_rn(s2, a.y);
  }
  const double w = __ddiv_rn(s3, s2);
  if (w > 1e10) {
    over[v] = 1;
    return;
  }
  over[v] = 0;
  weight[v] = w;
  if (w > 0) atomicMax(mx_bits, (unsigned long long)__double_as_longlong(w));
}

__global__ void k_vertex_fill(const unsigned char *__restrict__ over, int nv,
                              const unsigned long long *__restrict__ mx_bits, double *weight) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < nv && over[v]) weight[v] = __longlong_as_double((long long)*mx_bits);
}

inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

#define LCK(call)                                  \
  do {                                             \
    if ((call) != cudaSuccess) return GCVT_ERR_CUDA; \
  } while (0)
#define TAKE(ptr, T, count)                                   \
  do {                                                        \
    if (!((ptr) = sc.take<T>((size_t)(count)))) return GCVT_ERR_ALLOC; \
  } while (0)

// Device-pointer core of gcvt_lift.
int lift_device(Scratch &sc, const double *uv, const double *xyz, int nv, const int *tri, int nt,
                const double *pts, int np, int nfixed, const int *fixed_vertex, const int *cdt,
                int nc, double *out_xyz, int *out_face, unsigned char *keep) {
  LiftFace *faces;
  Box *ebox;
  unsigned char *kind;
  int *glist, *scal, *cnt, *off, *cur, *list, *face, *blast;
  long long *keys;
  TAKE(faces, LiftFace, nt);
  TAKE(ebox, Box, nt);
  TAKE(kind, unsigned char, nt);
  TAKE(glist, int, nt);
  TAKE(keys, long long, 4);
  TAKE(scal, int, 8);  // err, nlocal, gcount; list entries (64-bit) at byte 16
  int *err = scal, *nlocal = scal + 1, *gcount = scal + 2;
  unsigned long long *entries = (unsigned long long *)(scal + 4);
  const long long init[4] = {LLONG_MAX, LLONG_MAX, LLONG_MIN, LLONG_MIN};
  LCK(cudaMemcpy(keys, init, sizeof init, cudaMemcpyHostToDevice));
  LCK(cudaMemset(scal, 0, 32));
  if (nt > 0) {
    k_lift_faces<<<blocks(nt, 256), 256>>>(uv, nv, tri, nt, faces, ebox, kind, keys, nlocal, err);
    LCK(cudaGetLastError());
  }
  long long hk[4];
  int hs[4];
  LCK(cudaMemcpy(hk, keys, sizeof hk, cudaMemcpyDeviceToHost));
  LCK(cudaMemcpy(hs, scal, sizeof hs, cudaMemcpyDeviceToHost));
  Grid g{};
  if (hs[1] > 0) {
    g.x0 = dunkey(hk[0]);
    g.y0 = dunkey(hk[1]);
    g.x1 = dunkey(hk[2]);
    g.y1 = dunkey(hk[3]);
    const double ex = g.x1 - g.x0, ey = g.y1 - g.y0, e = fmax(ex, ey);
    // about one cell per local face, square cells
    const double cs = sqrt(fmax(ex * ey, e * e * 1e-6) / hs[1]);
    g.gx = ex > 0 && cs > 0 ? (int)fmin(kMaxGrid, fmax(1.0, ceil(ex / cs))) : 1;
    g.gy = ey > 0 && cs > 0 ? (int)fmin(kMaxGrid, fmax(1.0, ceil(ey / cs))) : 1;
    g.ix = ex > 0 ? g.gx / ex : 0.0;
    g.iy = ey > 0 ? g.gy / ey : 0.0;
  }
  const int ncell = g.gx * g.gy;
  TAKE(cnt, int, ncell);
  TAKE(off, int, ncell + 1);
  TAKE(cur, int, ncell);
  LCK(cudaMemset(cnt, 0, (size_t)ncell * sizeof(int)));
  if (nt > 0) {
    k_lift_count<<<blocks(nt, 256), 256>>>(ebox, kind, nt, g, cnt, glist, gcount, entries);
    LCK(cudaGetLastError());
  }
  unsigned long long nentries = 0;
  LCK(cudaMemcpy(&nentries, entries, sizeof nentries, cudaMemcpyDeviceToHost));
  if (nentries > (unsigned long long)INT_MAX) return GCVT_ERR_SIZE;
  int total = 0;
  if (ncell > 0) {
    LCK(launch_scan(cnt, ncell, off, cur, 0));
    LCK(cudaMemcpy(&total, off + ncell, sizeof(int), cudaMemcpyDeviceToHost));
  }
  TAKE(list, int, total);
  if (nt > 0 && ncell > 0) {
    k_lift_scatter<<<blocks(nt, 256), 256>>>(ebox, kind, nt, g, cur, list);
    LCK(cudaGetLastError());
    k_lift_sort<<<blocks(ncell, 256), 256>>>(off, ncell, list);
    LCK(cudaGetLastError());
  }
  LCK(cudaMemcpy(hs, scal, sizeof hs, cudaMemcpyDeviceToHost));
  Locator L{faces, ebox, off, list, glist, hs[2], nt, g};
  face = out_face;
  if (!face) TAKE(face, int, np);
  const long long nq = (long long)np + nc;
  if (nq > 0) {
    k_lift_locate<<<blocks(nq, 128), 128>>>(L, xyz, nv, tri, pts, np, fixed_vertex, nfixed, cdt,
                                            nc, out_xyz, face, keep, err);
    LCK(cudaGetLastError());
  }
  const int nfree = np - nfixed;
  if (nfree > 0) {
    const int nb = blocks(nfree, kScanBlock);
    TAKE(blast, int, nb);
    k_lift_last<<<nb, kScanBlock>>>(face, nfree, blast);
    LCK(cudaGetLastError());
    k_lift_stale<<<nb, kScanBlock>>>(face, nfree, blast, out_xyz);
    LCK(cudaGetLastError());
  }
  LCK(cudaMemcpy(hs, scal, sizeof hs, cudaMemcpyDeviceToHost));
  return hs[0] ? GCVT_ERR_ARGUMENT : GCVT_OK;
}

int weights_device(Scratch &sc, const double *uv, const double *xyz, int nv, const int *tri,
                   int nt, double *weight) {
  double2 *area;
  int *cnt, *off, *cur, *inc, *scal;
  unsigned char *over;
  TAKE(area, double2, nt);
  TAKE(cnt, int, nv);
  TAKE(off, int, nv + 1);
  TAKE(cur, int, nv);
  TAKE(inc, int, (size_t)nt * 3);
  TAKE(over, unsigned char, nv);
  TAKE(scal, int, 4);
  int *err = scal;
  unsigned long long *mx = (unsigned long long *)(scal + 2);
  LCK(cudaMemset(scal, 0, 16));  // mx starts at +0.0
  LCK(cudaMemset(cnt, 0, (size_t)nv * sizeof(int)));
  if (nt > 0) {
    k_face_areas<<<blocks(nt, 256), 256>>>(uv, xyz, nv, tri, nt, area, cnt, err);
    LCK(cudaGetLastError());
  }
  LCK(launch_scan(cnt, nv, off, cur, 0));
  if (nt > 0) {
    k_vertex_faces<<<blocks(nt, 256), 256>>>(tri, nt, nv, cur, inc);
    LCK(cudaGetLastError());
  }
  k_vertex_weight<<<blocks(nv, 256), 256>>>(off, inc, area, nv, weight, over, mx);
  LCK(cudaGetLastError());
  k_vertex_fill<<<blocks(nv, 256), 256>>>(over, nv, mx, weight);
  LCK(cudaGetLastError());
  int herr = 0;
  LCK(cudaMemcpy(&herr, err, sizeof herr, cudaMemcpyDeviceToHost));
  return herr ? GCVT_ERR_ARGUMENT : GCVT_OK;
}

// Host buffers: copied into scratch, results copied back.
template <class T> int copy_in(Scratch &sc, const T *h, size_t count, const T **d) {
  T *p = sc.take<T>(count);
  if (!p) return GCVT_ERR_ALLOC;
  if (count && cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return GCVT_ERR_CUDA;
  *d = p;
  return GCVT_OK;
}
template <class T> int take_out(Scratch &sc, size_t count, T **d) {
  *d = sc.take<T>(count);
  return *d ? GCVT_OK : GCVT_ERR_ALLOC;
}

#define HCK(call)               \
  do {                          \
    const int rc_ = (call);     \
    if (rc_ != GCVT_OK) return rc_; \
  } while (0)

}  // namespace
}  // namespace cvtgb

using namespace cvtgb;

extern "C" int gcvt_lift(const double *uv, const double *xyz, int num_vertex,
                         const int32_t *triangle, int num_tri, const double *points,
                         int num_points, int num_fixed, const int32_t *fixed_vertex,
                         const int32_t *cdt, int num_cdt, double *out_xyz, int32_t *out_face,
                         uint8_t *keep, int mem) {
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (num_vertex < 0 || num_tri < 0 || num_points < 0 || num_fixed < 0 || num_cdt < 0 ||
      num_fixed > num_points)
    return GCVT_ERR_ARGUMENT;
  if ((num_vertex && (!uv || !xyz)) || (num_tri && !triangle) || (num_points && !points) ||
      (num_points && !out_xyz) || (num_fixed && !fixed_vertex) || (num_cdt && (!cdt || !keep)))
    return GCVT_ERR_ARGUMENT;
  if ((long long)num_tri * 3 > INT_MAX || (long long)num_points * 3 > INT_MAX ||
      (long long)num_cdt * 3 > INT_MAX)
    return GCVT_ERR_SIZE;
  Scratch sc;
  if (mem == GCVT_MEM_DEVICE)
    return lift_device(sc, uv, xyz, num_vertex, triangle, num_tri, points, num_points, num_fixed,
                       fixed_vertex, cdt, num_cdt, out_xyz, out_face, keep);
  const double *d_uv = nullptr, *d_xyz = nullptr, *d_pts = nullptr;
  const int *d_tri = nullptr, *d_fix = nullptr, *d_cdt = nullptr;
  double *d_out = nullptr;
  int *d_face = nullptr;
  unsigned char *d_keep = nullptr;
  HCK(copy_in(sc, uv, (size_t)num_vertex * 2, &d_uv));
  HCK(copy_in(sc, xyz, (size_t)num_vertex * 3, &d_xyz));
  HCK(copy_in(sc, triangle, (size_t)num_tri * 3, &d_tri));
  HCK(copy_in(sc, points, (size_t)num_points * 2, &d_pts));
  HCK(copy_in(sc, fixed_vertex, (size_t)num_fixed, &d_fix));
  HCK(copy_in(sc, cdt, (size_t)num_cdt * 3, &d_cdt));
  HCK(take_out(sc, (size_t)num_points * 3, &d_out));
  HCK(take_out(sc, (size_t)num_points, &d_face));
  HCK(take_out(sc, (size_t)num_cdt, &d_keep));
  const int rc = lift_device(sc, d_uv, d_xyz, num_vertex, d_tri, num_tri, d_pts, num_points,
                             num_fixed, d_fix, d_cdt, num_cdt, d_out, d_face, d_keep);
  if (rc != GCVT_OK) return rc;
  if (num_points &&
      cudaMemcpy(out_xyz, d_out, (size_t)num_points * 3 * sizeof(double),
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCVT_ERR_CUDA;
  if (num_points && out_face &&
      cudaMemcpy(out_face, d_face, (size_t)num_points * sizeof(int), cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return GCVT_ERR_CUDA;
  if (num_cdt && cudaMemcpy(keep, d_keep, (size_t)num_cdt, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCVT_ERR_CUDA;
  return GCVT_OK;
}

extern "C" int gcvt_vertex_weights(const double *uv, const double *xyz, int num_vertex,
                                   const int32_t *triangle, int num_tri, double *weight,
                                   int mem) {
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (num_vertex < 0 || num_tri < 0) return GCVT_ERR_ARGUMENT;
  if ((num_vertex && (!uv || !xyz || !weight)) || (num_tri && !triangle))
    return GCVT_ERR_ARGUMENT;
  if ((long long)num_tri * 3 > INT_MAX) return GCVT_ERR_SIZE;
  if (num_vertex == 0) return GCVT_OK;
  Scratch sc;
  if (mem == GCVT_MEM_DEVICE)
    return weights_device(sc, uv, xyz, num_vertex, triangle, num_tri, weight);
  const double *d_uv = nullptr, *d_xyz = nullptr;
  const int *d_tri = nullptr;
  double *d_w = nullptr;
  HCK(copy_in(sc, uv, (size_t)num_vertex * 2, &d_uv));
  HCK(copy_in(sc, xyz, (size_t)num_vertex * 3, &d_xyz));
  HCK(copy_in(sc, triangle, (size_t)num_tri * 3, &d_tri));
  HCK(take_out(sc, (size_t)num_vertex, &d_w));
  const int rc = weights_device(sc, d_uv, d_xyz, num_vertex, d_tri, num_tri, d_w);
  if (rc != GCVT_OK) return rc;
  if (cudaMemcpy(weight, d_w, (size_t)num_vertex * sizeof(double), cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return GCVT_ERR_CUDA;
  return GCVT_OK;
}
