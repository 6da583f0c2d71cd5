// rasterizer.cu -- the density grid from a parameterised triangle mesh,
// equal to the reference's kernelDiscretization (discretization.cu:57-85)
// pixel for pixel.
//
// Reference semantics: pixel (tx, ty) samples the point (tx*scale, ty*scale);
// the first triangle in index order whose three FP64 barycentric weights are
// all >= 0 gives density = sum w_i * weight[v_i] (FP64, stored as float); no
// containing triangle gives 0.  The reference tests every pixel against every
// triangle (O(n^2 T), FP64).
//
// GB300 version: triangles are binned into 16x16-pixel tiles by their
// bounding boxes (count, scan, scatter); each pixel scans its tile's list,
// rejects triangles whose enlarged box misses it, runs the FP64 barycentric
// test -- the reference's expressions, with the fused multiply-adds nvcc
// forms from them written out explicitly -- on the rest, and keeps the
// smallest index that passes, which is the reference's first hit.  Triangles
// the boxes cannot place go to a global list every pixel tests: non-finite
// coordinates (their weights are NaN and pass the test), a negative
// denominator, a conditioning kappa = d00*d11/denom above 2^40 (near-flat
// slivers, whose rounded weights can pass far outside the triangle), or a box
// over more than 4096 tiles.  For the rest the box, enlarged by
// max(1e-6, kappa 2^-45) of its width + height, keeps every pixel whose FP64
// test can pass: a false hit at distance D needs D < 2^-48 kappa (D + L), L
// the triangle's size (u = 2^-53), so under 4e-9 L at kappa <= 2^20 and a
// factor 8 inside the margin up to kappa = 2^40.  A denominator of exactly 0
// never passes.  Tile lists are sorted, so a pixel stops at its first hit,
// and a weight whose numerator is already negative rejects a triangle before
// the FP64 divisions.
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <cstdio>
#include <cstdlib>

namespace cvtgb {

constexpr int kTile = 16;
constexpr double kMaxCond = 1099511627776.0;  // 2^40
constexpr int kMaxTilesPerTri = 4096;

// A triangle with the point-independent terms of barycentric_coordinate
// (discretization.cu:32-55) precomputed as the kernel would compute them.
struct TriData {
  double x1, y1, v0x, v0y, v1x, v1y, d00, d01, d11, denom;
  int p1, p2, p3;  // vertex indices (for the weights)
  int global;      // 1: on the global list
};

__device__ __forceinline__ void tri_terms(double x1, double y1, double x2, double y2, double x3,
                                          double y3, TriData &t) {
  t.x1 = x1;
  t.y1 = y1;
  t.v0x = __dsub_rn(x2, x1);
  t.v0y = __dsub_rn(y2, y1);
  t.v1x = __dsub_rn(x3, x1);
  t.v1y = __dsub_rn(y3, y1);
  t.d00 = __fma_rn(t.v0x, t.v0x, __dmul_rn(t.v0y, t.v0y));
  t.d01 = __fma_rn(t.v0x, t.v1x, __dmul_rn(t.v0y, t.v1y));
  t.d11 = __fma_rn(t.v1x, t.v1x, __dmul_rn(t.v1y, t.v1y));
  t.denom = __fma_rn(t.d00, t.d11, -__dmul_rn(t.d01, t.d01));
}

// barycentric_coordinate with the reference's operation order and the fused
// multiply-adds nvcc forms in it; returns the caller's (w1, w2, w3) after the
// reference's output-argument permutation.
__device__ __forceinline__ bool bary_inside(const TriData &t, double x0, double y0, double &w1,
                                            double &w2, double &w3) {
  const double v2x = __dsub_rn(x0, t.x1), v2y = __dsub_rn(y0, t.y1);
  const double d20 = __fma_rn(v2x, t.v0x, __dmul_rn(v2y, t.v0y));
  const double d21 = __fma_rn(v2x, t.v1x, __dmul_rn(v2y, t.v1y));
  if (t.denom == 0) return false;  // all weights -1 in the reference
  const double a = __ddiv_rn(__fma_rn(t.d11, d20, -__dmul_rn(t.d01, d21)), t.denom);
  const double b = __ddiv_rn(__fma_rn(t.d00, d21, -__dmul_rn(t.d01, d20)), t.denom);
  w2 = a;                                // the reference's w1 argument slot
  w3 = b;                                // w2 slot
  w1 = __dsub_rn(__dsub_rn(1.0, a), b);  // w3 slot: 1 - w1 - w2
  return !(w1 < 0 || w2 < 0 || w3 < 0);
}

// RN(num / denom) < 0 for denom > 0, decided without dividing (false: divide
// to know): num < 0 and the quotient too large to round to -0.
__device__ __forceinline__ bool quot_negative(double num, double denom) {
  return num < 0 && (denom <= 1.0 || -num >= __dmul_rn(denom, 0x1p-1000));
}

// bary_inside for a finite triangle with denom > 0: same results, but a
// weight whose numerator already shows it negative rejects the triangle
// before the divisions (FP64 issue is scarce on GB300).
__device__ __forceinline__ bool bary_inside_local(const TriData &t, double x0, double y0,
                                                  double &w1, double &w2, double &w3) {
  const double v2x = __dsub_rn(x0, t.x1), v2y = __dsub_rn(y0, t.y1);
  const double d20 = __fma_rn(v2x, t.v0x, __dmul_rn(v2y, t.v0y));
  const double d21 = __fma_rn(v2x, t.v1x, __dmul_rn(v2y, t.v1y));
  const double na = __fma_rn(t.d11, d20, -__dmul_rn(t.d01, d21));
  if (quot_negative(na, t.denom)) return false;
  const double nb = __fma_rn(t.d00, d21, -__dmul_rn(t.d01, d20));
  if (quot_negative(nb, t.denom)) return false;
  const double a = __ddiv_rn(na, t.denom);
  const double b = __ddiv_rn(nb, t.denom);
  w2 = a;
  w3 = b;
  w1 = __dsub_rn(__dsub_rn(1.0, a), b);
  return !(w1 < 0 || w2 < 0 || w3 < 0);
}

// An FP32 pre-test that rejects a pixel clearly outside a triangle before the
// FP64 test, for triangles with conditioning <= 2^20 (sgn = 0: no pre-test).
// In pixel units, r = q - P1, edge functions E0 = v0 x r, E1 = (v1 - v0) x
// (r - v0), E2 = (-v1) x (r - v1), all >= 0 inside a counter-clockwise
// triangle (sgn folds the orientation).  With M the largest coordinate
// magnitude, L the longest edge and |r| <= 3 L inside the triangle's box, the
// FP32 error of each E_k is below L (2^-22 M + 2^-19 L) (rounded coordinates
// and edge vectors, three roundings in the products); so sgn E_k < -t with
// t = L (2^-21 M + 2^-16 L) means E_k < -2^-17 L^2 exactly: the pixel lies
// more than 2^-17 L outside edge k, far beyond the FP64 test's own error
// there (2^-48 kappa (|r| + L) <= 2^-26 L), so the FP64 weight of the
// opposite vertex is negative and the reference's test fails too.
struct TriPre {
  float p1x, p1y, v0x, v0y, v1x, v1y, t, sgn;
};

__device__ __forceinline__ bool pre_outside(const TriPre &q, int tx, int ty) {
  if (q.sgn == 0.f) return false;
  const float rx = (float)tx - q.p1x, ry = (float)ty - q.p1y;
  const float e0 = q.v0x * ry - q.v0y * rx;
  const float e1 = (q.v1x - q.v0x) * (ry - q.v0y) - (q.v1y - q.v0y) * (rx - q.v0x);
  const float e2 = q.v1y * (rx - q.v1x) - q.v1x * (ry - q.v1y);
  return q.sgn * e0 < -q.t || q.sgn * e1 < -q.t || q.sgn * e2 < -q.t;
}

__device__ __forceinline__ TriPre make_pre(const TriData &t, double inv_scale, int n,
                                           double cond) {
  TriPre q{0, 0, 0, 0, 0, 0, 0, 0};
  if (!(cond <= 1048576.0)) return q;
  const double cr = t.v0x * t.v1y - t.v0y * t.v1x;
  if (!(cr != 0.0) || !isfinite(cr)) return q;
  const double p1x = t.x1 * inv_scale, p1y = t.y1 * inv_scale;
  const double ax = t.v0x * inv_scale, ay = t.v0y * inv_scale;
  const double bx = t.v1x * inv_scale, by = t.v1y * inv_scale;
  const double l0 = sqrt(ax * ax + ay * ay), l2 = sqrt(bx * bx + by * by);
  const double l1 = sqrt((bx - ax) * (bx - ax) + (by - ay) * (by - ay));
  const double L = fmax(l0, fmax(l1, l2));
  const double M = fmax((double)n, fmax(fabs(p1x), fabs(p1y)) + 4.0 * L);
  if (!(L >= 1e-9 && M <= 1e9)) return q;  // keep FP32 away from over/underflow
  const double thr = L * (0x1p-21 * M + 0x1p-16 * L) * 1.0625;
  q.p1x = (float)p1x;
  q.p1y = (float)p1y;
  q.v0x = (float)ax;
  q.v0y = (float)ay;
  q.v1x = (float)bx;
  q.v1y = (float)by;
  q.t = (float)thr;
  q.sgn = cr > 0 ? 1.f : -1.f;
  return q;
}

__global__ void k_tri_setup(const double *__restrict__ pts, const int *__restrict__ tri, int T,
                            double inv_scale, int n, TriData *td, TriPre *tpre, int4 *tbox,
                            int *tile_count, int *glist, int *gcount, int num_point,
                            int *err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T) return;
  tpre[i] = TriPre{0, 0, 0, 0, 0, 0, 0, 0};
  TriData t;
  t.p1 = tri[3 * i];
  t.p2 = tri[3 * i + 1];
  t.p3 = tri[3 * i + 2];
  t.global = 0;
  if (t.p1 < 0 || t.p2 < 0 || t.p3 < 0 || t.p1 >= num_point || t.p2 >= num_point ||
      t.p3 >= num_point) {
    atomicOr(err, 1);
    t.p1 = t.p2 = t.p3 = 0;
    tri_terms(0, 0, 0, 0, 0, 0, t);  // denominator 0: never passes
    td[i] = t;
    tbox[i] = make_int4(1, 1, 0, 0);
    return;
  }
  const double x1 = pts[2 * t.p1], y1 = pts[2 * t.p1 + 1];
  const double x2 = pts[2 * t.p2], y2 = pts[2 * t.p2 + 1];
  const double x3 = pts[2 * t.p3], y3 = pts[2 * t.p3 + 1];
  tri_terms(x1, y1, x2, y2, x3, y3, t);
  const double xmin = fmin(x1, fmin(x2, x3)), xmax = fmax(x1, fmax(x2, x3));
  const double ymin = fmin(y1, fmin(y2, y3)), ymax = fmax(y1, fmax(y2, y3));
  const bool finite = isfinite(x1) && isfinite(y1) && isfinite(x2) && isfinite(y2) &&
                      isfinite(x3) && isfinite(y3) && isfinite(t.denom);
  if (t.denom == 0) {  // never passes
    td[i] = t;
    tbox[i] = make_int4(1, 1, 0, 0);
    return;
  }
  const double cond = t.d00 * t.d11 / t.denom;
  if (!finite || !(t.denom > 0) || !(cond <= kMaxCond)) {
    t.global = 1;
    td[i] = t;
    tbox[i] = make_int4(0, 0, n - 1, n - 1);
    glist[atomicAdd(gcount, 1)] = i;
    return;
  }
  // pixel box: pixels whose sample point lies in the triangle's box enlarged
  // by max(1e-6, kappa 2^-45) of its width + height plus a pixel fraction
  const double m =
      fmax(1e-6, cond * 0x1p-45) * ((xmax - xmin) + (ymax - ymin)) + 1e-9 / inv_scale;
  // (clamped to [-1, n] before the conversion to int)
  int x0 = (int)fmin((double)n, fmax(-1.0, ceil((xmin - m) * inv_scale)));
  int x1p = (int)fmin((double)n, fmax(-1.0, floor((xmax + m) * inv_scale)));
  int y0 = (int)fmin((double)n, fmax(-1.0, ceil((ymin - m) * inv_scale)));
  int y1p = (int)fmin((double)n, fmax(-1.0, floor((ymax + m) * inv_scale)));
  x0 = max(x0, 0);
  y0 = max(y0, 0);
  x1p = min(x1p, n - 1);
  y1p = min(y1p, n - 1);
  if (x0 > x1p || y0 > y1p) {
    td[i] = t;
    tbox[i] = make_int4(1, 1, 0, 0);  // empty
    return;
  }
  tbox[i] = make_int4(x0, y0, x1p, y1p);
  const long long tiles = (long long)(x1p / kTile - x0 / kTile + 1) *
                          (long long)(y1p / kTile - y0 / kTile + 1);
  if (tiles > kMaxTilesPerTri) {
    t.global = 1;
    td[i] = t;
    glist[atomicAdd(gcount, 1)] = i;
    return;
  }
  td[i] = t;
  tpre[i] = make_pre(t, inv_scale, n, cond);
  const int nt = n / kTile;
  for (int ty = y0 / kTile; ty <= y1p / kTile; ++ty)
    for (int tx = x0 / kTile; tx <= x1p / kTile; ++tx) atomicAdd(&tile_count[ty * nt + tx], 1);
}

// Exclusive scan of the tile counts, one block (tiles <= 1024 * 64).
__global__ void __launch_bounds__(1024) k_tile_scan(const int *count, int ntiles, int *offset,
                                                   int *cursor) {
  __shared__ int part[1024];
  const int t = threadIdx.x;
  const int per = (ntiles + 1023) / 1024;
  const int b0 = min(ntiles, t * per), b1 = min(ntiles, b0 + per);
  int s = 0;
  for (int i = b0; i < b1; ++i) s += count[i];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int add = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += add;
    __syncthreads();
  }
  int run = part[t] - s;
  for (int i = b0; i < b1; ++i) {
    offset[i] = run;
    cursor[i] = run;
    run += count[i];
  }
  if (t == 1023) offset[ntiles] = part[1023];
}

cudaError_t launch_scan(const int *count, int n, int *offset, int *cursor, cudaStream_t s) {
  if (n < 0 || n > 1024 * 65536) return cudaErrorInvalidValue;
  k_tile_scan<<<1, 1024, 0, s>>>(count, n, offset, cursor);
  return cudaGetLastError();
}

__global__ void k_tri_scatter(const TriData *__restrict__ td, const int4 *__restrict__ tbox, int T,
                              int n, int *cursor, int *list) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T || td[i].global) return;
  const int4 b = tbox[i];
  if (b.x > b.z) return;
  const int nt = n / kTile;
  for (int ty = b.y / kTile; ty <= b.w / kTile; ++ty)
    for (int tx = b.x / kTile; tx <= b.z / kTile; ++tx) {
      const int pos = atomicAdd(&cursor[ty * nt + tx], 1);
      list[pos] = i;
    }
}

// Each tile's list in ascending triangle order (one thread per tile).
__global__ void k_tile_sort(const int *__restrict__ offset, int ntiles, int *list) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ntiles) return;
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

// One block per tile, one thread per pixel; the tile's list is sorted, so the
// first triangle that passes is the answer.
__global__ void __launch_bounds__(kTile *kTile) k_raster(const TriData *__restrict__ td,
                                                        const TriPre *__restrict__ tpre,
                                                        const int4 *__restrict__ tbox,
                                                        const int *__restrict__ offset,
                                                        const int *__restrict__ list,
                                                        const int *__restrict__ glist,
                                                        const int *__restrict__ gcount,
                                                        const double *__restrict__ weight,
                                                        double scale, int n, float *density) {
  const int nt = n / kTile;
  const int tile = blockIdx.x;
  const int tx = (tile % nt) * kTile + threadIdx.x % kTile;
  const int ty = (tile / nt) * kTile + threadIdx.x / kTile;
  const double x = tx * scale, y = ty * scale;
  const int l0 = offset[tile], l1 = offset[tile + 1];
  int best = 0x7fffffff;
  double bw1 = 0, bw2 = 0, bw3 = 0;
  for (int k = l0; k < l1; ++k) {
    const int i = list[k];
    const int4 b = __ldg(&tbox[i]);
    if (tx < b.x || tx > b.z || ty < b.y || ty > b.w) continue;
    if (pre_outside(tpre[i], tx, ty)) continue;
    double w1, w2, w3;
    if (bary_inside_local(td[i], x, y, w1, w2, w3)) {
      best = i;
      bw1 = w1;
      bw2 = w2;
      bw3 = w3;
      break;
    }
  }
  const int ng = *gcount;
  for (int k = 0; k < ng; ++k) {
    const int i = glist[k];
    if (i >= best) continue;
    const int4 b = __ldg(&tbox[i]);
    if (tx < b.x || tx > b.z || ty < b.y || ty > b.w) continue;
    double w1, w2, w3;
    if (bary_inside(td[i], x, y, w1, w2, w3)) {
      best = i;
      bw1 = w1;
      bw2 = w2;
      bw3 = w3;
    }
  }
  float res = 0.0f;
  if (best != 0x7fffffff) {
    const TriData t = td[best];
    // w1*weight[p1] + w2*weight[p2] + w3*weight[p3] as nvcc contracts it
    const double v = __fma_rn(bw3, weight[t.p3],
                              __fma_rn(bw1, weight[t.p1], __dmul_rn(bw2, weight[t.p2])));
    res = (float)v;
  }
  density[(size_t)ty * n + tx] = res;
}

}  // namespace cvtgb

using namespace cvtgb;

namespace {
#define RCK(call)                                  \
  do {                                             \
    if ((call) != cudaSuccess) return GCVT_ERR_CUDA; \
  } while (0)
}  // namespace

extern "C" int gcvt_rasterize(const double *points, const double *weight, int num_point,
                              const int32_t *triangle, int num_tri, float *density, double scale,
                              int n, int mem) {
  if (!points || !weight || !triangle || !density) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (num_point < 0 || num_tri < 0 || !(scale > 0)) return GCVT_ERR_ARGUMENT;
  if (n < kTile || n % kTile != 0 || n > 16384) return GCVT_ERR_SIZE;
  const int nt = n / kTile, ntiles = nt * nt;
  if (ntiles > 1024 * 65536) return GCVT_ERR_SIZE;
  Scratch sc;
  const double *P = points, *Wt = weight;
  const int *Tr = triangle;
  float *D = density;
  if (mem == GCVT_MEM_HOST) {
    double *d_pts = sc.take<double>((size_t)num_point * 2), *d_w = sc.take<double>(num_point);
    int *d_tri = sc.take<int>((size_t)num_tri * 3);
    D = sc.take<float>((size_t)n * n);
    if (!d_pts || !d_w || !d_tri || !D) return GCVT_ERR_ALLOC;
    RCK(cudaMemcpy(d_pts, points, (size_t)num_point * 2 * sizeof(double), cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(d_w, weight, (size_t)num_point * sizeof(double), cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(d_tri, triangle, (size_t)num_tri * 3 * sizeof(int), cudaMemcpyHostToDevice));
    P = d_pts;
    Wt = d_w;
    Tr = d_tri;
  }
  TriData *d_td = sc.take<TriData>(num_tri);
  TriPre *d_pre = sc.take<TriPre>(num_tri);
  int4 *d_box = sc.take<int4>(num_tri);
  int *d_cnt = sc.take<int>(ntiles), *d_off = sc.take<int>(ntiles + 1);
  int *d_cur = sc.take<int>(ntiles), *d_glist = sc.take<int>(num_tri);
  int *d_scal = sc.take<int>(2);  // global list length, error flag
  if (!d_td || !d_pre || !d_box || !d_cnt || !d_off || !d_cur || !d_glist || !d_scal) return GCVT_ERR_ALLOC;
  RCK(cudaMemset(d_scal, 0, 2 * sizeof(int)));
  RCK(cudaMemset(d_cnt, 0, (size_t)ntiles * sizeof(int)));
  if (num_tri > 0) {
    k_tri_setup<<<(num_tri + 255) / 256, 256>>>(P, Tr, num_tri, 1.0 / scale, n, d_td, d_pre, d_box,
                                                d_cnt, d_glist, d_scal, num_point, d_scal + 1);
    RCK(cudaGetLastError());
  }
  k_tile_scan<<<1, 1024>>>(d_cnt, ntiles, d_off, d_cur);
  RCK(cudaGetLastError());
  int total = 0;
  RCK(cudaMemcpy(&total, d_off + ntiles, sizeof(int), cudaMemcpyDeviceToHost));
  int *d_list = sc.take<int>(total);
  if (!d_list) return GCVT_ERR_ALLOC;
  if (num_tri > 0) {
    k_tri_scatter<<<(num_tri + 255) / 256, 256>>>(d_td, d_box, num_tri, n, d_cur, d_list);
    RCK(cudaGetLastError());
    k_tile_sort<<<(ntiles + 255) / 256, 256>>>(d_off, ntiles, d_list);
    RCK(cudaGetLastError());
  }
  k_raster<<<ntiles, kTile * kTile>>>(d_td, d_pre, d_box, d_off, d_list, d_glist, d_scal, Wt, scale, n,
                                      D);
  RCK(cudaGetLastError());
  int herr = 0;
  RCK(cudaMemcpy(&herr, d_scal + 1, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return GCVT_ERR_ARGUMENT;
  if (mem == GCVT_MEM_HOST)
    RCK(cudaMemcpy(density, D, (size_t)n * n * sizeof(float), cudaMemcpyDeviceToHost));
  return GCVT_OK;
}

// The reference's entry point (discretization.h:66, discretization.cu:87):
// host buffers in, host density out; failures print and exit.
void discretization_d(double *points, double *weight, int num_point, int *triangle, int num_tri,
                      float *density, double scale, int n) {
  int rc = gcvt_rasterize(points, weight, num_point, triangle, num_tri, density, scale, n,
                          GCVT_MEM_HOST);
  if (rc != GCVT_OK) {
    std::fprintf(stderr, "discretization_d: %s\n", gcvt_status_string(rc));
    std::exit(rc);
  }
}
