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
// denominator, a conditioning d00*d11/denom above 2^20 (slivers, whose
// rounded weights can pass far outside the triangle), or a box over more
// than 4096 tiles.  For the rest the box, enlarged by 1e-6 of its width +
// height, keeps every pixel whose FP64 test can pass: the weights' rounding
// errors are below 32 u kappa of the triangle's size (u = 2^-53), under 1e-8
// of it at kappa <= 2^20.  A denominator of exactly 0 never passes.
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <cstdio>
#include <cstdlib>

namespace cvtgb {

constexpr int kTile = 16;
constexpr double kMaxCond = 1048576.0;  // 2^20
constexpr int kMaxTilesPerTri = 4096;

struct TriData {
  double x1, y1, x2, y2, x3, y3;  // vertex coordinates, copied from points[]
  int p1, p2, p3;                 // vertex indices (for the weights)
  int global;                     // 1: on the global list
};

// The point-independent terms of the test, as bary_inside computes them.
__device__ __forceinline__ void tri_terms(const TriData &t, double &d00, double &d01,
                                          double &d11, double &denom) {
  const double v0x = __dsub_rn(t.x2, t.x1), v0y = __dsub_rn(t.y2, t.y1);
  const double v1x = __dsub_rn(t.x3, t.x1), v1y = __dsub_rn(t.y3, t.y1);
  d00 = __fma_rn(v0x, v0x, __dmul_rn(v0y, v0y));
  d01 = __fma_rn(v0x, v1x, __dmul_rn(v0y, v1y));
  d11 = __fma_rn(v1x, v1x, __dmul_rn(v1y, v1y));
  denom = __fma_rn(d00, d11, -__dmul_rn(d01, d01));
}

// barycentric_coordinate (discretization.cu:32-55) with the reference's
// operation order; returns the caller's (w1, w2, w3) after the reference's
// output-argument permutation.
__device__ __forceinline__ bool bary_inside(const TriData &t, double x0, double y0, double &w1,
                                            double &w2, double &w3) {
  const double v0x = __dsub_rn(t.x2, t.x1), v0y = __dsub_rn(t.y2, t.y1);
  const double v1x = __dsub_rn(t.x3, t.x1), v1y = __dsub_rn(t.y3, t.y1);
  const double v2x = __dsub_rn(x0, t.x1), v2y = __dsub_rn(y0, t.y1);
  const double d00 = __fma_rn(v0x, v0x, __dmul_rn(v0y, v0y));
  const double d01 = __fma_rn(v0x, v1x, __dmul_rn(v0y, v1y));
  const double d11 = __fma_rn(v1x, v1x, __dmul_rn(v1y, v1y));
  const double d20 = __fma_rn(v2x, v0x, __dmul_rn(v2y, v0y));
  const double d21 = __fma_rn(v2x, v1x, __dmul_rn(v2y, v1y));
  const double denom = __fma_rn(d00, d11, -__dmul_rn(d01, d01));
  if (denom == 0) return false;  // all weights -1 in the reference
  const double a = __ddiv_rn(__fma_rn(d11, d20, -__dmul_rn(d01, d21)), denom);
  const double b = __ddiv_rn(__fma_rn(d00, d21, -__dmul_rn(d01, d20)), denom);
  w2 = a;                               // the reference's w1 argument slot
  w3 = b;                               // w2 slot
  w1 = __dsub_rn(__dsub_rn(1.0, a), b); // w3 slot: 1 - w1 - w2
  return !(w1 < 0 || w2 < 0 || w3 < 0);
}

__global__ void k_tri_setup(const double *__restrict__ pts, const int *__restrict__ tri, int T,
                            double inv_scale, int n, TriData *td, int4 *tbox,
                            int *tile_count, int *glist, int *gcount, int num_point,
                            int *err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T) return;
  TriData t;
  t.p1 = tri[3 * i];
  t.p2 = tri[3 * i + 1];
  t.p3 = tri[3 * i + 2];
  if (t.p1 < 0 || t.p2 < 0 || t.p3 < 0 || t.p1 >= num_point || t.p2 >= num_point ||
      t.p3 >= num_point) {
    atomicOr(err, 1);
    t.p1 = t.p2 = t.p3 = 0;
    t.x1 = t.y1 = t.x2 = t.y2 = t.x3 = t.y3 = 0.0;  // denominator 0: never passes
    t.global = 0;
    td[i] = t;
    tbox[i] = make_int4(1, 1, 0, 0);
    return;
  }
  t.x1 = pts[2 * t.p1];
  t.y1 = pts[2 * t.p1 + 1];
  t.x2 = pts[2 * t.p2];
  t.y2 = pts[2 * t.p2 + 1];
  t.x3 = pts[2 * t.p3];
  t.y3 = pts[2 * t.p3 + 1];
  t.global = 0;
  double d00, d01, d11, denom;
  tri_terms(t, d00, d01, d11, denom);
  const double xmin = fmin(t.x1, fmin(t.x2, t.x3)), xmax = fmax(t.x1, fmax(t.x2, t.x3));
  const double ymin = fmin(t.y1, fmin(t.y2, t.y3)), ymax = fmax(t.y1, fmax(t.y2, t.y3));
  const bool finite = isfinite(t.x1) && isfinite(t.y1) && isfinite(t.x2) && isfinite(t.y2) &&
                      isfinite(t.x3) && isfinite(t.y3) && isfinite(denom);
  if (denom == 0) {  // never passes
    td[i] = t;
    tbox[i] = make_int4(1, 1, 0, 0);
    return;
  }
  if (!finite || !(denom > 0) || !(d00 * d11 / denom <= kMaxCond)) {
    t.global = 1;
    td[i] = t;
    tbox[i] = make_int4(0, 0, n - 1, n - 1);
    glist[atomicAdd(gcount, 1)] = i;
    return;
  }
  // pixel box: pixels whose sample point lies in the triangle's box enlarged
  // by 1e-6 of its width + height plus a pixel fraction
  const double m = ((xmax - xmin) + (ymax - ymin)) * 1e-6 + 1e-9 / inv_scale;
  int x0 = (int)fmax(-1.0, ceil((xmin - m) * inv_scale));
  int x1 = (int)fmin((double)n, floor((xmax + m) * inv_scale));
  int y0 = (int)fmax(-1.0, ceil((ymin - m) * inv_scale));
  int y1 = (int)fmin((double)n, floor((ymax + m) * inv_scale));
  x0 = max(x0, 0);
  y0 = max(y0, 0);
  x1 = min(x1, n - 1);
  y1 = min(y1, n - 1);
  if (x0 > x1 || y0 > y1) {
    td[i] = t;
    tbox[i] = make_int4(1, 1, 0, 0);  // empty
    return;
  }
  tbox[i] = make_int4(x0, y0, x1, y1);
  const long long tiles =
      (long long)(x1 / kTile - x0 / kTile + 1) * (long long)(y1 / kTile - y0 / kTile + 1);
  if (tiles > kMaxTilesPerTri) {
    t.global = 1;
    td[i] = t;
    glist[atomicAdd(gcount, 1)] = i;
    return;
  }
  td[i] = t;
  const int nt = n / kTile;
  for (int ty = y0 / kTile; ty <= y1 / kTile; ++ty)
    for (int tx = x0 / kTile; tx <= x1 / kTile; ++tx) atomicAdd(&tile_count[ty * nt + tx], 1);
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

// One block per tile, one thread per pixel.
__global__ void __launch_bounds__(kTile *kTile) k_raster(const TriData *__restrict__ td,
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
    if ((call) != cudaSuccess) { rc = GCVT_ERR_CUDA; goto done; } \
  } while (0)
}  // namespace

extern "C" int gcvt_rasterize(const double *points, const double *weight, int num_point,
                              const int32_t *triangle, int num_tri, float *density, double scale,
                              int n, int mem) {
  if (!points || !weight || !triangle || !density) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (num_point < 0 || num_tri < 0 || !(scale > 0)) return GCVT_ERR_ARGUMENT;
  if (n < kTile || n % kTile != 0 || n > 16384) return GCVT_ERR_SIZE;
  int rc = GCVT_OK;
  const int nt = n / kTile, ntiles = nt * nt;
  double *d_pts = nullptr, *d_w = nullptr;
  int *d_tri = nullptr, *d_cnt = nullptr, *d_off = nullptr, *d_cur = nullptr, *d_list = nullptr;
  int *d_glist = nullptr, *d_scal = nullptr;  // global list; [0] its length, [1] error flag
  int herr = 0;
  TriData *d_td = nullptr;
  int4 *d_box = nullptr;
  float *d_dens = nullptr;
  int total = 0;
  const cudaMemcpyKind h2d = mem == GCVT_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  if (ntiles > 1024 * 65536) return GCVT_ERR_SIZE;
  if (mem == GCVT_MEM_HOST) {
    RCK(cudaMalloc((void **)&d_pts, (size_t)num_point * 2 * sizeof(double) + 16));
    RCK(cudaMalloc((void **)&d_w, (size_t)num_point * sizeof(double) + 16));
    RCK(cudaMalloc((void **)&d_tri, (size_t)num_tri * 3 * sizeof(int) + 16));
    RCK(cudaMalloc((void **)&d_dens, (size_t)n * n * sizeof(float)));
    RCK(cudaMemcpy(d_pts, points, (size_t)num_point * 2 * sizeof(double), h2d));
    RCK(cudaMemcpy(d_w, weight, (size_t)num_point * sizeof(double), h2d));
    RCK(cudaMemcpy(d_tri, triangle, (size_t)num_tri * 3 * sizeof(int), h2d));
  }
  {
    const double *P = mem == GCVT_MEM_HOST ? d_pts : points;
    const double *Wt = mem == GCVT_MEM_HOST ? d_w : weight;
    const int *Tr = mem == GCVT_MEM_HOST ? d_tri : triangle;
    float *D = mem == GCVT_MEM_HOST ? d_dens : density;
    RCK(cudaMalloc((void **)&d_td, (size_t)num_tri * sizeof(TriData) + 16));
    RCK(cudaMalloc((void **)&d_box, (size_t)num_tri * sizeof(int4) + 16));
    RCK(cudaMalloc((void **)&d_cnt, (size_t)ntiles * sizeof(int)));
    RCK(cudaMalloc((void **)&d_off, (size_t)(ntiles + 1) * sizeof(int)));
    RCK(cudaMalloc((void **)&d_cur, (size_t)ntiles * sizeof(int)));
    RCK(cudaMalloc((void **)&d_glist, (size_t)num_tri * sizeof(int) + 16));
    RCK(cudaMalloc((void **)&d_scal, 2 * sizeof(int)));
    RCK(cudaMemset(d_scal, 0, 2 * sizeof(int)));
    RCK(cudaMemset(d_cnt, 0, (size_t)ntiles * sizeof(int)));
    if (num_tri > 0) {
      k_tri_setup<<<(num_tri + 255) / 256, 256>>>(P, Tr, num_tri, 1.0 / scale, n, d_td, d_box,
                                                  d_cnt, d_glist, d_scal, num_point, d_scal + 1);
      RCK(cudaGetLastError());
    }
    k_tile_scan<<<1, 1024>>>(d_cnt, ntiles, d_off, d_cur);
    RCK(cudaGetLastError());
    RCK(cudaMemcpy(&total, d_off + ntiles, sizeof(int), cudaMemcpyDeviceToHost));
    RCK(cudaMalloc((void **)&d_list, (size_t)total * sizeof(int) + 16));
    if (num_tri > 0) {
      k_tri_scatter<<<(num_tri + 255) / 256, 256>>>(d_td, d_box, num_tri, n, d_cur, d_list);
      RCK(cudaGetLastError());
    }
    k_raster<<<ntiles, kTile * kTile>>>(d_td, d_box, d_off, d_list, d_glist, d_scal, Wt, scale,
                                        n, D);
    RCK(cudaGetLastError());
    RCK(cudaMemcpy(&herr, d_scal + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
      rc = GCVT_ERR_ARGUMENT;
      goto done;
    }
    if (mem == GCVT_MEM_HOST)
      RCK(cudaMemcpy(density, d_dens, (size_t)n * n * sizeof(float), cudaMemcpyDeviceToHost));
    RCK(cudaDeviceSynchronize());
  }
done:
  cudaFree(d_pts);
  cudaFree(d_w);
  cudaFree(d_tri);
  cudaFree(d_dens);
  cudaFree(d_td);
  cudaFree(d_box);
  cudaFree(d_cnt);
  cudaFree(d_off);
  cudaFree(d_cur);
  cudaFree(d_list);
  cudaFree(d_glist);
  cudaFree(d_scal);
  return rc;
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
