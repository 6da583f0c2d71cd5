// lloyd.cu -- the pieces of the multi-level schedule around the Lloyd kernel
// (cells.cu): zooming the site set between levels and the density pyramid.
#include "gcvt_internal.cuh"

namespace cvtgb {

// kernelZoomIn (gcvt.cu:485-495): site (x, y) of the n-grid becomes (2x, 2y)
// of the 2n-grid; dst must be zero.
__global__ void k_zoom(const uint64_t *__restrict__ src, int n, uint64_t *dst) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)(n / kBand) * n) return;
  uint64_t w = src[t];
  const int b = (int)(t / n), x = (int)(t % n);
  const int n2 = 2 * n;
  while (w) {
    int i = __ffsll((long long)w) - 1;
    w &= w - 1ull;
    int y2 = 2 * (b * kBand + i), x2 = 2 * x;
    atomicOr(reinterpret_cast<unsigned long long *>(dst + (size_t)(y2 / kBand) * n2 + x2),
             1ull << (y2 % kBand));
  }
}

cudaError_t launch_zoom(const uint64_t *src, int n, uint64_t *dst, cudaStream_t s) {
  size_t nwords = (size_t)(n / kBand) * n;
  k_zoom<<<(unsigned)((nwords + 255) / 256), 256, 0, s>>>(src, n, dst);
  return cudaGetLastError();
}

// kernelDensityScaling (gcvt.cu:497-511): the four samples summed in the
// reference's order (x outer, y inner), then divided by 4.
__global__ void k_density_halve(const float *__restrict__ in, float *__restrict__ out, int n) {
  int tx = blockIdx.x * blockDim.x + threadIdx.x;
  int ty = blockIdx.y * blockDim.y + threadIdx.y;
  if (tx >= n || ty >= n) return;
  const int n2 = 2 * n;
  float d = 0.0f;
  d = __fadd_rn(d, in[(size_t)(2 * ty) * n2 + 2 * tx]);
  d = __fadd_rn(d, in[(size_t)(2 * ty + 1) * n2 + 2 * tx]);
  d = __fadd_rn(d, in[(size_t)(2 * ty) * n2 + 2 * tx + 1]);
  d = __fadd_rn(d, in[(size_t)(2 * ty + 1) * n2 + 2 * tx + 1]);
  out[(size_t)ty * n + tx] = (float)((double)d / 4.0);
}

cudaError_t launch_density_halve(const float *in, float *out, int n_out, cudaStream_t s) {
  dim3 blk(16, 16), grd((n_out + 15) / 16, (n_out + 15) / 16);
  k_density_halve<<<grd, blk, 0, s>>>(in, out, n_out);
  return cudaGetLastError();
}

}  // namespace cvtgb
