// extract.cu -- the CDT's input points from the converged sites, on the GPU:
// the loop of delaunayInput (delaunay.h:46-57) that scans the n^2 label grid
// on the host for pixels labelled with themselves and not fixed, and emits
// (x * scale + left, y * scale + lower) in x-major, then y order.  Here the
// site bitmap is compacted column by column: k_col_count counts each
// column's free sites, k_col_write finds each column's offset from those
// counts and writes the points in FP64 (products and sums rounded separately,
// as the host code computes them).
#include "gcvt_internal.cuh"

namespace cvtgb {

// Free (not fixed) sites per column of bits (fixed may be null).
__global__ void __launch_bounds__(256) k_col_count(const uint64_t *__restrict__ bits,
                                                   const uint64_t *__restrict__ fixed, int n,
                                                   unsigned *__restrict__ colcnt) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  unsigned c = 0;
  for (int b = 0; b < n / kBand; ++b) {
    uint64_t w = bits[(size_t)b * n + x];
    if (fixed) w &= ~fixed[(size_t)b * n + x];
    c += __popcll(w);
  }
  colcnt[x] = c;
}

// Block b writes columns [256 b, 256 b + 256): its offset is the sum of the
// counts before it, then an exclusive scan over its own columns.
__global__ void __launch_bounds__(256) k_col_write(const uint64_t *__restrict__ bits,
                                                   const uint64_t *__restrict__ fixed, int n,
                                                   const unsigned *__restrict__ colcnt,
                                                   double scale, double left, double lower,
                                                   double *__restrict__ xy, unsigned capacity,
                                                   unsigned *__restrict__ total) {
  __shared__ unsigned wsum[8];
  __shared__ unsigned base_s;
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  const int x0 = blockIdx.x * 256;
  unsigned pre = 0;
  for (int k = tid; k < x0; k += 256) pre += colcnt[k];
  pre = __reduce_add_sync(0xffffffffu, pre);
  if (lane == 0) wsum[wib] = pre;
  __syncthreads();
  if (tid == 0) {
    unsigned s = 0;
    for (int k = 0; k < 8; ++k) s += wsum[k];
    base_s = s;
  }
  __syncthreads();
  const unsigned base = base_s;
  const int x = x0 + tid;
  const unsigned cnt = x < n ? colcnt[x] : 0u;
  unsigned incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  __syncthreads();
  if (lane == 31) wsum[wib] = incl;
  __syncthreads();
  unsigned woff = 0, btotal = 0;
  for (int k = 0; k < 8; ++k) {
    if (k < wib) woff += wsum[k];
    btotal += wsum[k];
  }
  if (blockIdx.x == gridDim.x - 1 && tid == 0) *total = base + btotal;
  if (x >= n || cnt == 0) return;
  unsigned pos = base + woff + incl - cnt;
  const double px = __dadd_rn(__dmul_rn((double)x, scale), left);
  for (int b = 0; b < n / kBand && pos < capacity; ++b) {
    uint64_t w = bits[(size_t)b * n + x];
    if (fixed) w &= ~fixed[(size_t)b * n + x];
    while (w && pos < capacity) {
      const int i = __ffsll((long long)w) - 1;
      w &= w - 1ull;
      xy[2 * (size_t)pos] = px;
      xy[2 * (size_t)pos + 1] = __dadd_rn(__dmul_rn((double)(b * kBand + i), scale), lower);
      ++pos;
    }
  }
}

cudaError_t launch_extract(const uint64_t *bits, const uint64_t *fixed, int n, unsigned *colcnt,
                           double scale, double left, double lower, double *xy,
                           unsigned capacity, unsigned *total, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_col_count<<<blocks, 256, 0, s>>>(bits, fixed, n, colcnt);
  k_col_write<<<blocks, 256, 0, s>>>(bits, fixed, n, colcnt, scale, left, lower, xy, capacity,
                                     total);
  return cudaGetLastError();
}

}  // namespace cvtgb
