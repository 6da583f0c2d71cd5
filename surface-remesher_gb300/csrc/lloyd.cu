// lloyd.cu -- site update, energy total and the gCVT iteration schedule.
//
// k_update restates kernelFillShort + kernelUpdateSites (gcvt.cu:65-71,
// 753-781) over the site bitmap: one thread per 64-row word, one site per set
// bit.  The centroid comes from the compensated moments the row pass
// accumulated (FP64 only for the final division, as the reference's centroid
// is a float): c = site + SX/W, rounded once to float, then
//     new = trunc(fma(c - site, omega, site) + 0.5f), clamped to [0, n-1],
// unchanged for fixed sites or when the density at the new pixel is 0.  New
// positions are OR-ed into the other bitmap, so sites landing on one pixel
// merge, as the reference's scatter does.  The energy total is summed in FP64
// in a fixed order (threads, then blocks), and the last block runs the omega /
// stop schedule of gcvt.cu:1105-1142 on the device.
#include "gcvt_internal.cuh"

namespace cvtgb {

// float -> short as kernelUpdateSites converts it (round toward zero,
// saturating, NaN -> 0), then the clamp of gcvt.cu:774-775.
__device__ __forceinline__ int update_coord(float v, int n) {
  int c = __float2int_rz(v);  // saturates to int32, NaN -> 0
  return min(max(c, 0), n - 1);
}

__global__ void __launch_bounds__(kUpdateThreads) k_update(LevelBufs a) {
  DevState *st = a.st;
  if (st->stopped) return;
  const int n = a.n, nb = n / kBand;
  const size_t nwords = (size_t)nb * n;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int parity = st->parity;
  uint64_t *cur = parity ? a.bits[1] : a.bits[0];
  uint64_t *nxt = parity ? a.bits[0] : a.bits[1];
  const float omega = st->omega;
  double e = 0.0;
  if (t < nwords) {
    uint64_t w = cur[t];
    if (w) cur[t] = 0ull;  // this buffer receives the iteration after next
    const int b = (int)(t / n), x = (int)(t % n);
    while (w) {
      const int i = __ffsll((long long)w) - 1;
      w &= w - 1ull;
      const int y = b * kBand + i;
      const size_t pid = (size_t)y * n + x;
      const float4 h = a.mhi[pid], l = a.mlo[pid];
      a.mhi[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.mlo[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
      const double W = (double)h.x + (double)l.x;
      const double SX = (double)h.y + (double)l.y;
      const double SY = (double)h.z + (double)l.z;
      e += (double)h.w + (double)l.w;
      const float cx = (float)((double)x + SX / W);
      const float cy = (float)((double)y + SY / W);
      const float fx = __fadd_rn(__fmaf_rn(__fsub_rn(cx, (float)x), omega, (float)x), 0.5f);
      const float fy = __fadd_rn(__fmaf_rn(__fsub_rn(cy, (float)y), omega, (float)y), 0.5f);
      int nx = update_coord(fx, n), ny = update_coord(fy, n);
      if (a.fixed[pid] || a.density[(size_t)ny * n + nx] == 0.0f) { nx = x; ny = y; }
      atomicOr(reinterpret_cast<unsigned long long *>(nxt + (size_t)(ny / kBand) * n + nx),
               1ull << (ny % kBand));
    }
  }
  // fixed-order block reduction of the energy
  __shared__ double sred[kUpdateThreads];
  __shared__ bool is_last;
  sred[threadIdx.x] = e;
  __syncthreads();
  for (int s = kUpdateThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sred[threadIdx.x] += sred[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.blk_energy[blockIdx.x] = sred[0];
    __threadfence();
    unsigned prev = atomicAdd(&st->done_blocks, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  // last block: total energy in block order, then the schedule
  __threadfence();
  double acc = 0.0;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x)
    acc += ((volatile double *)a.blk_energy)[k];
  sred[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kUpdateThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sred[threadIdx.x] += sred[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double E = sred[0] * st->energy_scale;
    st->energy = E;
    const int i = st->iter;
    if (i % 10 == 0) st->sampled = E;          // gcvt.cu:1116-1117
    st->iter = i + 1;                          // gcvt.cu:1123
    st->level_iters += 1;
    int stop = 0;
    if ((i + 1) % 10 == 0) {                   // gcvt.cu:1125-1140
      const double diff = st->last_energy - st->sampled;
      const double grad = diff / 10.0;
      st->omega = (float)fmin(2.0, 1.0 + diff);
      if (st->use_stop_rule && (st->level ? grad < 3e-1 : grad < 1e-5)) stop = 1;
      else st->last_energy = st->sampled;
    }
    if (st->use_stop_rule ? (st->iter >= st->max_iter) : (st->level_iters >= st->fixed_iters))
      stop = 1;                                // gcvt.cu:1142
    if (stop) st->stopped = 1;
    st->parity = parity ^ 1;
    st->done_blocks = 0;
    __threadfence();
  }
}

int update_blocks(int n) {
  size_t nwords = (size_t)(n / kBand) * n;
  return (int)((nwords + kUpdateThreads - 1) / kUpdateThreads);
}

cudaError_t launch_update(const LevelBufs &b, cudaStream_t s) {
  k_update<<<update_blocks(b.n), kUpdateThreads, 0, s>>>(b);
  return cudaGetLastError();
}

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

// Moments of the current sites in absolute coordinates (W, X, Y, E) at each
// site pixel, 0 elsewhere; the accumulators are cleared.  Parity tests only.
__global__ void k_read_moments(LevelBufs a, double *out) {
  const int n = a.n;
  size_t pid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= (size_t)n * n) return;
  const int x = (int)(pid % n), y = (int)(pid / n);
  const uint64_t w = (a.st->parity ? a.bits[1] : a.bits[0])[(size_t)(y / kBand) * n + x];
  double W = 0, X = 0, Y = 0, E = 0;
  if ((w >> (y % kBand)) & 1ull) {
    const float4 h = a.mhi[pid], l = a.mlo[pid];
    W = (double)h.x + (double)l.x;
    X = (double)x * W + ((double)h.y + (double)l.y);
    Y = (double)y * W + ((double)h.z + (double)l.z);
    E = (double)h.w + (double)l.w;
  }
  a.mhi[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
  a.mlo[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
  const size_t nn = (size_t)n * n;
  out[pid] = W;
  out[nn + pid] = X;
  out[2 * nn + pid] = Y;
  out[3 * nn + pid] = E;
}

cudaError_t launch_read_moments(const LevelBufs &b, double *out4, cudaStream_t s) {
  size_t nn = (size_t)b.n * b.n;
  k_read_moments<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(b, out4);
  return cudaGetLastError();
}

}  // namespace cvtgb
