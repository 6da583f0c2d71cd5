// lloyd.cu -- site update, energy total and the gCVT iteration schedule.
//
// k_update restates kernelFillShort + kernelUpdateSites (gcvt.cu:65-71,
// 753-781) over the site bitmap: one thread per 64-row word, one site per set
// bit.  The centroid comes from the compensated moments the row pass
// accumulated, divided in two-float arithmetic (GB300 runs FP64 at a small
// fraction of FP32 rate, and this kernel was FP64-bound): c = site + SX/W,
// rounded once to float, then
//     new = trunc(fma(c - site, omega, site) + 0.5f), clamped to [0, n-1],
// unchanged for fixed sites or when the density at the new pixel is 0.  New
// positions are OR-ed into the other bitmap, so sites landing on one pixel
// merge, as the reference's scatter does.  The energy is summed in two-float
// arithmetic in a fixed order (threads, then blocks), the global total is
// formed in FP64 once, and the last block runs the omega / stop schedule of
// gcvt.cu:1105-1142 on the device.
#include "gcvt_internal.cuh"

namespace cvtgb {

// float -> short as kernelUpdateSites converts it (round toward zero,
// saturating, NaN -> 0), then the clamp of gcvt.cu:774-775.
__device__ __forceinline__ int update_coord(float v, int n) {
  int c = __float2int_rz(v);  // saturates to int32, NaN -> 0
  return min(max(c, 0), n - 1);
}

// Error-free sum of two floats (TwoSum).
__device__ __forceinline__ void tsum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bp = __fsub_rn(s, a);
  float ap = __fsub_rn(s, bp);
  e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// (ah, al) + (bh, bl) in two-float arithmetic.
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl) {
  float s, e;
  tsum(ah, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(al, bl));
  ah = __fadd_rn(s, e);
  al = __fsub_rn(e, __fsub_rn(ah, s));
}

// Centroid coordinate base + (Sh + Sl) / (Wh + Wl) rounded once to float.
// The quotient is formed in two-float arithmetic (about 44 significant
// bits): q = Sh / Wh, remainder r = (Sh - q Wh) + Sl - q Wl (the first term
// exact by fma), q2 = r / Wh; then base + q + q2 is summed error-free and
// rounded.  W = 0 gives NaN, as the reference's 0/0 does.
__device__ __forceinline__ float centroid_coord(int base, float Sh, float Sl, float Wh, float Wl) {
  const float q = __fdiv_rn(Sh, Wh);
  const float rr = __fadd_rn(__fmaf_rn(-q, Wh, Sh), __fmaf_rn(-q, Wl, Sl));
  const float q2 = __fdiv_rn(rr, Wh);
  float s, e;
  tsum((float)base, q, s, e);
  return __fadd_rn(s, __fadd_rn(e, q2));
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
  float eh = 0.f, el = 0.f;  // energy, two-float
  if (t < nwords) {
    uint64_t w = cur[t];
    if (w) cur[t] = 0ull;  // this buffer receives the iteration after next
    const int b = (int)(t / (unsigned)n), x = (int)(t % (unsigned)n);
    const uint64_t fw = w ? a.fixed_bits[t] : 0ull;
    int slot = w ? a.group_offset[x >> 5] + a.word_rank[t] : 0;
    while (w) {
      const int i = __ffsll((long long)w) - 1;
      w &= w - 1ull;
      const int y = b * kBand + i;
      const float4 h = a.mhi[slot], l = a.mlo[slot];
      a.mhi[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.mlo[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
      ++slot;
      df_add(eh, el, h.w, l.w);
      const float cx = centroid_coord(x, h.y, l.y, h.x, l.x);
      const float cy = centroid_coord(y, h.z, l.z, h.x, l.x);
      const float fx = __fadd_rn(__fmaf_rn(__fsub_rn(cx, (float)x), omega, (float)x), 0.5f);
      const float fy = __fadd_rn(__fmaf_rn(__fsub_rn(cy, (float)y), omega, (float)y), 0.5f);
      int nx = update_coord(fx, n), ny = update_coord(fy, n);
      if (((fw >> i) & 1ull) || a.density[(size_t)ny * n + nx] == 0.0f) { nx = x; ny = y; }
      atomicOr(reinterpret_cast<unsigned long long *>(nxt + (size_t)(ny / kBand) * n + nx),
               1ull << (ny % kBand));
    }
  }
  // fixed-order two-float block reduction of the energy
  __shared__ float sh[kUpdateThreads], sl[kUpdateThreads];
  __shared__ bool is_last;
  sh[threadIdx.x] = eh;
  sl[threadIdx.x] = el;
  __syncthreads();
  for (int s = kUpdateThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      float ah = sh[threadIdx.x], al = sl[threadIdx.x];
      df_add(ah, al, sh[threadIdx.x + s], sl[threadIdx.x + s]);
      sh[threadIdx.x] = ah;
      sl[threadIdx.x] = al;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.blk_energy[2 * blockIdx.x] = sh[0];
    a.blk_energy[2 * blockIdx.x + 1] = sl[0];
    __threadfence();
    unsigned prev = atomicAdd(&st->done_blocks, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  // last block: total energy in block order (two-float, then one FP64 total),
  // then the schedule
  __threadfence();
  float ah = 0.f, al = 0.f;
  const volatile float *be = a.blk_energy;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) df_add(ah, al, be[2 * k], be[2 * k + 1]);
  sh[threadIdx.x] = ah;
  sl[threadIdx.x] = al;
  __syncthreads();
  for (int s = kUpdateThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      float xh = sh[threadIdx.x], xl = sl[threadIdx.x];
      df_add(xh, xl, sh[threadIdx.x + s], sl[threadIdx.x + s]);
      sh[threadIdx.x] = xh;
      sl[threadIdx.x] = xl;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double E = ((double)sh[0] + (double)sl[0]) * st->energy_scale;
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
  const uint64_t *bits = a.st->parity ? a.bits[1] : a.bits[0];
  const uint64_t w = bits[(size_t)(y / kBand) * n + x];
  double W = 0, X = 0, Y = 0, E = 0;
  if ((w >> (y % kBand)) & 1ull) {
    const int slot = site_slot(bits, a.word_rank, a.group_offset, n, x, y);
    const float4 h = a.mhi[slot], l = a.mlo[slot];
    W = (double)h.x + (double)l.x;
    X = (double)x * W + ((double)h.y + (double)l.y);
    Y = (double)y * W + ((double)h.z + (double)l.z);
    E = (double)h.w + (double)l.w;
    a.mhi[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    a.mlo[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
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
