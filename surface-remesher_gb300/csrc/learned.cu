// learned.cu -- the learned step: a small per-site MLP that predicts where a
// site's Lloyd trajectory ends, trained on trajectories the plain method
// produces, and applied as a jump that the energy decides on.
//
// Features of a site (k_cell MODE 2 or k_features): its last four integer
// moves (newest first) and the density gradient over the density at the
// site, in units of the mean cell radius r: 10 inputs.  The MLP 10 -> 64 ->
// 64 -> 2 (ReLU) predicts the displacement to the site's converged position,
// in units of r.  Weights are bfloat16 (the forward pass rounds weights and
// activations to bfloat16 and accumulates in FP32, the tensor cores'
// arithmetic); training keeps FP32 master weights (Adam).
//
// A jump (host side in api.cu): features pass on the sites S (energy E(S)),
// MLP, k_apply writes the jumped sites L into the next bitmap, an energy pass
// on L computes E(L); k_gate_resolve keeps L if E(L) < E(S) and otherwise
// restores S -- the plain method is the fallback and the judge.
#include "gcvt_internal.cuh"

#include <cuda_bf16.h>

namespace cvtgb {

// Parameter layout: W1[10][64], b1[64], W2[64][64], b2[64], W3[64][2], b3[2].
constexpr int kIn = 10, kHid = 64, kOut = 2;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid,
              kW3 = kB2 + kHid, kB3 = kW3 + kHid * kOut, kMlpParams = kB3 + kOut;  // 4994

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Forward pass of one site with parameters w (bfloat16 values held as float).
__device__ __forceinline__ void mlp_forward(const float *__restrict__ w, const float *x_in,
                                            float *out) {
  float x[kIn];
#pragma unroll
  for (int i = 0; i < kIn; ++i) x[i] = bf(x_in[i]);
  float h1[kHid];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    float acc = w[kB1 + j];
#pragma unroll
    for (int i = 0; i < kIn; ++i) acc = fmaf(x[i], w[kW1 + i * kHid + j], acc);
    h1[j] = bf(fmaxf(acc, 0.f));
  }
  float o0 = w[kB3], o1 = w[kB3 + 1];
  for (int j = 0; j < kHid; ++j) {
    float acc = w[kB2 + j];
#pragma unroll
    for (int k = 0; k < kHid; ++k) acc = fmaf(h1[k], w[kW2 + k * kHid + j], acc);
    const float h2 = bf(fmaxf(acc, 0.f));
    o0 = fmaf(h2, w[kW3 + j * kOut], o0);
    o1 = fmaf(h2, w[kW3 + j * kOut + 1], o1);
  }
  out[0] = o0;
  out[1] = o1;
}

// Predicted jumps of *count feature vectors (the listed sites: their count
// is DevState::snap_count).
__global__ void __launch_bounds__(128) k_mlp_infer(const float *__restrict__ feat,
                                                   const int *count,
                                                   const float *__restrict__ params_bf,
                                                   float *__restrict__ pred) {
  __shared__ float w[kMlpParams];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = params_bf[i];
  __syncthreads();
  const int ns = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    float o[2];
    mlp_forward(w, feat + (size_t)i * kIn, o);
    pred[2 * (size_t)i] = o[0];
    pred[2 * (size_t)i + 1] = o[1];
  }
}

// The jumped sites: site i of the list moves by round(pred_i * r), clamped to
// the grid; fixed sites, and jumps onto zero density, stay.  They go into the
// bitmap after the current one, with their histories (unchanged: a jump is
// not a Lloyd move) and ids.
__global__ void __launch_bounds__(256) k_apply(LevelBufs a, const float *__restrict__ pred) {
  DevState *st = a.st;
  const int n = a.n, cur = st->snap_cur, hc = st->snap_hist, ns = st->snap_count;
  const float r = st->feat_scale;
  uint64_t *nxt = cur == 0 ? a.bits[1] : (cur == 1 ? a.bits[2] : a.bits[0]);
  unsigned *cnx = cur == 0 ? a.counts[1] : (cur == 1 ? a.counts[2] : a.counts[0]);
  unsigned m2 = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    const uint32_t e = a.list[i];
    const int sx = (int)(e & 0x7fffu), sy = (int)(e >> 16);
    int nx = sx, ny = sy;
    if (!(e & 0x8000u)) {
      const float jx = pred[2 * (size_t)i] * r, jy = pred[2 * (size_t)i + 1] * r;
      if (isfinite(jx) && isfinite(jy)) {
        const int cx = min(max((int)rintf(fminf(fmaxf(jx, -1e6f), 1e6f)) + sx, 0), n - 1);
        const int cy = min(max((int)rintf(fminf(fmaxf(jy, -1e6f), 1e6f)) + sy, 0), n - 1);
        if (a.density[(size_t)cy * n + cx] != 0.0f) {
          nx = cx;
          ny = cy;
        }
      }
    }
    m2 = max(m2, (unsigned)((nx - sx) * (nx - sx) + (ny - sy) * (ny - sy)));
    const size_t widx = (size_t)(ny / kBand) * n + nx;
    const unsigned long long bit = 1ull << (ny % kBand);
    const unsigned long long old = atomicOr(reinterpret_cast<unsigned long long *>(nxt + widx), bit);
    if (!(old & bit)) atomicAdd(cnx + widx / kListWords, 1u);
    const size_t pid = (size_t)sy * n + sx, npid = (size_t)ny * n + nx;
    a.hist[hc ^ 1][npid] = a.hist[hc][pid];
    if (a.ids[0]) a.ids[hc ^ 1][npid] = a.ids[hc][pid];
  }
  m2 = __reduce_max_sync(0xffffffffu, m2);
  if ((threadIdx.x & 31) == 0 && m2) atomicMax(&st->gate_jump2, m2);
}

// Switch to the jumped sites for the energy pass, remembering the state to
// restore: current bitmap, covering bound (grown by the largest jump: every
// density pixel was within cover of its owner, which moved by at most that).
__global__ void k_gate_switch(DevState *st, int n) {
  const int cur = st->cur;
  st->gate_cur = cur;
  st->gate_cover = st->cover;
  const unsigned j2 = st->gate_jump2;
  int j = (int)sqrtf((float)j2);
  while (j * j < (int)j2) ++j;
  st->cover = min(st->cover + j, 2 * n);
  st->cur = cur == 2 ? 0 : cur + 1;
  st->hist_cur ^= 1;
  st->gate_jump2 = 0;
}

// After the energy pass: keep the jump (clear the bitmap the next iteration
// writes) or undo it (clear the jumped bitmap, restore the state).
__global__ void __launch_bounds__(256) k_gate_resolve(LevelBufs a) {
  DevState *st = a.st;
  const int g = st->gate_cur, acc = st->gate_accept;
  const int k = acc ? (g + 2) % 3 : (g + 1) % 3;
  uint64_t *bz = k == 0 ? a.bits[0] : (k == 1 ? a.bits[1] : a.bits[2]);
  unsigned *cz = k == 0 ? a.counts[0] : (k == 1 ? a.counts[1] : a.counts[2]);
  const size_t nwords = (size_t)(a.n / kBand) * a.n;
  const size_t nlb = (nwords + kListWords - 1) / kListWords;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (size_t)gridDim.x * blockDim.x;
  for (size_t i = t0; i < nwords; i += gs) bz[i] = 0ull;
  for (size_t i = t0; i < nlb; i += gs) cz[i] = 0u;
  if (t0 == 0) {
    st->gate_tried += 1;
    st->gate_kept += acc;
    if (!acc) {
      st->cur = g;
      st->cover = st->gate_cover;
      st->hist_cur ^= 1;
    }
  }
}

// Features of the listed sites without their cells (training samples).
__global__ void __launch_bounds__(256) k_features(LevelBufs a, int *out_ids, int *out_xy) {
  const DevState *st = a.st;
  const int n = a.n, hc = st->snap_hist, ns = st->snap_count;
  const float r = st->feat_scale, ir = 1.0f / r;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    const uint32_t e = a.list[i];
    const int sx = (int)(e & 0x7fffu), sy = (int)(e >> 16);
    const size_t pid = (size_t)sy * n + sx;
    const uint64_t h = a.hist[hc][pid];
    float *f = a.feat + (size_t)i * kIn;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      f[2 * k] = (float)(int8_t)(h >> (16 * k)) * ir;
      f[2 * k + 1] = (float)(int8_t)(h >> (16 * k + 8)) * ir;
    }
    const float *d = a.density;
    const float r0 = d[pid];
    const int xa = max(sx - 1, 0), xb = min(sx + 1, n - 1), ya = max(sy - 1, 0), yb = min(sy + 1, n - 1);
    const float gx = (d[(size_t)sy * n + xb] - d[(size_t)sy * n + xa]) / (float)(xb - xa);
    const float gy = (d[(size_t)yb * n + sx] - d[(size_t)ya * n + sx]) / (float)(yb - ya);
    f[8] = r0 > 0.f ? gx / r0 * r : 0.f;
    f[9] = r0 > 0.f ? gy / r0 * r : 0.f;
    if (out_ids) out_ids[i] = a.ids[0] ? a.ids[hc][pid] : -1;
    if (out_xy) {
      out_xy[2 * i] = sx;
      out_xy[2 * i + 1] = sy;
    }
  }
}

// Every listed site gets its list index as id, and an empty history.
__global__ void __launch_bounds__(256) k_ids_init(LevelBufs a) {
  const DevState *st = a.st;
  const int n = a.n, hc = st->snap_hist, ns = st->snap_count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    const uint32_t e = a.list[i];
    const size_t pid = (size_t)(e >> 16) * n + (e & 0x7fffu);
    a.ids[hc][pid] = i;
    a.hist[hc][pid] = 0ull;
  }
}

// ---- training: forward, backward, Adam -----------------------------------

// splitmix-style hash: the sample of batch slot `i` at step `step`
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

constexpr int kTrainTile = 64;  // samples per block

// One block: forward and backward of kTrainTile samples (x: 10 features,
// y: 2 targets per sample, 12 floats), the block's weight gradients summed
// in fixed order and added to grad (divided by the batch size).
__global__ void __launch_bounds__(kTrainTile) k_mlp_grad(const float *__restrict__ samples,
                                                         long long count,
                                                         const float *__restrict__ master,
                                                         float *grad, float *loss, int batch,
                                                         unsigned long long seed, int step) {
  extern __shared__ float sm[];
  float *w = sm;                              // bfloat16-rounded weights
  float *X = w + kMlpParams;                  // [tile][10]
  float *H1 = X + kTrainTile * kIn;           // [tile][64]
  float *H2 = H1 + kTrainTile * kHid;         // [tile][64]
  float *D2 = H2 + kTrainTile * kHid;         // dL/dz2 [tile][64]
  float *D1 = D2 + kTrainTile * kHid;         // dL/dz1 [tile][64]
  float *DO = D1 + kTrainTile * kHid;         // dL/dout [tile][2]
  const int t = threadIdx.x;
  for (int i = t; i < kMlpParams; i += blockDim.x) w[i] = bf(master[i]);
  __syncthreads();
  const int slot = blockIdx.x * kTrainTile + t;
  float l = 0.f;
  if (slot < batch) {
    const long long s = (long long)(mix64(seed ^ ((unsigned long long)step << 32) ^ (unsigned)slot) %
                                    (unsigned long long)count);
    const float *sp = samples + s * 12;
    float x[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = X[t * kIn + i] = bf(sp[i]);
    for (int j = 0; j < kHid; ++j) {
      float acc = w[kB1 + j];
#pragma unroll
      for (int i = 0; i < kIn; ++i) acc = fmaf(x[i], w[kW1 + i * kHid + j], acc);
      H1[t * kHid + j] = bf(fmaxf(acc, 0.f));
    }
    float o0 = w[kB3], o1 = w[kB3 + 1];
    for (int j = 0; j < kHid; ++j) {
      float acc = w[kB2 + j];
      for (int k = 0; k < kHid; ++k) acc = fmaf(H1[t * kHid + k], w[kW2 + k * kHid + j], acc);
      const float h = bf(fmaxf(acc, 0.f));
      H2[t * kHid + j] = h;
      o0 = fmaf(h, w[kW3 + j * kOut], o0);
      o1 = fmaf(h, w[kW3 + j * kOut + 1], o1);
    }
    const float d0 = o0 - sp[10], d1 = o1 - sp[11];
    l = 0.5f * (d0 * d0 + d1 * d1);
    DO[t * 2] = d0;
    DO[t * 2 + 1] = d1;
    for (int j = 0; j < kHid; ++j) {
      const float g = d0 * w[kW3 + j * kOut] + d1 * w[kW3 + j * kOut + 1];
      D2[t * kHid + j] = H2[t * kHid + j] > 0.f ? g : 0.f;
    }
    for (int k = 0; k < kHid; ++k) {
      float g = 0.f;
      for (int j = 0; j < kHid; ++j) g = fmaf(w[kW2 + k * kHid + j], D2[t * kHid + j], g);
      D1[t * kHid + k] = H1[t * kHid + k] > 0.f ? g : 0.f;
    }
  } else {
    for (int i = 0; i < kIn; ++i) X[t * kIn + i] = 0.f;
    for (int j = 0; j < kHid; ++j) H1[t * kHid + j] = H2[t * kHid + j] = D2[t * kHid + j] = D1[t * kHid + j] = 0.f;
    DO[t * 2] = DO[t * 2 + 1] = 0.f;
  }
  __syncthreads();
  const float inv = 1.0f / (float)batch;
  for (int e = t; e < kMlpParams; e += blockDim.x) {
    float g = 0.f;
    if (e < kB1) {
      const int i = e / kHid, k = e % kHid;
      for (int q = 0; q < kTrainTile; ++q) g = fmaf(X[q * kIn + i], D1[q * kHid + k], g);
    } else if (e < kW2) {
      for (int q = 0; q < kTrainTile; ++q) g += D1[q * kHid + (e - kB1)];
    } else if (e < kB2) {
      const int k = (e - kW2) / kHid, j = (e - kW2) % kHid;
      for (int q = 0; q < kTrainTile; ++q) g = fmaf(H1[q * kHid + k], D2[q * kHid + j], g);
    } else if (e < kW3) {
      for (int q = 0; q < kTrainTile; ++q) g += D2[q * kHid + (e - kB2)];
    } else if (e < kB3) {
      const int j = (e - kW3) / kOut, o = (e - kW3) % kOut;
      for (int q = 0; q < kTrainTile; ++q) g = fmaf(H2[q * kHid + j], DO[q * 2 + o], g);
    } else {
      for (int q = 0; q < kTrainTile; ++q) g += DO[q * 2 + (e - kB3)];
    }
    atomicAdd(grad + e, g * inv);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((t & 31) == 0) atomicAdd(loss, l * inv);
}

// Adam step on the FP32 master weights; clears the gradient; writes the
// bfloat16-rounded copy used for inference.  (Blocks add their gradients with
// atomics, so training is not bit-reproducible; inference is.)
__global__ void __launch_bounds__(256) k_adam(float *master, float *grad, float *m, float *v,
                                              float *params_bf, float lr, int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float g = grad[i];
  grad[i] = 0.f;
  const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step)), vh = vi / (1.f - powf(b2, (float)step));
  master[i] -= lr * mh / (sqrtf(vh) + eps);
  params_bf[i] = bf(master[i]);
}

__global__ void k_round_params(const float *master, float *params_bf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kMlpParams) params_bf[i] = bf(master[i]);
}

int mlp_param_count() { return kMlpParams; }

cudaError_t launch_mlp_infer(const float *feat, const int *count, const float *params_bf,
                             float *pred, int grid, cudaStream_t s) {
  k_mlp_infer<<<grid, 128, 0, s>>>(feat, count, params_bf, pred);
  return cudaGetLastError();
}

cudaError_t launch_apply(const LevelBufs &b, const float *pred, int grid, cudaStream_t s) {
  k_apply<<<grid, 256, 0, s>>>(b, pred);
  return cudaGetLastError();
}

cudaError_t launch_gate_switch(DevState *st, int n, cudaStream_t s) {
  k_gate_switch<<<1, 1, 0, s>>>(st, n);
  return cudaGetLastError();
}

cudaError_t launch_gate_resolve(const LevelBufs &b, int grid, cudaStream_t s) {
  k_gate_resolve<<<grid, 256, 0, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_features(const LevelBufs &b, int *ids, int *xy, int grid, cudaStream_t s) {
  k_features<<<grid, 256, 0, s>>>(b, ids, xy);
  return cudaGetLastError();
}

cudaError_t launch_ids_init(const LevelBufs &b, int grid, cudaStream_t s) {
  k_ids_init<<<grid, 256, 0, s>>>(b);
  return cudaGetLastError();
}

size_t mlp_grad_smem() {
  return (size_t)(kMlpParams + kTrainTile * (kIn + 4 * kHid + 2)) * sizeof(float);
}

cudaError_t mlp_configure() {
  return cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)mlp_grad_smem());
}

cudaError_t launch_mlp_train_step(const float *samples, long long count, float *master,
                                  float *grad, float *m, float *v, float *params_bf, float *loss,
                                  int batch, unsigned long long seed, int step, float lr,
                                  cudaStream_t s) {
  const int blocks = (batch + kTrainTile - 1) / kTrainTile;
  k_mlp_grad<<<blocks, kTrainTile, mlp_grad_smem(), s>>>(samples, count, master, grad, loss,
                                                         batch, seed, step);
  k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, grad, m, v, params_bf, lr, step + 1);
  return cudaGetLastError();
}

cudaError_t launch_round_params(const float *master, float *params_bf, cudaStream_t s) {
  k_round_params<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, params_bf);
  return cudaGetLastError();
}

}  // namespace cvtgb
