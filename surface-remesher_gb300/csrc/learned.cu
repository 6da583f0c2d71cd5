// learned.cu -- the learned step: a small per-site MLP that predicts where a
// site's Lloyd trajectory ends, trained on trajectories the plain method
// produces, and applied as a jump that the energy decides on.
//
// Features of a site (k_cell MODE 2): its pending Lloyd displacement (the
// centroid of its cell minus the site, sub-pixel), its last three integer
// moves (newest first) and the density gradient over the density at the
// site, in units of the mean cell radius r: 10 inputs.  The MLP 10 -> 64 ->
// 64 -> 2 (ReLU) predicts the displacement to the site's converged position,
// in units of r.  Weights are bfloat16 (the forward pass rounds weights and
// activations to bfloat16 and accumulates in FP32, the tensor cores'
// arithmetic); training keeps FP32 master weights (Adam).
//
// A jump (kernels below, sequence in api.cu): the plain iteration from the
// sites S also writes their features, the MLP predicts, k_apply places the
// jumped sites L, and the iteration of L decides: L stands if E(L) < E(S),
// otherwise the plain step's sites are current again -- the plain method is
// both the fallback and the test a jump must pass.
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

// A learned step, over charts descs[0 .. nchart) (a single context is a batch
// of one).  The plain iteration from the sites S (k_cell MODE 4: bitmap cur
// -> cur + 1, also the features of S) is followed by:
//   k_apply        the jumped sites L = S + round(pred r) into bitmap cur + 2
//                  (cleared by that iteration); bitmap cur, whose sites are no
//                  longer needed, is cleared for the iteration of L;
//   k_gate_switch  saves the state after the plain iteration and makes L
//                  current, with the covering bound grown by the largest jump;
//   k_list, k_cell MODE 5: the plain iteration of L (L -> bitmap cur), which
//                  also decides: the jump stands if E(L) < E(S);
//   k_gate_clear   clears the bitmap of the loser: the plain step's sites
//                  (bitmap cur + 1) when the jump stands, else L;
//   k_gate_commit  restores the saved state when the jump is rejected -- the
//                  run then goes on from the plain step, exactly as without
//                  the jump.
// An accepted jump thus costs no extra pass: its iteration of L is the next
// Lloyd iteration.  A rejected one costs the pass over L.

// The jumped sites of chart blockIdx.y: listed site i moves by
// round(pred_i * r), clamped to the grid; fixed sites, and jumps onto zero
// density, stay.  A jumped site keeps its history and id (a jump is not a
// Lloyd move) and gets the window of its cell in S grown by twice the jump.
__global__ void __launch_bounds__(256) k_apply(const LevelBufs *__restrict__ descs) {
  const LevelBufs &a = descs[blockIdx.y];
  DevState *st = a.st;
  // no jump when the plain iteration ended the level, or once the schedule
  // has lowered omega below 2 (the plain iterations then settle by
  // themselves; a jump would only knock the sites out of their settling)
  if (st->snap_stopped || st->stopped || st->omega < 2.0f) return;
  const int n = a.n, cur = st->snap_cur, ns = st->snap_count;
  const int lj = cur == 0 ? 2 : cur - 1;  // (cur + 2) mod 3
  const float r = st->feat_scale;
  uint64_t *dst = lj == 0 ? a.bits[0] : (lj == 1 ? a.bits[1] : a.bits[2]);
  unsigned *cdst = lj == 0 ? a.counts[0] : (lj == 1 ? a.counts[1] : a.counts[2]);
  uint64_t *old_bits = cur == 0 ? a.bits[0] : (cur == 1 ? a.bits[1] : a.bits[2]);
  unsigned *old_cnt = cur == 0 ? a.counts[0] : (cur == 1 ? a.counts[1] : a.counts[2]);
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x,
               gs = (size_t)gridDim.x * blockDim.x;
  const size_t nwords = (size_t)(n / kBand) * n, nlb = (nwords + kListWords - 1) / kListWords;
  for (size_t i = t0; i < nwords; i += gs) old_bits[i] = 0ull;
  for (size_t i = t0; i < nlb; i += gs) old_cnt[i] = 0u;
  unsigned m2 = 0;
  for (size_t i = t0; i < (size_t)ns; i += gs) {
    const uint32_t e = a.list[i];
    const int sx = (int)(e & 0x7fffu), sy = (int)(e >> 16);
    int nx = sx, ny = sy;
    if (!(e & 0x8000u)) {
      const float jx = a.pred[2 * i] * r, jy = a.pred[2 * i + 1] * r;
      if (isfinite(jx) && isfinite(jy)) {
        const int cx = min(max((int)rintf(fminf(fmaxf(jx, -1e6f), 1e6f)) + sx, 0), n - 1);
        const int cy = min(max((int)rintf(fminf(fmaxf(jy, -1e6f), 1e6f)) + sy, 0), n - 1);
        if (a.density[(size_t)cy * n + cx] != 0.0f) {
          nx = cx;
          ny = cy;
        }
      }
    }
    const unsigned j2 = (unsigned)((nx - sx) * (nx - sx) + (ny - sy) * (ny - sy));
    m2 = max(m2, j2);
    const size_t widx = (size_t)(ny / kBand) * n + nx;
    const unsigned long long bit = 1ull << (ny % kBand);
    const unsigned long long was = atomicOr(reinterpret_cast<unsigned long long *>(dst + widx), bit);
    // counted per list block, one atomic per block a warp's sites reached
    const int entry = (was & bit) ? -1 : (int)(widx / kListWords);
    const unsigned want = __ballot_sync(__activemask(), entry >= 0);
    if (entry >= 0) {
      const unsigned peers = __match_any_sync(want, entry);
      if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(cdst + entry, (unsigned)__popc(peers));
    }
    const size_t pid = (size_t)sy * n + sx, npid = (size_t)ny * n + nx;
    a.hist[lj][npid] = a.hist[cur][pid];
    if (a.ids[0]) a.ids[lj][npid] = a.ids[cur][pid];
    int j = (int)sqrtf((float)j2);
    while (j * j < (int)j2) ++j;
    a.hint[npid] = (uint8_t)min((int)a.jaux[i] + 2 * j, 255);
  }
  // the block's largest jump, one atomic per block onto the chart's maximum
  __shared__ unsigned wmax[8];
  m2 = __reduce_max_sync(0xffffffffu, m2);
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m2;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) m2 = max(m2, wmax[w]);
    if (m2) atomicMax(&st->gate_jump2, m2);
  }
}

// One thread per chart: save the state after the plain iteration, make the
// jumped sites current.  Every density pixel was within snap_cover of its
// owner in S, which moved by at most the largest jump, so snap_cover plus
// that jump bounds L's covering distance.  A chart whose plain iteration
// stopped its level proposes nothing.
__global__ void k_gate_switch(const LevelBufs *__restrict__ descs, int nchart) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchart) return;
  const LevelBufs &a = descs[c];
  DevState *st = a.st;
  if (st->snap_stopped || st->stopped || st->omega < 2.0f) {  // as k_apply decided
    st->gate_active = 0;
    st->gate_jump2 = 0;
    return;
  }
  *a.gsave = *st;
  const unsigned j2 = st->gate_jump2;
  int j = (int)sqrtf((float)j2);
  while (j * j < (int)j2) ++j;
  st->gate_active = 1;
  st->gate_accept = 0;
  st->gate_e0 = st->energy;  // E(S), from the plain iteration
  st->cover = min(st->snap_cover + j, 2 * a.n);
  st->cur = st->snap_cur == 0 ? 2 : st->snap_cur - 1;
  st->gate_jump2 = 0;
}

// Chart blockIdx.y: clear the bitmap the next iteration writes -- the plain
// step's sites when the jump stands, the jumped sites when it does not.
// Reads the decision only; k_gate_commit changes the state afterwards.
__global__ void __launch_bounds__(256) k_gate_clear(const LevelBufs *__restrict__ descs) {
  const LevelBufs &a = descs[blockIdx.y];
  const DevState *st = a.st;
  if (!st->gate_active) return;
  const int p = a.gsave->cur;  // the plain step's bitmap; the jumped sites are in p + 1
  const int k = st->gate_accept ? p : (p == 2 ? 0 : p + 1);
  uint64_t *bz = k == 0 ? a.bits[0] : (k == 1 ? a.bits[1] : a.bits[2]);
  unsigned *cz = k == 0 ? a.counts[0] : (k == 1 ? a.counts[1] : a.counts[2]);
  const size_t nwords = (size_t)(a.n / kBand) * a.n;
  const size_t nlb = (nwords + kListWords - 1) / kListWords;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (size_t)gridDim.x * blockDim.x;
  for (size_t i = t0; i < nwords; i += gs) bz[i] = 0ull;
  for (size_t i = t0; i < nlb; i += gs) cz[i] = 0u;
}

// One thread per chart: count the jump; a rejected jump restores the state
// saved after the plain iteration (the bitmap written by the jumped sites'
// iteration is cleared ahead by the next iteration, as every third one is).
__global__ void k_gate_commit(const LevelBufs *__restrict__ descs, int nchart) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchart) return;
  const LevelBufs &a = descs[c];
  DevState *st = a.st;
  if (!st->gate_active) return;
  const int acc = st->gate_accept, tried = st->gate_tried + 1, kept = st->gate_kept + acc;
  const double e0 = st->gate_e0, e1 = st->gate_e1;
  if (!acc) *st = *a.gsave;
  st->gate_tried = tried;
  st->gate_kept = kept;
  st->gate_e0 = e0;
  st->gate_e1 = e1;
  st->gate_active = 0;
  __threadfence();
}

// Ids and pixel positions of the listed sites (training samples; their
// features come from a features pass, k_cell MODE 2, over the same list).
__global__ void __launch_bounds__(256) k_features(LevelBufs a, int *out_ids, int *out_xy) {
  const DevState *st = a.st;
  const int n = a.n, cur = st->snap_cur, ns = st->snap_count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    const uint32_t e = a.list[i];
    const int sx = (int)(e & 0x7fffu), sy = (int)(e >> 16);
    const size_t pid = (size_t)sy * n + sx;
    if (out_ids) out_ids[i] = a.ids[0] ? a.ids[cur][pid] : -1;
    if (out_xy) {
      out_xy[2 * i] = sx;
      out_xy[2 * i + 1] = sy;
    }
  }
}

// Every listed site gets its list index as id, and an empty history.
__global__ void __launch_bounds__(256) k_ids_init(LevelBufs a) {
  const DevState *st = a.st;
  const int n = a.n, cur = st->snap_cur, ns = st->snap_count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    const uint32_t e = a.list[i];
    const size_t pid = (size_t)(e >> 16) * n + (e & 0x7fffu);
    a.ids[cur][pid] = i;
    a.hist[cur][pid] = 0ull;
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


// ---- tensor-core forward: tcgen05.mma with accumulators in TMEM -----------
//
// One CTA of 128 threads takes tiles of 128 sites.  Layer 1 (K = 10, padded
// to 16) and layer 2 (K = 64) are tcgen05.mma of kind f16 with bfloat16 A
// (activations, one row per site) and B (weights, one row per output) in
// shared memory in the no-swizzle K-major layout -- 8 x 8 core matrices of
// 128 contiguous bytes, consecutive along K (LBO 128 B), rows of cores
// KC * 128 B apart (SBO) -- and FP32 accumulators D (128 lanes x 64 columns)
// in tensor memory.  Thread m reads row m of D with tcgen05.ld, adds the
// bias, applies ReLU, rounds to bfloat16 and writes row m of the next A;
// layer 3 (64 -> 2) runs on the CUDA cores from the same registers.

constexpr int kTcRows = 128;
constexpr uint32_t kTcA1 = 0, kTcA2 = kTcA1 + kTcRows * 16 * 2, kTcB1 = kTcA2 + kTcRows * 64 * 2,
                   kTcB2 = kTcB1 + 64 * 16 * 2, kTcP = kTcB2 + 64 * 64 * 2,
                   kTcBar = kTcP + 264 * 4, kTcSlot = kTcBar + 8, kTcSmem = kTcSlot + 8;

// byte offset of element (row, k) in a K-major no-swizzle operand with KC
// core matrices along K
__device__ __forceinline__ uint32_t core_off(int row, int k, int kc) {
  return (uint32_t)((((row >> 3) * kc + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1, no swizzle
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t to_smem(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Bounded wait for phase `parity` of the mbarrier; false if it never came.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // a in the low half
  return *reinterpret_cast<const uint32_t *>(&v);
}

__global__ void __launch_bounds__(kTcRows, 1) k_mlp_tc(const float *__restrict__ feat,
                                                       const int *count,
                                                       const float *__restrict__ params_bf,
                                                       float *__restrict__ pred, int *err) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  const int m = threadIdx.x, warp = m >> 5;
  const uint32_t base = to_smem(tsm);
  float *P = reinterpret_cast<float *>(tsm + kTcP);  // b1[64], b2[64], W3[128], b3[2]
  uint32_t *slot = reinterpret_cast<uint32_t *>(tsm + kTcSlot);
  const uint32_t bar = base + kTcBar;
  // weights as bfloat16 B operands: B1[n][k] = W1[k][n] (k < 10), B2[n][k] = W2[k][n]
  for (int e = m; e < 64 * 16; e += kTcRows) {
    const int nn = e / 16, k = e % 16;
    const float w = k < kIn ? params_bf[kW1 + k * kHid + nn] : 0.f;
    *reinterpret_cast<__nv_bfloat16 *>(tsm + kTcB1 + core_off(nn, k, 2)) = __float2bfloat16_rn(w);
  }
  for (int e = m; e < 64 * 64; e += kTcRows) {
    const int nn = e / 64, k = e % 64;
    *reinterpret_cast<__nv_bfloat16 *>(tsm + kTcB2 + core_off(nn, k, 8)) =
        __float2bfloat16_rn(params_bf[kW2 + k * kHid + nn]);
  }
  for (int e = m; e < 64; e += kTcRows) {
    P[e] = params_bf[kB1 + e];
    P[64 + e] = params_bf[kB2 + e];
  }
  for (int e = m; e < 128; e += kTcRows) P[128 + e] = params_bf[kW3 + e];
  if (m < 2) P[256 + m] = params_bf[kB3 + m];
  if (m == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     to_smem(slot)),
                 "r"(128u));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  const uint32_t idesc = mma_idesc(128, 64);
  const int ns = *count;
  uint32_t phase = 0;
  bool ok = true;
  for (int tile = blockIdx.x; tile * kTcRows < ns && ok; tile += gridDim.x) {
    const int i = tile * kTcRows + m;
    // A1 row m: the features as bfloat16, zero beyond the 10th
    float x[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = (i < ns && k < kIn) ? feat[(size_t)i * kIn + k] : 0.f;
#pragma unroll
    for (int c = 0; c < 2; ++c)
      *reinterpret_cast<uint4 *>(tsm + kTcA1 + core_off(m, 8 * c, 2)) =
          make_uint4(pack_bf2(x[8 * c], x[8 * c + 1]), pack_bf2(x[8 * c + 2], x[8 * c + 3]),
                     pack_bf2(x[8 * c + 4], x[8 * c + 5]), pack_bf2(x[8 * c + 6], x[8 * c + 7]));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (m == 0) {
      const uint64_t a = smem_desc(base + kTcA1, 128, 256), b = smem_desc(base + kTcB1, 128, 256);
      asm volatile(
          "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(
              tmem),
          "l"(a), "l"(b), "r"(idesc), "r"(0u)
          : "memory");
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       bar)
                   : "memory");
    }
    ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(ok)) break;
    tc_fence_after();
    // layer 1 epilogue -> A2 row m
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tmem_ld32(lane_base + 32 * half, v);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float h[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) h[q] = fmaxf(v[8 * c + q] + P[32 * half + 8 * c + q], 0.f);
        *reinterpret_cast<uint4 *>(tsm + kTcA2 + core_off(m, 32 * half + 8 * c, 8)) =
            make_uint4(pack_bf2(h[0], h[1]), pack_bf2(h[2], h[3]), pack_bf2(h[4], h[5]),
                       pack_bf2(h[6], h[7]));
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (m == 0) {
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const uint64_t a = smem_desc(base + kTcA2 + 256 * s, 128, 1024),
                       b = smem_desc(base + kTcB2 + 256 * s, 128, 1024);
        asm volatile(
            "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(
                tmem + 64),
            "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)s)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       bar)
                   : "memory");
    }
    ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(ok)) break;
    tc_fence_after();
    // layer 2 epilogue and layer 3 on the CUDA cores
    float o0 = P[256], o1 = P[257];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tmem_ld32(lane_base + 64 + 32 * half, v);
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int j = 32 * half + q;
        const float h = bf(fmaxf(v[q] + P[64 + j], 0.f));
        o0 = fmaf(h, P[128 + 2 * j], o0);
        o1 = fmaf(h, P[128 + 2 * j + 1], o1);
      }
    }
    if (i < ns) {
      pred[2 * (size_t)i] = o0;
      pred[2 * (size_t)i + 1] = o1;
    }
    tc_fence_before();
    __syncthreads();  // A1, A2 and the accumulators are reused by the next tile
    tc_fence_after();
  }
  if (!ok && m == 0) atomicOr(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u));
}

cudaError_t launch_mlp_tc(const float *feat, const int *count, const float *params_bf,
                          float *pred, int *err, cudaStream_t s) {
  static bool configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!configured[dev]) {
    if ((e = cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kTcSmem)) != cudaSuccess)
      return e;
    configured[dev] = true;
  }
  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;
  // two CTAs per SM hold 256 of the 512 TMEM columns
  k_mlp_tc<<<2 * sms, kTcRows, kTcSmem, s>>>(feat, count, params_bf, pred, err);
  return cudaGetLastError();
}

int mlp_param_count() { return kMlpParams; }

cudaError_t launch_mlp_infer(const float *feat, const int *count, const float *params_bf,
                             float *pred, int grid, cudaStream_t s) {
  k_mlp_infer<<<grid, 128, 0, s>>>(feat, count, params_bf, pred);
  return cudaGetLastError();
}

cudaError_t launch_apply(const LevelBufs *descs, int nchart, cudaStream_t s) {
  const int per = max(8, 1216 / max(nchart, 1));  // blocks per chart
  k_apply<<<dim3((unsigned)per, (unsigned)nchart), 256, 0, s>>>(descs);
  return cudaGetLastError();
}

cudaError_t launch_gate_switch(const LevelBufs *descs, int nchart, cudaStream_t s) {
  k_gate_switch<<<(nchart + 127) / 128, 128, 0, s>>>(descs, nchart);
  return cudaGetLastError();
}

cudaError_t launch_gate_resolve(const LevelBufs *descs, int nchart, cudaStream_t s) {
  const int per = max(8, 1216 / max(nchart, 1));
  k_gate_clear<<<dim3((unsigned)per, (unsigned)nchart), 256, 0, s>>>(descs);
  k_gate_commit<<<(nchart + 127) / 128, 128, 0, s>>>(descs, nchart);
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

cudaError_t launch_mlp_grad(const float *samples, long long count, const float *master,
                            float *grad, float *loss, int batch, unsigned long long seed, int step,
                            cudaStream_t s) {
  const int blocks = (batch + kTrainTile - 1) / kTrainTile;
  k_mlp_grad<<<blocks, kTrainTile, mlp_grad_smem(), s>>>(samples, count, master, grad, loss,
                                                         batch, seed, step);
  return cudaGetLastError();
}

cudaError_t launch_round_params(const float *master, float *params_bf, cudaStream_t s) {
  k_round_params<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, params_bf);
  return cudaGetLastError();
}

}  // namespace cvtgb
