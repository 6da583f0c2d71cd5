// jfa.cu -- jump-flooding Voronoi labelling: an approximate labeller beside
// the exact one (labeller.cu), with its error measured against it.
//
// The result is a label grid of one int32 per pixel (x in the low, y in the
// high 16 bits), the same words as the reference's short2 grids; the grids
// between launches hold (x << 16) | y instead, the order of the tie rule, and
// the last launch swaps the halves back.  A step of offset k gives pixel p
// the nearest of the nine labels at p + (dx, dy) k, dx, dy in {-1, 0, 1};
// ties go to the smaller x, then the smaller y (the exact labeller's column
// order).  The schedule is k = n/2, n/4, ..., 1 and one more step of 1 (for a
// side that is not a power of two, from the largest power of two <= n/2).
// Between launches "no label" is kJfaNone, the point (16383, 16383): farther
// from every pixel than any site, so it needs no test of its own; the
// seeding writes it and the last launch turns it into MARKER.
//
// All kernels work on units of 16 pixels: (a, b, i) at column x0 + a cs + i,
// row y + b k (a, b in {0, 1}, i < 4), whose candidates lie in 16 aligned
// 16-byte words (r, s) at column x0 + (s - 1) cs, row y + (r - 1) k.  For k a
// multiple of 4, cs = k and a pixel's candidates are component i of nine of
// the words; for k = 1 or 2, cs = 4 (eight adjacent columns).  The unit walks
// its 64 labels once: each is unpacked once, and its key for a pixel p,
//   e = |c|^2 - 2 c.p + bias  (= |c - p|^2 - |p|^2 + bias),
// costs one multiply-add per further pixel that uses it; |p|^2 is the same for
// all nine candidates of p, so (e, x, y) orders them as (distance, x, y) does.
// A pixel's first candidate initialises its key; the other eight compare.
// The compare and select of the 64-bit keys (four integer-ALU instructions
// per candidate) bound the kernels: the integer ALU pipe runs at ~85 %.
//
//   * k > H/2: k_jfa_step, one launch per step, one unit per thread, every
//     load and store 128-bit (a warp reads 512 contiguous bytes per row).
//   * H = 0 (the fastest on GB300, as the autotuner finds): every step its
//     own launch, k_jfa_step down to k = 4, k_jfa_step_small for 2, 1, 1.
//   * H = 8, 16 or 32: k = H/2, ..., 1, 1 in one k_jfa_tail<H> launch.  A
//     block loads its 64 x 64 tile with an H-pixel halo ((64 + 2H)^2 labels)
//     into shared memory with one TMA tile copy, runs the steps there on a
//     region that shrinks by each step's offset, ping-ponging between two
//     shared buffers, and writes the tile back with 128-bit stores.  It saves
//     DRAM traffic, which is not the limit, and costs halo work, barriers and
//     instruction-cache misses (five unrolled steps), so it runs slower than
//     separate launches.
#include "gcvt_internal.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

namespace cvtgb {

constexpr int kTile = 64;
constexpr int kTailThreads = 128;
// keeps e = |c - p|^2 - |p|^2 + kJfaBias in [0, 2^31) for pixels and labels of
// a grid of side <= 8192 (|p|^2 < 2^27; |c - p|^2 < 2^30 with kJfaNone)
constexpr unsigned kJfaBias = 1u << 27;
// Tail of halo H: steps H/2, H/4, ..., 1 and the extra 1 (they sum to H) on
// a (64 + 2H)^2 region; H = 8, 16 or 32 (fusion depths the autotuner tries).
template <int H> __host__ __device__ constexpr int tail_reg() { return kTile + 2 * H; }
template <int H> constexpr unsigned tail_bytes() {
  return 2u * tail_reg<H>() * tail_reg<H>() * 4u + 64u;  // two buffers + mbarrier
}

__device__ __forceinline__ int lab_x(uint32_t v) { return (int)(int16_t)(v & 0xffffu); }
__device__ __forceinline__ int lab_y(uint32_t v) { return (int)(int16_t)(v >> 16); }

__device__ __forceinline__ unsigned long long kmin(unsigned long long a, unsigned long long b) {
  return b < a ? b : a;
}

__device__ __forceinline__ uint32_t comp(const uint4 &v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// the words of four keys, as they are between launches
__device__ __forceinline__ uint4 words(const unsigned long long (&k)[4]) {
  return make_uint4((uint32_t)k[0], (uint32_t)k[1], (uint32_t)k[2], (uint32_t)k[3]);
}

// a word between launches -> the label of the result (MARKER for none)
__device__ __forceinline__ uint32_t final_label(uint32_t w) {
  return w == kJfaNone ? kMarkerWord : __byte_perm(w, 0, 0x1032);
}

__device__ __forceinline__ uint4 final_labels(uint4 v) {
  return make_uint4(final_label(v.x), final_label(v.y), final_label(v.z), final_label(v.w));
}

// The 16 words (r, s) of a unit at column x0 + (s - 1) cs, row y + (r - 1) k;
// outside the grid kJfaNone.  (A second path without the bounds tests, for
// units wholly inside the grid, measured slower: it raised the registers.)
__device__ __forceinline__ void unit_load(const uint32_t *__restrict__ in, int n, int x0, int y,
                                          int k, int cs, uint4 (&w)[4][4]) {
  const uint4 none = make_uint4(kJfaNone, kJfaNone, kJfaNone, kJfaNone);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int yy = y + (r - 1) * k;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int xx = x0 + (s - 1) * cs;
      w[r][s] = (yy >= 0 && yy < n && xx >= 0 && xx < n)
                    ? __ldg(reinterpret_cast<const uint4 *>(in + (size_t)yy * n + xx))
                    : none;
    }
  }
}

// The nearest label of each pixel of a unit (see the file comment) among its
// nine candidates, words (x << 16) | y: best[a][b][i] = (e << 32) | word,
// smallest first.
// KS = 0: cs = k, k a multiple of 4 (any value); KS = 1 or 2: k = KS, cs = 4.
template <int KS>
__device__ __forceinline__ void unit_best(const uint4 (&w)[4][4], int x0, int y, int k,
                                          unsigned long long (&best)[2][2][4]) {
  const unsigned m2x = 0u - 2u * (unsigned)x0, m2y = 0u - 2u * (unsigned)y;
  const unsigned m2k = 0u - 2u * (unsigned)(KS ? KS : k);
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t c = comp(w[r][s], j);
        const unsigned cx = c >> 16, cy = c & 0xffffu;
        // e for the pixel at (x0, y)
        const unsigned base = cx * cx + cy * cy + kJfaBias + cx * m2x + cy * m2y;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
          if (r - 1 - b < -1 || r - 1 - b > 1) continue;
          const unsigned eb = b ? base + cy * m2k : base;
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              unsigned e;
              bool first;  // the pixel's first candidate in this loop order
              if (KS == 0) {
                if (i != j || s - 1 - a < -1 || s - 1 - a > 1) continue;
                e = eb + cx * (0u - 2u * (unsigned)i) + (a ? cx * m2k : 0u);
                first = r - 1 - b == -1 && s - 1 - a == -1;
              } else {
                const int off = 4 * (s - 1) + j - 4 * a - i;
                if (off != -KS && off != 0 && off != KS) continue;
                e = eb + cx * (0u - 2u * (unsigned)(4 * a + i));
                first = r - 1 - b == -1 && off == -KS;
              }
              const unsigned long long key = ((unsigned long long)e << 32) | c;
              best[a][b][i] = first ? key : kmin(best[a][b][i], key);
            }
        }
      }
}

// One step of offset k (a multiple of 4): thread qi of row yi takes the unit
// with cs = k at x0 = (qi / (k/4)) 2k + 4 (qi % (k/4)), y = (yi / k) 2k + yi % k.
__global__ void __launch_bounds__(256) k_jfa_step(const uint32_t *__restrict__ in,
                                                  uint32_t *__restrict__ out, int n, int k) {
  const int kq = k / 4;
  const int blocks = (n + 2 * k - 1) / (2 * k);  // k-blocks of even index
  const int qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= blocks * kq) return;
  const int yi = blockIdx.y;
  const int x0 = (qi / kq) * 2 * k + (qi % kq) * 4;
  const int y = (yi / k) * 2 * k + (yi % k);
  uint4 w[4][4];
  unit_load(in, n, x0, y, k, k, w);
  unsigned long long best[2][2][4];
  unit_best<0>(w, x0, y, k, best);
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int py = y + b * k;
    if (py >= n) continue;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int px = x0 + a * k;
      if (px >= n) continue;
      *reinterpret_cast<uint4 *>(out + (size_t)py * n + px) = words(best[a][b]);
    }
  }
}

// A step of offset KS = 2 or 1 (on the last step, "no label" becomes MARKER):
// thread qi of row pair yi takes the unit with cs = 4 at x0 = 8 qi,
// y = (yi / KS) 2 KS + yi % KS.
template <int KS, bool LAST>
__global__ void __launch_bounds__(256) k_jfa_step_small(const uint32_t *__restrict__ in,
                                                        uint32_t *__restrict__ out, int n) {
  const int qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= n / 8) return;
  const int yi = blockIdx.y;
  const int x0 = 8 * qi, y = (yi / KS) * 2 * KS + yi % KS;
  uint4 w[4][4];
  unit_load(in, n, x0, y, KS, 4, w);
  unsigned long long best[2][2][4];
  unit_best<KS>(w, x0, y, KS, best);
#pragma unroll
  for (int b = 0; b < 2; ++b)
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const uint4 v = words(best[a][b]);
      *reinterpret_cast<uint4 *>(out + (size_t)(y + b * KS) * n + x0 + 4 * a) =
          LAST ? final_labels(v) : v;
    }
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// One step of offset K inside the tail's shared buffers (side R = 64 + 2H,
// grid position of [0][0] = (ox, oy)): pixels of rows and columns [HH, R - HH)
// (HH = the halo left after the step) from `cur` into `nxt`.  Units of cs = K
// for K >= 4, cs = 4 for K < 4 (their columns rounded out to whole units;
// the extra pixels lie outside the region and are never read as valid).
// Pixels outside the grid stay kJfaNone.
template <int K, int HH, int R>
__device__ __forceinline__ void tail_step(const uint32_t *__restrict__ cur,
                                          uint32_t *__restrict__ nxt, int ox, int oy, int n,
                                          bool inner) {
  constexpr int KS = K >= 4 ? 0 : K;
  constexpr int CS = K >= 4 ? K : 4;
  constexpr int W = R - 2 * HH;               // the region's side
  constexpr int PAIRS = W / 2;                // row pairs (y, y + K)
  constexpr int X0 = KS ? (HH / 4) * 4 : HH;  // first unit's column
  constexpr int UNITS = KS ? (R - HH - X0 + 7) / 8 : W / 8;
  static_assert(W % (2 * K) == 0, "rows pair up");
  static_assert(KS || (W % (2 * K) == 0 && HH % 4 == 0), "units tile the region");
  static_assert(X0 - CS >= 0 && HH >= K, "reads stay in the buffer");
  static_assert(KS ? X0 + 8 * UNITS + 4 <= R : HH + W + K <= R, "reads stay in the buffer");
  for (int u = threadIdx.x; u < PAIRS * UNITS; u += kTailThreads) {
    const int p = u / UNITS, q = u % UNITS;
    const int y = HH + (p / K) * 2 * K + p % K;
    const int x0 = KS ? X0 + 8 * q : HH + (q / (K / 4)) * 2 * K + 4 * (q % (K / 4));
    uint4 w[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s < 4; ++s)
        w[r][s] = *reinterpret_cast<const uint4 *>(cur + (y + (r - 1) * K) * R + x0 + (s - 1) * CS);
    unsigned long long best[2][2][4];
    unit_best<KS>(w, ox + x0, oy + y, K, best);
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int row = y + b * K, col = x0 + a * CS;
        uint4 v = words(best[a][b]);
        if (!inner) {
          const int gy = oy + row, gx = ox + col;
          const bool rin = gy >= 0 && gy < n;
          if (!rin || gx < 0 || gx >= n) v.x = kJfaNone;
          if (!rin || gx + 1 < 0 || gx + 1 >= n) v.y = kJfaNone;
          if (!rin || gx + 2 < 0 || gx + 2 >= n) v.z = kJfaNone;
          if (!rin || gx + 3 < 0 || gx + 3 >= n) v.w = kJfaNone;
        }
        *reinterpret_cast<uint4 *>(nxt + row * R + col) = v;
      }
  }
}

// Steps K, K/2, ..., 1 and the extra 1; HH is the halo left after step K.
template <int K, int HH, int R>
__device__ __forceinline__ uint32_t *tail_steps(uint32_t *cur, uint32_t *nxt, int ox, int oy,
                                                int n, bool inner) {
  tail_step<K, HH, R>(cur, nxt, ox, oy, n, inner);
  __syncthreads();
  if constexpr (K > 1) {
    return tail_steps<K / 2, HH + K / 2, R>(nxt, cur, ox, oy, n, inner);
  } else if constexpr (HH < (R - kTile) / 2) {
    return tail_steps<1, HH + 1, R>(nxt, cur, ox, oy, n, inner);  // the extra step of 1
  } else {
    return nxt;
  }
}

// Steps H/2 .. 1, 1 on one 64 x 64 tile; `tm` maps the input label grid
// (n x n uint32, box (64 + 2H)^2).  err[0] is set if the tile copy does not
// arrive within the wait limit (the block then writes nothing).
template <int H>
__global__ void __launch_bounds__(kTailThreads) k_jfa_tail(const __grid_constant__ CUtensorMap tm,
                                                           uint32_t *__restrict__ out, int n,
                                                           int *err) {
  constexpr int kHalo = H, kReg = tail_reg<H>();
  extern __shared__ __align__(1024) uint32_t smem[];
  uint32_t *buf0 = smem, *buf1 = smem + kReg * kReg;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + 2 * kReg * kReg);
  const int tx = blockIdx.x * kTile, ty = blockIdx.y * kTile;
  const int ox = tx - kHalo, oy = ty - kHalo;  // grid position of buf[0][0]
  const int tid = threadIdx.x;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)),
                 "r"((unsigned)(kReg * kReg * 4))
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(buf0)),
        "l"(reinterpret_cast<uint64_t>(&tm)), "r"(ox), "r"(oy), "r"(smem_addr(mbar))
        : "memory");
  }
  // wait for the tile, a bounded number of times
  unsigned done = 0;
  for (int it = 0; it < (1 << 22) && !done; ++it)
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_addr(mbar)), "r"(0u)
        : "memory");
  if (!__syncthreads_and((int)done)) {
    if (tid == 0) atomicOr(err, 1);
    return;
  }
  // the copy fills positions outside the grid with zeros: no label there
  const bool inner = ox >= 0 && oy >= 0 && ox + kReg <= n && oy + kReg <= n;
  if (!inner) {
    for (int p = tid; p < kReg * kReg; p += kTailThreads) {
      const int gx = ox + p % kReg, gy = oy + p / kReg;
      if (gx < 0 || gy < 0 || gx >= n || gy >= n) buf0[p] = kJfaNone;
    }
  }
  __syncthreads();
  const uint32_t *res = tail_steps<H / 2, H / 2, kReg>(buf0, buf1, ox, oy, n, inner);
  // the tile: buffer rows / columns [H, H + 64), 16-byte stores, as labels
  for (int p = tid; p < kTile * kTile / 4; p += kTailThreads) {
    const int i = p / (kTile / 4), j = 4 * (p % (kTile / 4));
    const uint4 v = *reinterpret_cast<const uint4 *>(res + (kHalo + i) * kReg + kHalo + j);
    if (ty + i < n && tx + j < n)
      *reinterpret_cast<uint4 *>(out + (size_t)(ty + i) * n + tx + j) = final_labels(v);
  }
}

// Pixels whose label differs from the exact one, and pixels whose label is
// strictly farther than the exact one's (the jump-flooding error proper).
__global__ void __launch_bounds__(256) k_jfa_compare(const uint32_t *__restrict__ jfa,
                                                     const uint32_t *__restrict__ exact, int n,
                                                     unsigned long long *counts) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned diff = 0, far = 0;
  if (p < (size_t)n * n) {
    const uint32_t a = jfa[p], b = exact[p];
    if (a != b) {
      diff = 1;
      const int x = (int)(p % n), y = (int)(p / n);
      const int da = a == kMarkerWord ? 0x7fffffff
                                      : (lab_x(a) - x) * (lab_x(a) - x) + (lab_y(a) - y) * (lab_y(a) - y);
      const int db = (lab_x(b) - x) * (lab_x(b) - x) + (lab_y(b) - y) * (lab_y(b) - y);
      far = da > db;
    }
  }
  diff = __reduce_add_sync(0xffffffffu, diff);
  far = __reduce_add_sync(0xffffffffu, far);
  if ((threadIdx.x & 31) == 0 && diff) {
    atomicAdd(counts, (unsigned long long)diff);
    if (far) atomicAdd(counts + 1, (unsigned long long)far);
  }
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
bool g_tail_configured[64] = {};

template <int H>
cudaError_t tail_attr() {
  return cudaFuncSetAttribute(k_jfa_tail<H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tail_bytes<H>());
}

template <int H>
cudaError_t launch_tail(uint32_t *in, uint32_t *out, int n, int *err, cudaStream_t s) {
  CUtensorMap tm;
  const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)n * 4};
  const cuuint32_t box[2] = {(cuuint32_t)tail_reg<H>(), (cuuint32_t)tail_reg<H>()};
  const cuuint32_t estr[2] = {1, 1};
  if (g_encode(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, in, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  const dim3 grid((unsigned)(n / kTile), (unsigned)(n / kTile));
  k_jfa_tail<H><<<grid, kTailThreads, tail_bytes<H>(), s>>>(tm, out, n, err);
  return cudaGetLastError();
}
}  // namespace

cudaError_t jfa_configure() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!g_encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (!g_tail_configured[dev]) {
    if ((e = tail_attr<8>()) != cudaSuccess) return e;
    if ((e = tail_attr<16>()) != cudaSuccess) return e;
    if ((e = tail_attr<32>()) != cudaSuccess) return e;
    g_tail_configured[dev] = true;
  }
  return cudaSuccess;
}

// Jump flooding of the grid `a` (seeded: every site holds its word
// (x << 16) | y, kJfaNone elsewhere) for a grid of side n (a multiple of 64 >= 128); `b` is
// the ping-pong partner; steps above tail_halo / 2 run one launch each, the
// rest in one fused tail launch (tail_halo = 8, 16 or 32); tail_halo = 0:
// every step its own launch.  Returns the buffer holding the result in
// *result.
cudaError_t launch_jfa(uint32_t *a, uint32_t *b, int n, int *err, uint32_t **result,
                       cudaStream_t s, int tail_halo) {
  cudaError_t e = jfa_configure();
  if (e != cudaSuccess) return e;
  if (tail_halo != 0 && tail_halo != 8 && tail_halo != 32) tail_halo = 16;
  while (tail_halo > 8 && tail_halo > n / 4) tail_halo /= 2;  // the steps start at <= n/2
  uint32_t *in = a, *out = b;
  int k = 1;
  while (2 * k <= n / 2) k *= 2;  // the largest power of two <= n/2
  for (; k > (tail_halo ? tail_halo / 2 : 2); k /= 2) {
    const int blocks = (n + 2 * k - 1) / (2 * k);
    const dim3 grid((unsigned)((blocks * (k / 4) + 255) / 256), (unsigned)(blocks * k));
    k_jfa_step<<<grid, 256, 0, s>>>(in, out, n, k);
    uint32_t *t = in;
    in = out;
    out = t;
  }
  if (!tail_halo) {  // k = 2, 1 and the extra 1
    const dim3 grid((unsigned)((n / 8 + 255) / 256), (unsigned)(n / 2));
    k_jfa_step_small<2, false><<<grid, 256, 0, s>>>(in, out, n);
    k_jfa_step_small<1, false><<<grid, 256, 0, s>>>(out, in, n);
    k_jfa_step_small<1, true><<<grid, 256, 0, s>>>(in, out, n);
    *result = out;
    return cudaGetLastError();
  }
  if (tail_halo == 8) e = launch_tail<8>(in, out, n, err, s);
  else if (tail_halo == 32) e = launch_tail<32>(in, out, n, err, s);
  else e = launch_tail<16>(in, out, n, err, s);
  *result = out;
  return e;
}

cudaError_t launch_jfa_compare(const uint32_t *jfa, const uint32_t *exact, int n,
                               unsigned long long *counts, cudaStream_t s) {
  const size_t nn = (size_t)n * n;
  k_jfa_compare<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(jfa, exact, n, counts);
  return cudaGetLastError();
}

}  // namespace cvtgb
