// jfa.cu -- jump-flooding Voronoi labelling: an approximate labeller beside
// the exact one (labeller.cu), with its error measured against it.
//
// The label grid holds one int32 per pixel (x in the low, y in the high 16
// bits, MARKER for none), the same words as the reference's short2 grids.
// A step of offset k gives pixel p the nearest of the nine labels at
// p + (dx, dy) k, dx, dy in {-1, 0, 1} (ties: smaller x, then smaller y).
// The schedule is k = n/2, n/4, ..., 1 and one more step of 1 (for a side
// that is not a power of two, from the largest power of two <= n/2).
//
//   * k > H/2: k_jfa_step, one launch per step, sixteen pixels per thread:
//     four groups of four at (x0 + a k, y + b k), whose neighbours are 4 x 4
//     aligned 16-byte words (k is a multiple of 4) -- 16 loads for 16
//     pixels, every load and store 128-bit, a warp reading 512 contiguous
//     bytes per row.  The nearest label is the smallest 64-bit key
//     (distance, then x, then y).
//   * k = H/2, ..., 1, 1: k_jfa_tail<H>, one launch (H = 8, 16 or 32, the
//     fusion depth; 16 by default, the autotuner picks).  A block loads its
//     64 x 64 tile with an H-pixel halo (96 x 96 labels, 36 KB, for H = 16)
//     into shared memory with one TMA tile copy, runs the steps there on a
//     region that shrinks by each step's offset (8 + 4 + 2 + 1 + 1 = 16),
//     ping-ponging between two shared buffers, and writes the tile back with
//     128-bit stores: five passes over the grid for one read and one write.
#include "gcvt_internal.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

namespace cvtgb {

constexpr int kTile = 64;
// Tail of halo H: steps H/2, H/4, ..., 1 and the extra 1 (they sum to H) on
// a (64 + 2H)^2 region; H = 8, 16 or 32 (the fusion depth the autotuner picks).
template <int H> __host__ __device__ constexpr int tail_reg() { return kTile + 2 * H; }
template <int H> constexpr unsigned tail_bytes() {
  return 2u * tail_reg<H>() * tail_reg<H>() * 4u + 64u;  // two buffers + mbarrier
}

__device__ __forceinline__ int lab_x(uint32_t v) { return (int)(int16_t)(v & 0xffffu); }
__device__ __forceinline__ int lab_y(uint32_t v) { return (int)(int16_t)(v >> 16); }

// Comparison key of label c for pixel (x, y): squared distance in the high
// word, the site's (x, y) in the low word (so ties go to the smaller x, then
// y).  The nearest label is the smallest key.  "No label" (MARKER, -32768 in
// both halves) needs no special case: its squared distance from a pixel of a
// grid of side <= 8192 lies in [2^31, 3.4e9], no overflow of 32 bits, and is
// larger than any site's (< 2 * 8192^2).
__device__ __forceinline__ unsigned long long jkey(uint32_t c, int x, int y) {
  const unsigned dx = (unsigned)(lab_x(c) - x), dy = (unsigned)(lab_y(c) - y);
  return ((unsigned long long)(dx * dx + dy * dy) << 32) | __byte_perm(c, 0, 0x1032);
}

__device__ __forceinline__ uint32_t jlabel(unsigned long long k) {
  return __byte_perm((uint32_t)k, 0, 0x1032);
}

__device__ __forceinline__ unsigned long long kmin(unsigned long long a, unsigned long long b) {
  return b < a ? b : a;
}

__device__ __forceinline__ uint32_t comp(const uint4 &v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// One step of offset k (a multiple of 4).  A thread takes the 2 x 2 groups of
// four pixels at (x0 + a k, y + b k), a, b in {0, 1}, (x0, y) in the even
// k-blocks: their nine neighbours each are 4 x 4 aligned 16-byte words, 16
// loads for 16 pixels.
__global__ void __launch_bounds__(256) k_jfa_step(const uint32_t *__restrict__ in,
                                                  uint32_t *__restrict__ out, int n, int k) {
  const int kq = k / 4;
  const int blocks = (n + 2 * k - 1) / (2 * k);  // k-blocks of even index
  const int qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= blocks * kq) return;
  const int yi = blockIdx.y;
  const int x0 = (qi / kq) * 2 * k + (qi % kq) * 4;
  const int y = (yi / k) * 2 * k + (yi % k);
  const uint4 none = make_uint4(kMarkerWord, kMarkerWord, kMarkerWord, kMarkerWord);
  uint4 c[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int yy = y + (r - 1) * k;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int xx = x0 + (s - 1) * k;
      c[r][s] = (yy >= 0 && yy < n && xx >= 0 && xx < n)
                    ? __ldg(reinterpret_cast<const uint4 *>(in + (size_t)yy * n + xx))
                    : none;
    }
  }
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int py = y + b * k;
    if (py >= n) continue;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int px = x0 + a * k;
      if (px >= n) continue;
      uint32_t res[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        unsigned long long best = ~0ull;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int s = 0; s < 3; ++s) best = kmin(best, jkey(comp(c[b + r][a + s], i), px + i, py));
        res[i] = jlabel(best);
      }
      *reinterpret_cast<uint4 *>(out + (size_t)py * n + px) =
          make_uint4(res[0], res[1], res[2], res[3]);
    }
  }
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Steps H/2 .. 1, 1 on one 64 x 64 tile; `tm` maps the input label grid
// (n x n uint32, box (64 + 2H)^2).  err[0] is set if the tile copy does not
// arrive within the wait limit (the block then writes nothing).
template <int H>
__global__ void __launch_bounds__(256) k_jfa_tail(const __grid_constant__ CUtensorMap tm,
                                                  uint32_t *__restrict__ out, int n, int *err) {
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
  for (int p = tid; p < kReg * kReg; p += blockDim.x) {
    const int gx = ox + p % kReg, gy = oy + p / kReg;
    if (gx < 0 || gy < 0 || gx >= n || gy >= n) buf0[p] = kMarkerWord;
  }
  __syncthreads();
  uint32_t *cur = buf0, *nxt = buf1;
  int h = 0;  // rows / columns of the region already out of date
#pragma unroll
  for (int k2 = H; k2 >= 1; k2 >>= 1) {  // k = H/2, ..., 1, then 1 again
    const int k = k2 > 1 ? k2 / 2 : 1;
    h += k;
    const int w = kReg - 2 * h;
    for (int p = tid; p < w * w; p += blockDim.x) {
      const int i = h + p / w, j = h + p % w;  // buffer row, column
      const int gx = ox + j, gy = oy + i;
      unsigned long long best = ~0ull;  // outside the grid: no label
      if (gx >= 0 && gy >= 0 && gx < n && gy < n) {
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx)
            best = kmin(best, jkey(cur[(i + dy * k) * kReg + j + dx * k], gx, gy));
      }
      nxt[i * kReg + j] = best == ~0ull ? kMarkerWord : jlabel(best);
    }
    __syncthreads();
    uint32_t *t = cur;
    cur = nxt;
    nxt = t;
  }
  // the tile: buffer rows / columns [16, 80), 16-byte stores
  for (int p = tid; p < kTile * kTile / 4; p += blockDim.x) {
    const int i = p / (kTile / 4), j = 4 * (p % (kTile / 4));
    const uint32_t *src = cur + (kHalo + i) * kReg + kHalo + j;
    if (ty + i < n && tx + j < n)
      *reinterpret_cast<uint4 *>(out + (size_t)(ty + i) * n + tx + j) =
          *reinterpret_cast<const uint4 *>(src);
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
  k_jfa_tail<H><<<grid, 256, tail_bytes<H>(), s>>>(tm, out, n, err);
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

// Jump flooding of the label grid `a` (seeded: every site labels itself,
// MARKER elsewhere) for a grid of side n (a multiple of 64 >= 128); `b` is
// the ping-pong partner; steps above tail_halo / 2 run one launch each, the
// rest in one fused tail launch (tail_halo = 8, 16 or 32).  Returns the
// buffer holding the result in *result.
cudaError_t launch_jfa(uint32_t *a, uint32_t *b, int n, int *err, uint32_t **result,
                       cudaStream_t s, int tail_halo) {
  cudaError_t e = jfa_configure();
  if (e != cudaSuccess) return e;
  if (tail_halo != 8 && tail_halo != 32) tail_halo = 16;
  while (tail_halo > 8 && tail_halo > n / 4) tail_halo /= 2;  // the steps start at <= n/2
  uint32_t *in = a, *out = b;
  int k = 1;
  while (2 * k <= n / 2) k *= 2;  // the largest power of two <= n/2
  for (; k > tail_halo / 2; k /= 2) {
    const int blocks = (n + 2 * k - 1) / (2 * k);
    const dim3 grid((unsigned)((blocks * (k / 4) + 255) / 256), (unsigned)(blocks * k));
    k_jfa_step<<<grid, 256, 0, s>>>(in, out, n, k);
    uint32_t *t = in;
    in = out;
    out = t;
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
