// labeller.cu -- exact Voronoi labelling of a site grid, bit-identical to the
// reference's PBA+ (gcvt.cu:77-479 driven by pba2DCompute, gcvt.cu:967-978).
//
// PBA+ resolves every pixel to the nearest site; its ties resolve as follows
// (derived from the kernels and checked against a literal restatement and
// against the reference kernels themselves):
//   * column pass (gcvt.cu:77-216): the vertically nearest site of a column;
//     a tie between the site above-or-at row r and the one below goes to the
//     lower site only when it lies in r's 64-row band (FloodUp's strict '<'
//     at gcvt.cu:114 against the margin merges at gcvt.cu:197-200);
//   * row pass (gcvt.cu:227-479): nearest of the column candidates, ties to
//     the smaller column (kernelColor's '>' break at gcvt.cu:457).
//
// GB300 layout (three kernels instead of ~20 launches and ~60 B/px):
//   * sites live in a bitmap of 64-row words, bits[band][column] -- one
//     64-bit word per column and PBA band, so the band tie rule is "the lower
//     site came from the same word";
//   * k_summary: per (band, column), the nearest site row above / below the
//     band (a scan over bands, 32 columns x 32 band groups per block);
//   * k_rows: one warp per row (one row per block).  The lanes derive the
//     column candidates 32 columns at a time from the bitmap word and the
//     summaries (no column-nearest grid is ever written); candidate (x, g)
//     is the point (x, B = x^2 + g^2) and the pixels it wins lie under the
//     lower convex hull of the points.  Each chunk of 32 first drops, by
//     three rounds of chord removal among its own points (every point
//     strictly above the chord of its neighbours goes), points that cannot be
//     on the hull; the survivors go to a 2/5-row buffer in shared memory, where rounds
//     of simultaneous chord removal over the whole row finish the hull (after
//     24 rounds a sequential monotone chain finishes any input).  Then the
//     lanes write the row's label words from the hull's breakpoints.  A row
//     whose survivors do not fit the buffer is flagged and redone by
//     k_rows_full with a whole-row buffer: the smaller buffer lets 2.5 times
//     the rows share an SM.  The Lloyd iteration does not use this pass (cells.cu
//     sums each site's cell directly); it gives the final label grid and the
//     covering bound at a level's start.
#include "gcvt_internal.cuh"

namespace cvtgb {

// ---------------------------------------------------------------------------
// Site grid <-> bitmap
// ---------------------------------------------------------------------------

// One thread per (band, column): 64 coalesced row reads, one word written.
// A pixel is a site when its x half is not MARKER (gcvt.cu:90); a site pixel
// must hold its own coordinates, else err gets bit 0.
__global__ void k_grid_to_bits(const uint32_t *__restrict__ grid, int n,
                               uint64_t *__restrict__ bits, int *err, int *count) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y;
  if (x >= n) return;
  uint64_t w = 0;
  bool bad = false;
  const uint32_t *p = grid + (size_t)(b * kBand) * n + x;
#pragma unroll 8
  for (int i = 0; i < kBand; ++i) {
    uint32_t v = __ldg(p + (size_t)i * n);
    int vx = (int16_t)(v & 0xffffu);
    if (vx != kMarker) {
      int vy = (int16_t)(v >> 16);
      bad |= (vx != x) || (vy != b * kBand + i);
      w |= 1ull << i;
    }
  }
  bits[(size_t)b * n + x] = w;
  if (bad) atomicOr(err, 1);
  if (count) {  // one atomic per warp: every thread adding to one counter serialises
    const unsigned m = __activemask();
    const unsigned c = __reduce_add_sync(m, (unsigned)__popcll(w));
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1 && c) atomicAdd(count, (int)c);
  }
}

__global__ void k_bits_to_grid(const uint64_t *__restrict__ bits, int n,
                               uint32_t *__restrict__ grid, uint32_t empty, bool swap) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y;
  if (x >= n) return;
  uint64_t w = bits[(size_t)b * n + x];
  uint32_t *p = grid + (size_t)(b * kBand) * n + x;
#pragma unroll 8
  for (int i = 0; i < kBand; ++i)
    p[(size_t)i * n] = !((w >> i) & 1ull) ? empty
                       : swap                ? pack_xy(b * kBand + i, x)
                                             : pack_xy(x, b * kBand + i);
}

cudaError_t launch_grid_to_bits(const uint32_t *grid, int n, uint64_t *bits, int *err,
                                int *count, cudaStream_t s) {
  dim3 blk(128), grd((n + 127) / 128, n / kBand);
  k_grid_to_bits<<<grd, blk, 0, s>>>(grid, n, bits, err, count);
  return cudaGetLastError();
}

cudaError_t launch_bits_to_grid(const uint64_t *bits, int n, uint32_t *grid, cudaStream_t s,
                                uint32_t empty, bool swap) {
  dim3 blk(128), grd((n + 127) / 128, n / kBand);
  k_bits_to_grid<<<grd, blk, 0, s>>>(bits, n, grid, empty, swap);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Column summaries: prev[b][x] = last site row in bands < b, next[b][x] =
// first site row in bands > b (kNoneAbove / kNoneBelow when there is none).
// One block per 32-column group: 32 columns x 32 band groups, each thread
// owning ceil(nb/32) consecutive bands.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_summary(LevelBufs a, int respect_stop) {
  if (respect_stop && a.st->stopped) return;
  __shared__ int sLast[32][33];
  __shared__ int sFirst[32][33];
  const int n = a.n, nb = n / kBand;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = blockIdx.x * 32 + tx;
  const uint64_t *bits = cur_bits(a);
  const int G = (nb + 31) / 32;
  const int b0 = min(nb, ty * G), b1 = min(nb, b0 + G);
  int myLast = kNoneAbove, myFirst = kNoneBelow;
  for (int b = b0; b < b1; ++b) {
    uint64_t w = bits[(size_t)b * n + x];
    if (w) {
      if (myFirst == kNoneBelow) myFirst = b * kBand + __ffsll((long long)w) - 1;
      myLast = b * kBand + 63 - __clzll((long long)w);
    }
  }
  sLast[ty][tx] = myLast;
  sFirst[ty][tx] = myFirst;
  __syncthreads();
  int pv = kNoneAbove;
  for (int k = 0; k < ty; ++k) pv = max(pv, sLast[k][tx]);
  int nx = kNoneBelow;
  for (int k = ty + 1; k < 32; ++k) nx = min(nx, sFirst[k][tx]);
  for (int b = b0; b < b1; ++b) {
    a.prev[(size_t)b * n + x] = (int16_t)pv;
    uint64_t w = bits[(size_t)b * n + x];
    if (w) pv = b * kBand + 63 - __clzll((long long)w);
  }
  for (int b = b1 - 1; b >= b0; --b) {
    a.next[(size_t)b * n + x] = (int16_t)nx;
    uint64_t w = bits[(size_t)b * n + x];
    if (w) nx = b * kBand + __ffsll((long long)w) - 1;
  }
}

cudaError_t launch_summary(const LevelBufs &b, int respect_stop, cudaStream_t s) {
  dim3 blk(32, 32), grd(b.n / 32);
  k_summary<<<grd, blk, 0, s>>>(b, respect_stop);
  return cudaGetLastError();
}

// Fixed-site bitmap of a level from the mask.  The reference indexes the full-
// resolution mask with the level's own pitch (gcvt.cu:777); so does this.
__global__ void k_fixed_bits(const uint8_t *__restrict__ mask, int n, uint64_t *fb) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y;
  if (x >= n) return;
  uint64_t w = 0;
  for (int i = 0; i < kBand; ++i)
    if (mask[(size_t)(b * kBand + i) * n + x]) w |= 1ull << i;
  fb[(size_t)b * n + x] = w;
}

cudaError_t launch_fixed_bits(const uint8_t *mask, int n, uint64_t *fixed_bits, cudaStream_t s) {
  dim3 blk(128), grd((n + 127) / 128, n / kBand);
  k_fixed_bits<<<grd, blk, 0, s>>>(mask, n, fixed_bits);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Row pass
// ---------------------------------------------------------------------------

// Hull entry packed as (x << 16) | (uint16_t)g, g = candidate row - r.
__device__ __forceinline__ int ent_x(int e) { return (int)((unsigned)e >> 16); }
__device__ __forceinline__ int ent_g(int e) { return (int)(int16_t)(e & 0xffff); }
__device__ __forceinline__ int ent_B(int e) {
  int x = ent_x(e), g = ent_g(e);
  return x * x + g * g;
}
__device__ __forceinline__ int pack_ent(int x, int g) { return (x << 16) | (g & 0xffff); }
constexpr int kNoEnt = -1;  // x = 0xffff never occurs (n <= 8192)

// 1 when b lies strictly below the segment a-c on the points (x, B), i.e. b
// survives a chord test.  Exact in 64-bit integers.
__device__ __forceinline__ bool below_chord(int a, int b, int c) {
  const int ax = ent_x(a), bx = ent_x(b), cx = ent_x(c);
  const int aB = ent_B(a), bB = ent_B(b), cB = ent_B(c);
  return (long long)(bx - ax) * (long long)(cB - aB) - (long long)(bB - aB) * (long long)(cx - ax) > 0;
}

// First pixel owned by entry e2 when e1 precedes it on the envelope:
// floor((B2 - B1) / (2 (x2 - x1))) + 1; an integer tie stays with e1 (the
// smaller column), as kernelColor's '>' break does (gcvt.cu:457).
__device__ __forceinline__ int start_pixel(int e1, int e2) {
  const int num = ent_B(e2) - ent_B(e1);
  const int den = 2 * (ent_x(e2) - ent_x(e1));
  int q = (int)floorf(__fdividef((float)num, (float)den));
  // exact fix-up: q = floor(num / den)
  while (q * den > num) --q;
  while ((q + 1) * den <= num) ++q;
  return q + 1;
}

// Column candidate: the vertically nearest site row of one column for row r,
// PBA+ band tie rule included.  kNoneAbove when the column has no site.
__device__ __forceinline__ int column_candidate(uint64_t w, int pv, int nx, uint64_t le,
                                                int base, int r) {
  uint64_t ab = w & le, be = w & ~le;
  int a = ab ? base + 63 - __clzll((long long)ab) : pv;
  int b = be ? base + __ffsll((long long)be) - 1 : nx;
  if (a == kNoneAbove) return b == kNoneBelow ? kNoneAbove : b;
  if (b == kNoneBelow) return a;
  int da = r - a, db = b - r;
  return da < db ? a : (db < da ? b : (be ? b : a));
}

// Lower envelope of the row's column candidates, left in C[0, K).
// Candidates are generated 32 columns at a time (lane = column, coalesced
// loads, the next chunk's loads in flight) and each chunk first drops, by
// three rounds of chord removal among its own points, points strictly above
// the chord of their neighbours there -- no such point is on the lower hull
// of any superset.  The survivors are appended to C; further rounds over C
// remove, all at once, every point strictly above the chord of its current
// neighbours, until a round removes nothing -- the surviving chain is then
// convex, i.e. the lower hull.  After kMaxRounds the remaining points go
// through one sequential monotone-chain pass, so any input ends exactly.
// cap: the entries C holds; -1 when the survivors do not fit.
constexpr int kMaxRounds = 24;
constexpr int kChunkRounds = 3;  // chord rounds within a chunk (28-31 % of a row survive three)

__device__ int row_hull(const LevelBufs &a, int r, int *C, int cap) {
  const int n = a.n;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int band = r >> 6, bi = r & 63;
  const uint64_t le = (bi == 63) ? ~0ull : ((2ull << bi) - 1ull);
  const int base = band * kBand;
  const uint64_t *wrow = cur_bits(a) + (size_t)band * n;
  const int16_t *prow = a.prev + (size_t)band * n;
  const int16_t *nrow = a.next + (size_t)band * n;

  auto cand = [&](int c) -> int {  // packed candidate of column 32c+lane or kNoEnt
    const int x = c * 32 + lane;
    const int cr = column_candidate(__ldg(wrow + x), __ldg(prow + x), __ldg(nrow + x), le, base, r);
    return cr == kNoneAbove ? kNoEnt : pack_ent(x, cr - r);
  };

  // ---- phase 1: candidates, chunk-local chord rounds ------------------------
  const int nchunks = n >> 5;
  int K = 0;
  int cur = cand(0);
  for (int c = 0; c < nchunks; ++c) {
    const int nxt = (c + 1 < nchunks) ? cand(c + 1) : kNoEnt;
    unsigned vm = __ballot_sync(0xffffffffu, cur != kNoEnt);
    for (int it = 0; it < kChunkRounds; ++it) {
      const unsigned lower = vm & lt, upper = vm & ~lt & ~(1u << lane);
      const int left = __shfl_sync(0xffffffffu, cur, lower ? 31 - __clz(lower) : lane);
      const int right = __shfl_sync(0xffffffffu, cur, upper ? __ffs(upper) - 1 : lane);
      const bool keep = cur != kNoEnt && (!lower || !upper || below_chord(left, cur, right));
      const unsigned km = __ballot_sync(0xffffffffu, keep);
      if (km == vm) break;
      vm = km;
      if (!keep) cur = kNoEnt;
    }
    if (K + __popc(vm) > cap) return -1;
    if (cur != kNoEnt) C[K + __popc(vm & lt)] = cur;
    K += __popc(vm);
    cur = nxt;
  }
  __syncwarp();

  // ---- further rounds of simultaneous chord removal ------------------------
  int round = 0;
  for (; round < kMaxRounds; ++round) {
    int w = 0;
    int prevv = kNoEnt;  // last (original) value of the previous chunk
    bool changed = false;
    for (int c = 0; c < K; c += 32) {
      const int idx = c + lane;
      const int v = idx < K ? C[idx] : kNoEnt;
      const int look = (lane == 31 && c + 32 < K) ? C[c + 32] : kNoEnt;
      __syncwarp();
      int left = __shfl_up_sync(0xffffffffu, v, 1);
      if (lane == 0) left = prevv;
      int right = __shfl_down_sync(0xffffffffu, v, 1);
      if (lane == 31) right = look;
      if (idx + 1 >= K) right = kNoEnt;
      const bool keep = v != kNoEnt && (left == kNoEnt || right == kNoEnt || below_chord(left, v, right));
      const unsigned km = __ballot_sync(0xffffffffu, keep);
      const unsigned vm = __ballot_sync(0xffffffffu, v != kNoEnt);
      changed |= (km != vm);
      if (keep) C[w + __popc(km & lt)] = v;
      w += __popc(km);
      prevv = __shfl_sync(0xffffffffu, v, 31);
      __syncwarp();
    }
    K = w;
    if (!changed) break;
  }
  if (round == kMaxRounds) {  // not converged: one exact sequential pass
    int sp = 0;
    if (lane == 0) {
      for (int i = 0; i < K; ++i) {
        const int P = C[i];
        while (sp >= 2 && !below_chord(C[sp - 2], C[sp - 1], P)) --sp;
        C[sp++] = P;
      }
    }
    K = __shfl_sync(0xffffffffu, sp, 0);
    __syncwarp();
  }
  return K;
}

// The row's label words from its hull C[0, K).
__device__ void write_row(uint32_t *out, int n, int r, const int *C, int K) {
  const int lane = threadIdx.x & 31;
  if (K == 0) {  // no site anywhere
    for (int p = lane; p < n; p += 32) out[p] = kMarkerWord;
    return;
  }
  for (int k0 = 0; k0 < K; k0 += 32) {
    const int k = k0 + lane;
    int s0 = 0, s1 = 0;
    uint32_t lab = 0;
    if (k < K) {
      const int e = C[k];
      s0 = k == 0 ? 0 : max(0, start_pixel(C[k - 1], e));
      s1 = k + 1 == K ? n : min(n, start_pixel(e, C[k + 1]));
      lab = pack_xy(ent_x(e), ent_g(e) + r);
      if (s1 - s0 <= 16)
        for (int p = s0; p < s1; ++p) out[p] = lab;
    }
    // long ranges: written by the whole warp, coalesced
    unsigned lm = __ballot_sync(0xffffffffu, s1 - s0 > 16);
    while (lm) {
      const int L = __ffs(lm) - 1;
      lm &= lm - 1;
      const int b0 = __shfl_sync(0xffffffffu, s0, L), b1 = __shfl_sync(0xffffffffu, s1, L);
      const uint32_t lv = __shfl_sync(0xffffffffu, lab, L);
      for (int p = b0 + lane; p < b1; p += 32) out[p] = lv;
    }
  }
}

// Label pass: one warp per row writes the row's label words.  A row's hull
// buffer holds 2/5 of a row (the survivors of the chunk-local rounds of a
// typical row fit): 2.5 times the rows per SM of a whole-row buffer.  A row whose survivors do
// not fit (a row crowded with sites, where most columns' candidates stay on
// the hull) is flagged in DevState::row_ovf and done by k_rows_full with a
// whole-row buffer.
constexpr int row_cap(int n) { return n * 2 / 5; }

__global__ void __launch_bounds__(32) k_rows(LevelBufs a, int respect_stop) {
  extern __shared__ __align__(16) int smem[];
  if (respect_stop && a.st->stopped) return;
  const int n = a.n, r = blockIdx.x;
  if (r >= n) return;
  const int K = row_hull(a, r, smem, row_cap(n));
  if (K < 0) {
    if ((threadIdx.x & 31) == 0) atomicOr(&a.st->row_ovf[r >> 5], 1u << (r & 31));
    return;
  }
  write_row(a.labels + (size_t)r * n, n, r, smem, K);
}

// The flagged rows, with a whole-row buffer (a grid of a few blocks per SM
// striding over the rows); clears their flags.
__global__ void __launch_bounds__(32) k_rows_full(LevelBufs a, int respect_stop) {
  extern __shared__ __align__(16) int smem[];
  if (respect_stop && a.st->stopped) return;
  const int n = a.n;
  for (int r = blockIdx.x; r < n; r += gridDim.x) {
    if (!((a.st->row_ovf[r >> 5] >> (r & 31)) & 1u)) continue;
    const int K = row_hull(a, r, smem, n);
    write_row(a.labels + (size_t)r * n, n, r, smem, K);
    __syncwarp();
    if ((threadIdx.x & 31) == 0) atomicAnd(&a.st->row_ovf[r >> 5], ~(1u << (r & 31)));
  }
}

size_t rows_smem_bytes(int n) { return (size_t)n * sizeof(int); }

cudaError_t rows_configure() {
  return cudaFuncSetAttribute(k_rows_full, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)rows_smem_bytes(kMaxN));
}

cudaError_t launch_rows(const LevelBufs &b, int respect_stop, cudaStream_t s) {
  k_rows<<<b.n, 32, rows_smem_bytes(row_cap(b.n)), s>>>(b, respect_stop);
  k_rows_full<<<b.n < 304 ? b.n : 304, 32, rows_smem_bytes(b.n), s>>>(b, respect_stop);
  return cudaGetLastError();
}

// Row support of a density grid: [first, last + 1) of its nonzero pixels per
// row (an empty row gets [0, 0)), the range of rows holding any (range must
// start at (n, 0)), and the number of support pixels.  One warp per row.
__global__ void k_row_support(const float *__restrict__ d, int n, int2 *sup, int2 *range,
                              unsigned long long *pixels) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  int lo = n, hi = -1;
  for (int p = lane; p < n; p += 32) {
    if (d[(size_t)r * n + p] != 0.0f) {
      lo = min(lo, p);
      hi = max(hi, p);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    sup[r] = hi < 0 ? make_int2(0, 0) : make_int2(lo, hi + 1);
    if (hi >= 0) {
      atomicMin(&range->x, r);
      atomicMax(&range->y, r + 1);
      atomicAdd(pixels, (unsigned long long)(hi + 1 - lo));
    }
  }
}

cudaError_t launch_row_support(const float *density, int n, int2 *sup, int2 *range,
                               unsigned long long *pixels, cudaStream_t s) {
  const int2 init = make_int2(n, 0);
  cudaError_t e = cudaMemcpyAsync(range, &init, sizeof(int2), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(pixels, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  k_row_support<<<(n + 7) / 8, 256, 0, s>>>(density, n, sup, range, pixels);
  return cudaGetLastError();
}

}  // namespace cvtgb
