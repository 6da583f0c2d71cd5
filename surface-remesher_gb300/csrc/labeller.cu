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
// GB300 layout (two kernels instead of ~20 launches and ~60 B/px):
//   * sites live in a bitmap of 64-row words, bits[band][column] -- one
//     64-bit word per column and PBA band, so the band tie rule is "the lower
//     site came from the same word";
//   * k_summary: per (band, column), the nearest site row above / below the
//     band (a scan over bands, 32 columns x 32 band groups per block);
//   * k_rows: one warp per row.  Lane j owns columns [j*S, (j+1)*S),
//     S = n/32: it derives each column's candidate from the bitmap word and
//     summaries (no column-nearest grid is ever written), pushes candidates
//     (x, B = x^2 + g^2) onto a lower-hull stack in shared memory, five
//     levels of bridge merges join the 32 hulls, and every lane walks the
//     joint envelope across its own pixels with division-free breakpoint
//     tests.  In label mode it writes label words; in Lloyd mode it fuses the
//     per-site moment and energy accumulation (density read once, 4 B/px).
#include "gcvt_internal.cuh"

namespace cvtgb {

// ---------------------------------------------------------------------------
// Site grid <-> bitmap
// ---------------------------------------------------------------------------

// One thread per (band, column): 64 coalesced row reads, one word written.
// A pixel is a site when its x half is not MARKER (gcvt.cu:90); a site pixel
// must hold its own coordinates, else err gets bit 0.
__global__ void k_grid_to_bits(const uint32_t *__restrict__ grid, int n,
                               uint64_t *__restrict__ bits, int *err) {
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
}

__global__ void k_bits_to_grid(const uint64_t *__restrict__ bits, int n,
                               uint32_t *__restrict__ grid) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y;
  if (x >= n) return;
  uint64_t w = bits[(size_t)b * n + x];
  uint32_t *p = grid + (size_t)(b * kBand) * n + x;
#pragma unroll 8
  for (int i = 0; i < kBand; ++i)
    p[(size_t)i * n] = ((w >> i) & 1ull) ? pack_xy(x, b * kBand + i) : kMarkerWord;
}

cudaError_t launch_grid_to_bits(const uint32_t *grid, int n, uint64_t *bits, int *err,
                                cudaStream_t s) {
  dim3 blk(128), grd((n + 127) / 128, n / kBand);
  k_grid_to_bits<<<grd, blk, 0, s>>>(grid, n, bits, err);
  return cudaGetLastError();
}

cudaError_t launch_bits_to_grid(const uint64_t *bits, int n, uint32_t *grid, cudaStream_t s) {
  dim3 blk(128), grd((n + 127) / 128, n / kBand);
  k_bits_to_grid<<<grd, blk, 0, s>>>(bits, n, grid);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Column summaries: prev[b][x] = last site row in bands < b, next[b][x] =
// first site row in bands > b (kNoneAbove / kNoneBelow when there is none).
// Block = 32 columns x 32 band groups; each thread owns ceil(nb/32) bands.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_summary(LevelBufs a, int respect_stop) {
  if (respect_stop && a.st->stopped) return;
  __shared__ int sLast[32][33];
  __shared__ int sFirst[32][33];
  const int n = a.n, nb = n / kBand;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = blockIdx.x * 32 + tx;
  const uint64_t *bits = (a.st->parity ? a.bits[1] : a.bits[0]);
  const int G = (nb + 31) / 32;
  const int b0 = ty * G, b1 = min(nb, b0 + G);
  int myLast = kNoneAbove, myFirst = kNoneBelow;
  if (x < n) {
    for (int b = b0; b < b1; ++b) {
      uint64_t w = bits[(size_t)b * n + x];
      if (w) {
        if (myFirst == kNoneBelow) myFirst = b * kBand + __ffsll((long long)w) - 1;
        myLast = b * kBand + 63 - __clzll((long long)w);
      }
    }
  }
  sLast[ty][tx] = myLast;
  sFirst[ty][tx] = myFirst;
  __syncthreads();
  if (x >= n || b0 >= nb) return;
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
  dim3 blk(32, 32), grd((b.n + 31) / 32);
  k_summary<<<grd, blk, 0, s>>>(b, respect_stop);
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

// 1 if pixel p lies at or after the first pixel that entry e2 (successor of
// e1 on the envelope) owns: e2 starts at floor((B2-B1) / (2(x2-x1))) + 1,
// ties at an integer breakpoint staying with the smaller column.
__device__ __forceinline__ bool past_start(int e1, int e2, int p) {
  int num = ent_B(e2) - ent_B(e1);
  int den = 2 * (ent_x(e2) - ent_x(e1));
  return num < p * den;
}

// Orientation of (o, a, b) on points (x, B); > 0 when a lies strictly below
// the segment o-b, i.e. a stays on the lower hull.
__device__ __forceinline__ long long hull_cross(int ox, int oB, int ax, int aB, int bx, int bB) {
  return (long long)(ax - ox) * (long long)(bB - oB) - (long long)(aB - oB) * (long long)(bx - ox);
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

struct RowSmem {
  int *base;  // 32 lanes x SP stack slots, then lo[32], hi[32]
  int SP;
  __device__ __forceinline__ int *stk(int lane) const { return base + lane * SP; }
  __device__ __forceinline__ int *lo() const { return base + 32 * SP; }
  __device__ __forceinline__ int *hi() const { return base + 32 * SP + 32; }
  __device__ __forceinline__ int at(int lane, int k) const { return base[lane * SP + k]; }
};

// Join the hulls of lanes [L0, M) and [M, L1) along their lower bridge.  Run
// by one lane; every loop advances a finger monotonically, so it ends.
__device__ void bridge_merge(const RowSmem &sm, int L0, int M, int L1) {
  int *lo = sm.lo(), *hi = sm.hi();
  int iL = -1, kL = -1;
  for (int j = M - 1; j >= L0; --j)
    if (hi[j] > lo[j]) { iL = j; break; }
  for (int j = M; j < L1; ++j)
    if (hi[j] > lo[j]) { kL = j; break; }
  if (iL < 0 || kL < 0) return;
  int ik = hi[iL] - 1, kk = lo[kL];
  int I = sm.at(iL, ik), K = sm.at(kL, kk);
  bool changed = true;
  while (changed) {
    changed = false;
    for (;;) {  // drop left-hull points on or above the line pred(i) -> k
      int pL = iL, pk = ik - 1;
      if (pk < lo[pL]) {
        pL = -1;
        for (int j = iL - 1; j >= L0; --j)
          if (hi[j] > lo[j]) { pL = j; pk = hi[j] - 1; break; }
        if (pL < 0) break;
      }
      int P = sm.at(pL, pk);
      if (hull_cross(ent_x(P), ent_B(P), ent_x(I), ent_B(I), ent_x(K), ent_B(K)) <= 0) {
        iL = pL; ik = pk; I = P; changed = true;
      } else {
        break;
      }
    }
    for (;;) {  // drop right-hull points on or above the line i -> succ(k)
      int sL = kL, sk = kk + 1;
      if (sk >= hi[sL]) {
        sL = -1;
        for (int j = kL + 1; j < L1; ++j)
          if (hi[j] > lo[j]) { sL = j; sk = lo[j]; break; }
        if (sL < 0) break;
      }
      int Q = sm.at(sL, sk);
      if (hull_cross(ent_x(I), ent_B(I), ent_x(K), ent_B(K), ent_x(Q), ent_B(Q)) <= 0) {
        kL = sL; kk = sk; K = Q; changed = true;
      } else {
        break;
      }
    }
  }
  hi[iL] = ik + 1;
  for (int j = iL + 1; j < M; ++j) hi[j] = lo[j];
  lo[kL] = kk;
  for (int j = M; j < kL; ++j) lo[j] = hi[j];
}

// Compensated accumulation of v into the per-site (hi, lo) pair: the vector
// atomic returns the old hi, the rounding error of old + v (round to nearest,
// as the atomic unit computes it) is recovered exactly by TwoSum and added to
// lo.
__device__ __forceinline__ void atomic_add_comp(float4 *hi, float4 *lo, float4 v) {
  float4 o;
  asm volatile("atom.global.add.v4.f32 {%0,%1,%2,%3}, [%4], {%5,%6,%7,%8};"
               : "=f"(o.x), "=f"(o.y), "=f"(o.z), "=f"(o.w)
               : "l"(hi), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
  float4 e;
#define TWO_SUM_ERR(A, B, E)                 \
  {                                          \
    float s_ = __fadd_rn(A, B);              \
    float bp_ = __fsub_rn(s_, A);            \
    float ap_ = __fsub_rn(s_, bp_);          \
    E = __fadd_rn(__fsub_rn(A, ap_), __fsub_rn(B, bp_)); \
  }
  TWO_SUM_ERR(o.x, v.x, e.x);
  TWO_SUM_ERR(o.y, v.y, e.y);
  TWO_SUM_ERR(o.z, v.z, e.z);
  TWO_SUM_ERR(o.w, v.w, e.w);
#undef TWO_SUM_ERR
  if (e.x != 0.f || e.y != 0.f || e.z != 0.f || e.w != 0.f)
    asm volatile("red.global.add.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(lo), "f"(e.x), "f"(e.y),
                 "f"(e.z), "f"(e.w)
                 : "memory");
}

template <int MODE>  // 0: write labels; 1: accumulate Lloyd moments
__global__ void __launch_bounds__(kRowsPerBlock * 32) k_rows(LevelBufs a, int respect_stop) {
  extern __shared__ __align__(16) int smem[];
  if (respect_stop && a.st->stopped) return;
  const int n = a.n;
  const int S = n >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kRowsPerBlock + warp;
  if (r >= n) return;
  RowSmem sm;
  sm.SP = S + 1;
  sm.base = smem + warp * (32 * sm.SP + 64);
  int *stk = sm.stk(lane);

  // ---- local lower hull of this lane's columns ----------------------------
  const int band = r >> 6, bi = r & 63;
  const uint64_t le = (bi == 63) ? ~0ull : ((2ull << bi) - 1ull);
  const int base = band * kBand;
  const int xbeg = lane * S;
  const uint64_t *wrow = (a.st->parity ? a.bits[1] : a.bits[0]) + (size_t)band * n + xbeg;
  const int16_t *prow = a.prev + (size_t)band * n + xbeg;
  const int16_t *nrow = a.next + (size_t)band * n + xbeg;
  int sp = 0;
  int t0x = 0, t0B = 0, t1x = 0, t1B = 0;  // second and top of the stack
  for (int k0 = 0; k0 < S; k0 += 8) {
    ulonglong2 w01 = *reinterpret_cast<const ulonglong2 *>(wrow + k0);
    ulonglong2 w23 = *reinterpret_cast<const ulonglong2 *>(wrow + k0 + 2);
    ulonglong2 w45 = *reinterpret_cast<const ulonglong2 *>(wrow + k0 + 4);
    ulonglong2 w67 = *reinterpret_cast<const ulonglong2 *>(wrow + k0 + 6);
    uint4 pv4 = *reinterpret_cast<const uint4 *>(prow + k0);
    uint4 nx4 = *reinterpret_cast<const uint4 *>(nrow + k0);
    uint64_t ws[8] = {w01.x, w01.y, w23.x, w23.y, w45.x, w45.y, w67.x, w67.y};
    unsigned pvs[4] = {pv4.x, pv4.y, pv4.z, pv4.w};
    unsigned nxs[4] = {nx4.x, nx4.y, nx4.z, nx4.w};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      int pv = (int)(int16_t)((pvs[q >> 1] >> ((q & 1) * 16)) & 0xffffu);
      int nx = (int)(int16_t)((nxs[q >> 1] >> ((q & 1) * 16)) & 0xffffu);
      int c = column_candidate(ws[q], pv, nx, le, base, r);
      if (c == kNoneAbove) continue;
      const int x = xbeg + k0 + q;
      const int g = c - r;
      const int B = x * x + g * g;
      while (sp >= 2) {
        if (hull_cross(t0x, t0B, t1x, t1B, x, B) > 0) break;
        --sp;
        t1x = t0x; t1B = t0B;
        if (sp >= 2) {
          int e = stk[sp - 2];
          t0x = ent_x(e); t0B = ent_B(e);
        }
      }
      stk[sp++] = (x << 16) | (g & 0xffff);
      t0x = t1x; t0B = t1B; t1x = x; t1B = B;
    }
  }
  sm.lo()[lane] = 0;
  sm.hi()[lane] = sp;
  __syncwarp();

  // ---- five levels of bridge merges ----------------------------------------
#pragma unroll 1
  for (int G = 1; G < 32; G <<= 1) {
    if ((lane & (2 * G - 1)) == 0) bridge_merge(sm, lane, lane + G, lane + 2 * G);
    __syncwarp();
  }

  // ---- locate the envelope entry covering this lane's first pixel ---------
  const int mylo = sm.lo()[lane], myhi = sm.hi()[lane];
  const unsigned ne = __ballot_sync(0xffffffffu, myhi > mylo);
  const int X0 = xbeg;
  uint32_t *lab_out = (MODE == 0) ? a.labels + (size_t)r * n + X0 : nullptr;
  if (ne == 0) {  // no site anywhere
    if (MODE == 0)
      for (int p = 0; p < S; p += 4)
        *reinterpret_cast<uint4 *>(lab_out + p) =
            make_uint4(kMarkerWord, kMarkerWord, kMarkerWord, kMarkerWord);
    return;
  }
  int fe = 0, pe = 0;
  bool has_pred = false;
  if (myhi > mylo) {
    fe = stk[mylo];
    unsigned lower = ne & ((1u << lane) - 1u);
    if (lower) {
      int pl = 31 - __clz(lower);
      pe = sm.at(pl, sm.hi()[pl] - 1);
      has_pred = true;
    }
  }
  int ansL = 0;
#pragma unroll 4
  for (int q = 0; q < 32; ++q) {
    bool ok = (myhi > mylo) && (!has_pred || past_start(pe, fe, q * S));
    unsigned m = __ballot_sync(0xffffffffu, ok);
    if (lane == q) ansL = 31 - __clz(m);
  }
  int cL = ansL, ck;
  {
    int k0 = sm.lo()[ansL], k1 = sm.hi()[ansL] - 1;
    while (k0 < k1) {
      int mid = (k0 + k1 + 1) >> 1;
      if (past_start(sm.at(ansL, mid - 1), sm.at(ansL, mid), X0)) k0 = mid;
      else k1 = mid - 1;
    }
    ck = k0;
  }
  int cur = sm.at(cL, ck);
  // successor on the envelope
  int sL = cL, sk = ck + 1, suc = 0;
  bool has_suc = true;
  if (sk >= sm.hi()[sL]) {
    unsigned above = (cL == 31) ? 0u : (ne & ~((2u << cL) - 1u));
    if (above) { sL = __ffs(above) - 1; sk = sm.lo()[sL]; }
    else has_suc = false;
  }
  if (has_suc) suc = sm.at(sL, sk);

  // ---- walk the envelope over pixels [X0, X0 + S) --------------------------
  const int ry = r;
  if (MODE == 0) {
    for (int p0 = 0; p0 < S; p0 += 4) {
      uint32_t out[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int p = X0 + p0 + q;
        while (has_suc && past_start(cur, suc, p)) {
          cur = suc; cL = sL; ck = sk;
          sk = ck + 1;
          if (sk >= sm.hi()[sL]) {
            unsigned above = (cL == 31) ? 0u : (ne & ~((2u << cL) - 1u));
            if (above) { sL = __ffs(above) - 1; sk = sm.lo()[sL]; }
            else has_suc = false;
          }
          if (has_suc) suc = sm.at(sL, sk);
        }
        out[q] = pack_xy(ent_x(cur), ent_g(cur) + ry);
      }
      *reinterpret_cast<uint4 *>(lab_out + p0) = make_uint4(out[0], out[1], out[2], out[3]);
    }
  } else {
    const float *drow = a.density + (size_t)r * n + X0;
    float W = 0.f, SX = 0.f, Q = 0.f;
    auto flush = [&](int e) {
      if (W != 0.f) {
        const int ex = ent_x(e), eg = ent_g(e);
        const float fg = (float)eg;
        float4 v = make_float4(W, SX, __fmul_rn(-fg, W), __fmaf_rn((float)(eg * eg), W, Q));
        size_t pid = (size_t)(eg + ry) * n + ex;
        atomic_add_comp(a.mhi + pid, a.mlo + pid, v);
      }
      W = 0.f; SX = 0.f; Q = 0.f;
    };
    for (int p0 = 0; p0 < S; p0 += 4) {
      float4 d4 = __ldg(reinterpret_cast<const float4 *>(drow + p0));
      float ds[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int p = X0 + p0 + q;
        while (has_suc && past_start(cur, suc, p)) {
          flush(cur);
          cur = suc; cL = sL; ck = sk;
          sk = ck + 1;
          if (sk >= sm.hi()[sL]) {
            unsigned above = (cL == 31) ? 0u : (ne & ~((2u << cL) - 1u));
            if (above) { sL = __ffs(above) - 1; sk = sm.lo()[sL]; }
            else has_suc = false;
          }
          if (has_suc) suc = sm.at(sL, sk);
        }
        const float rho = ds[q];
        const float dx = (float)(p - ent_x(cur));
        W = __fadd_rn(W, rho);
        SX = __fmaf_rn(dx, rho, SX);
        Q = __fmaf_rn(__fmul_rn(dx, dx), rho, Q);
      }
    }
    flush(cur);
  }
}

size_t rows_smem_bytes(int n) {
  int S = n >> 5;
  return (size_t)kRowsPerBlock * (32 * (S + 1) + 64) * sizeof(int);
}

cudaError_t rows_configure() {
  cudaError_t e = cudaFuncSetAttribute(k_rows<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)rows_smem_bytes(kMaxN));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_rows<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)rows_smem_bytes(kMaxN));
}

cudaError_t launch_rows(const LevelBufs &b, int label_mode, int respect_stop, cudaStream_t s) {
  size_t smem = rows_smem_bytes(b.n);
  dim3 blk(kRowsPerBlock * 32), grd((b.n + kRowsPerBlock - 1) / kRowsPerBlock);
  if (label_mode) k_rows<0><<<grd, blk, smem, s>>>(b, respect_stop);
  else k_rows<1><<<grd, blk, smem, s>>>(b, respect_stop);
  return cudaGetLastError();
}

}  // namespace cvtgb
