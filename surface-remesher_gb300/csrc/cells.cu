// cells.cu -- one Lloyd iteration as two launches: k_list lays the current
// sites out in bitmap order, then k_cell lets every site compute its own
// Voronoi cell exactly, sum the density moments over it, and move.
//
// In a Lloyd iteration the labels themselves are never needed, only each
// site's sums over its cell (gcvt.cu:1008-1023) and the energy
// (gcvt.cu:1059-1083).  The PBA+ labelling (labeller.cu) is a total order per
// pixel -- nearest site, then smaller x, then the 64-row band rule for a mirror
// pair -- so "pixel p belongs to site s" is "s beats every other site t at p".
// In coordinates relative to s (p = s + (u, v), t = s + (A, B)):
//     |p - s|^2 - |p - t|^2 = 2Au + 2Bv - (A^2 + B^2)
//     A > 0 (t right of s, s wins ties):   u <= floor(N / 2A)
//     A < 0 (t left of s, t wins ties):    u >= floor(N / 2A) + 1
//     A = 0 (same column): row v is s's iff B (2v - B) < 0, or = 0 and the
//                          band rule picks s,
// with N = A^2 + B^2 - 2Bv, exact in 32-bit integers.  The cell is the
// intersection, one interval per row.
//
// Candidates t come from the site bitmap in the disc of radius W around s.
// Certificate: if every summed pixel lies within R of s and 2R <= W, no site
// outside the disc can beat s there (|p - t| > W - R >= R); otherwise the
// window grows (W <- min(2R + 1, 2W)) and the cell is redone; a window
// covering the grid is exact by construction.  The starting W of a site is
// the hint at its pixel: 2R + slack of the cell the site that moved there
// had, or, after a load, of its own cell in the level start's label grid
// (k_cover).
//
// Rows are visited outward from s.  A row may hold no pixel of the cell while
// a row further out does (a sliver narrower than a pixel), so the walk ends
// only when lo > hi + 1: then the largest lower cut is at least lo - 1 >= hi + 1,
// above the smallest upper cut (< hi + 1), so the real chord of the convex
// cell is empty, and so is every chord further from s.
//
// Covering bound.  A cell at the domain boundary is open towards the empty
// region, so its row walk alone would cross the whole grid.  Every density
// pixel p lies within `cover` of its owner (DevState::cover), so only pixels
// with |p - s| <= cover can be s's: the walk stays in that disc and the
// window never needs to exceed 2 cover.  The bound carries itself from one
// iteration to the next: if the pixel p was within R of its owner s and s
// moved by d, p is within R + d of the site now at s's new pixel (a merged
// site leaves another at that pixel), so cover' = ceil(sqrt(max R^2)) +
// ceil(sqrt(max d^2)), both maxima taken over this iteration's cells.  The
// first iteration of a level takes it from a label grid (k_cover).
//
// Work split.  k_cell runs one warp per block, as many blocks as fit on the
// GPU; each warp takes the next group of 32 listed sites from a ticket, one
// site per lane.  A lane keeps its site's candidates as 8-byte records and
// bounds two rows per pass over them.  The energy is reduced in a fixed order
// whatever warp takes which group: the sites of a group by a butterfly, 64
// groups by the warp finishing the last of them, the 64-group totals by the
// warp finishing the last 64-group; that warp also runs the schedule.  Sites move by atomicOr into the next bitmap;
// the first to set a bit also counts it for the next k_list.
#include "gcvt_internal.cuh"

namespace cvtgb {

constexpr int kMaxCand = 64;  // candidate records per site; more: streamed
constexpr int kGroupsPerSlot = 64;

__device__ __forceinline__ void tsum_c(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bp = __fsub_rn(s, a);
  float ap = __fsub_rn(s, bp);
  e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// (ah, al) += (bh, bl), two-float.  Commutative: the error term of TwoSum is
// exact, so both lanes of a butterfly get the same result.
__device__ __forceinline__ void dfa(float &ah, float &al, float bh, float bl) {
  float s, e;
  tsum_c(ah, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(al, bl));
  ah = __fadd_rn(s, e);
  al = __fsub_rn(e, __fsub_rn(ah, s));
}

// (ah, al) += k * (bh, bl) for a small integer k (exact product via fma).
__device__ __forceinline__ void dfa_scaled(float &ah, float &al, float k, float bh, float bl) {
  const float ph = __fmul_rn(k, bh);
  const float pl = __fmaf_rn(k, bh, -ph) + k * bl;
  dfa(ah, al, ph, pl);
}

// floor(sqrt(v)) and ceil(sqrt(v)) for 0 <= v < 2^30, exact.
__device__ __forceinline__ int isqrt_floor(int v) {
  int h = (int)sqrtf((float)v);
  while (h * h > v) --h;
  while ((h + 1) * (h + 1) <= v) ++h;
  return h;
}
__device__ __forceinline__ int isqrt_ceil(int v) {
  const int h = isqrt_floor(v);
  return h * h == v ? h : h + 1;
}

// floor(N / D) for D > 0, exact: from a float estimate when |N| < 2^24 (then
// the estimate is within 1 of it), else by integer division.
__device__ __forceinline__ int floordiv_est(int N, int D, float inv, bool fast) {
  if (fast) {
    int q = __float2int_rd(__fmul_rn((float)N, inv));
    const int r = N - q * D;
    q += (r >= D) - (r < 0);
    return q;
  }
  int q = N / D;
  if ((N % D != 0) && (N < 0)) --q;
  return q;
}

// Row-v bounds from the site t = s + (A, B), A != 0, when the candidates do
// not fit the record list (same-column sites are already row limits).
__device__ __forceinline__ void constrain_rel(int A, int B, int v, int &lo, int &hi) {
  if (A == 0) return;
  const int N = A * A + B * B - 2 * B * v;
  if (A > 0) hi = min(hi, floordiv_est(N, 2 * A, 0.f, false));
  else lo = max(lo, floordiv_est(-N, -2 * A, 0.f, false) + 1);
}

__device__ __forceinline__ uint64_t row_mask(int lo_i, int hi_i) {  // bits lo_i..hi_i
  const uint64_t up = hi_i >= 63 ? ~0ull : ((2ull << hi_i) - 1ull);
  return up & ~((1ull << lo_i) - 1ull);
}

struct CellSums {
  float wh, wl, xh, xl, yh, yl, eh, el;  // W, SX, SY (relative to the site), E
  int r2;                                // max |p - s|^2 over the summed pixels
};

// floor(N / D), D > 0, |N| < 2^23, given r ~ 1/D from rcp.approx (at most 1
// ulp off): the estimate is within 1, one exact correction fixes it.
__device__ __forceinline__ int floordiv_r(int N, int D, float r) {
  int q = __float2int_rd(__fmul_rn((float)N, r));
  const int rem = N - q * D;
  q += (rem >= D) - (rem < 0);
  return q;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Bounds of rows v0 and v0 + dir (relative to s) in one pass over the
// records.  A record {K, S | D << 16} bounds row v by floor((K - S v) / |D|):
// an upper bound when D > 0, a lower one (+1) when D < 0.  When the records
// did not hold every candidate, the candidates are read from the bitmap.
struct RowPair {
  int lo0, hi0, lo1, hi1;
};

__device__ __forceinline__ RowPair row_bounds2(const int2 *rec, int cnt, bool ovf, bool fast,
                                               const uint64_t *__restrict__ bits, int n, int sx,
                                               int sy, int x0, int x1, int b0, int b1, int y0,
                                               int y1, long long Wc, int v0, int dir) {
  RowPair p{-sx, n - 1 - sx, -sx, n - 1 - sx};
  const int v1 = v0 + dir;
  if (!ovf) {
    for (int k = 0; k < cnt; ++k) {
      const int2 r = rec[k];
      const int S = (int)(int16_t)((unsigned)r.y & 0xffffu);
      const int D = (int)(int16_t)((unsigned)r.y >> 16);
      const int aD = abs(D);
      const int N0 = r.x - S * v0, N1 = N0 - S * dir;
      int q0, q1;
      if (fast) {
        const float rr = rcp_approx((float)aD);
        q0 = floordiv_r(N0, aD, rr);
        q1 = floordiv_r(N1, aD, rr);
      } else {
        q0 = floordiv_est(N0, aD, 0.f, false);
        q1 = floordiv_est(N1, aD, 0.f, false);
      }
      if (D > 0) {
        p.hi0 = min(p.hi0, q0);
        p.hi1 = min(p.hi1, q1);
      } else {
        p.lo0 = max(p.lo0, q0 + 1);
        p.lo1 = max(p.lo1, q1 + 1);
      }
    }
    return p;
  }
  for (int x = x0; x <= x1; ++x)
    for (int b = b0; b <= b1; ++b) {
      uint64_t w = __ldg(bits + (size_t)b * n + x) &
                   row_mask(max(y0 - 64 * b, 0), min(y1 - 64 * b, 63));
      while (w) {
        const int i = __ffsll((long long)w) - 1;
        w &= w - 1ull;
        const int A = x - sx, B = 64 * b + i - sy;
        const int K = A * A + B * B;
        if (K == 0 || (long long)K > Wc) continue;
        constrain_rel(A, B, v0, p.lo0, p.hi0);
        constrain_rel(A, B, v1, p.lo1, p.hi1);
      }
    }
  return p;
}

// FP32 sums of one chunk [u0, u1] (at most 16 pixels) of a row: density,
// x-moment and x^2-moment relative to the site.
__device__ __forceinline__ void chunk_sums(const float *__restrict__ row, int u0, int u1,
                                           float &rw, float &rx, float &rq) {
  rw = 0.f, rx = 0.f, rq = 0.f;
  float dx = (float)u0;
#pragma unroll 4
  for (int u = u0; u <= u1; ++u) {
    const float rho = __ldg(row + u);
    const float t = __fmul_rn(dx, rho);
    rw = __fadd_rn(rw, rho);
    rx = __fadd_rn(rx, t);
    rq = __fmaf_rn(t, dx, rq);
    dx = __fadd_rn(dx, 1.0f);
  }
}

// A chunk of row v (fv = v, fv2 = v^2) folded into the two-float cell sums.
__device__ __forceinline__ void fold_chunk(CellSums &c, float rw, float rx, float rq, float fv,
                                           float fv2) {
  dfa(c.wh, c.wl, rw, 0.f);
  dfa(c.xh, c.xl, rx, 0.f);
  dfa_scaled(c.yh, c.yl, fv, rw, 0.f);
  float qh = rq, ql = 0.f;
  dfa_scaled(qh, ql, fv2, rw, 0.f);
  dfa(c.eh, c.el, qh, ql);
}

// Sums of row v = [da, db] (relative columns) into c: FP32 over chunks of at
// most 16 pixels (relative error below 16 ulp of the chunk), chunks folded
// into the two-float cell sums.
__device__ __forceinline__ void row_sums(const float *__restrict__ row, int da, int db, int v,
                                         CellSums &c) {
  const float fv = (float)v, fv2 = (float)(v * v);
  for (int u0 = da; u0 <= db; u0 += 16) {
    float rw, rx, rq;
    chunk_sums(row, u0, min(db, u0 + 15), rw, rx, rq);
    fold_chunk(c, rw, rx, rq, fv, fv2);
  }
}

// The pixels [da, db] of row v the cell with bounds [lo, hi] sums: clipped to
// the density support and the covering disc; false when none.
__device__ __forceinline__ bool row_span(const LevelBufs &a, int sx, int sy, int rb2, int v,
                                         int lo, int hi, int &da, int &db) {
  const int2 s = a.support[sy + v];
  da = max(lo, s.x - sx), db = min(hi, s.y - 1 - sx);
  if (da > db) return false;
  if (max(da * da, db * db) + v * v > rb2) {  // clip to the covering disc
    const int hx = isqrt_floor(rb2 - v * v);
    da = max(da, -hx);
    db = min(db, hx);
    if (da > db) return false;
  }
  return true;
}

// Row v of the cell with bounds [lo, hi]: its span, R2, its sums.
__device__ __forceinline__ void take_row(const LevelBufs &a, int n, int sx, int sy, int rb2, int v,
                                         int lo, int hi, int &R2, CellSums &c) {
  int da, db;
  if (!row_span(a, sx, sy, rb2, v, lo, hi, da, db)) return;
  R2 = max(R2, max(da * da, db * db) + v * v);
  row_sums(a.density + (size_t)(sy + v) * n + sx, da, db, v, c);
}

// A site in s's own column at row offset B != 0: s keeps the rows strictly on
// its side of the mirror row, and the mirror row (B even) if the band rule
// says so.
__device__ __forceinline__ void same_column_limit(int B, int sy, int &vmin, int &vmax) {
  if (B > 0) {
    int m = (B - 1) >> 1;
    if (!(B & 1) && (((sy + B) >> 6) != ((sy + B / 2) >> 6))) m = B / 2;
    vmax = min(vmax, m);
  } else {
    int m = -((-B - 1) >> 1);
    if (!(B & 1) && ((sy >> 6) == ((sy + B / 2) >> 6))) m = B / 2;
    vmin = max(vmin, m);
  }
}

// The record {K, S | D << 16} of candidate t = s + (A, B), A != 0, K = A^2 + B^2
// (|S|, |D| <= 2 (n - 1) fit 16 bits).
__device__ __forceinline__ int2 make_rec(int A, int B, int K) {
  const int S = A > 0 ? 2 * B : -2 * B;
  return make_int2(A > 0 ? K : -K, (int)(((unsigned)S & 0xffffu) | ((unsigned)(2 * A) << 16)));
}

// The sites of one bitmap word (column offset A, bit i at row offset B0 + i)
// as candidates of s: a record each, or a row limit for a site in s's column.
__device__ __forceinline__ void gather_word(uint64_t w, int A, int B0, int sy, long long Wc,
                                            int2 *rec, int &cnt, bool &ovf, int &vmin,
                                            int &vmax) {
  while (w) {
    const int i = __ffsll((long long)w) - 1;
    w &= w - 1ull;
    const int B = B0 + i;
    const int K = A * A + B * B;
    if (K == 0 || (long long)K > Wc) continue;  // s itself; outside the disc
    if (A == 0) {
      same_column_limit(B, sy, vmin, vmax);
      continue;
    }
    if (cnt >= kMaxCand) {
      ovf = true;
      continue;
    }
    rec[cnt++] = make_rec(A, B, K);
  }
}

// Exact cell of site (sx, sy) and its sums.  bits: current site bitmap;
// W: initial window radius; rb: the covering bound.
__device__ CellSums cell_sums(const LevelBufs &a, const uint64_t *__restrict__ bits, int n, int sx,
                              int sy, int W, int rb) {
  int2 rec[kMaxCand];  // {K, S | D << 16} of the window's candidates
  const int2 yr = *a.sup_range;  // rows [yr.x, yr.y) hold every nonzero density
  const int vlo_sup = max(yr.x, sy - rb) - sy, vhi_sup = min(yr.y - 1, sy + rb) - sy;
  const int rb2 = rb * rb;
  W = max(1, min(W, 2 * rb));
  CellSums c;
  for (;;) {
    const int x0 = max(0, sx - W), x1 = min(n - 1, sx + W);
    const int y0 = max(0, sy - W), y1 = min(n - 1, sy + W);
    const bool whole = x0 == 0 && y0 == 0 && x1 == n - 1 && y1 == n - 1;
    const int b0 = y0 >> 6, b1 = y1 >> 6;
    const long long W2 = (long long)W * W;
    // candidates: the disc of radius W, or every site when the window holds
    // the grid (no certificate needed then)
    const long long Wc = whole ? (1ll << 62) : W2;
    int cnt = 0;
    bool ovf = false;
    int vmin = vlo_sup, vmax = vhi_sup;  // row limits, same-column sites folded in
    if (b1 - b0 <= 1) {  // one or two bands: load the next column ahead
      const uint64_t *p0 = bits + (size_t)b0 * n, *p1 = bits + (size_t)b1 * n;
      const uint64_t m0 = row_mask(y0 - 64 * b0, min(y1 - 64 * b0, 63));
      const uint64_t m1 = b1 > b0 ? row_mask(0, y1 - 64 * b1) : 0ull;
      uint64_t c0 = __ldg(p0 + x0) & m0, c1 = m1 ? __ldg(p1 + x0) & m1 : 0ull;
      for (int x = x0; x <= x1; ++x) {
        uint64_t n0 = 0ull, n1 = 0ull;
        if (x < x1) {
          n0 = __ldg(p0 + x + 1) & m0;
          if (m1) n1 = __ldg(p1 + x + 1) & m1;
        }
        gather_word(c0, x - sx, 64 * b0 - sy, sy, Wc, rec, cnt, ovf, vmin, vmax);
        gather_word(c1, x - sx, 64 * b1 - sy, sy, Wc, rec, cnt, ovf, vmin, vmax);
        c0 = n0;
        c1 = n1;
      }
    } else {
      for (int x = x0; x <= x1; ++x)
        for (int b = b0; b <= b1; ++b)
          gather_word(__ldg(bits + (size_t)b * n + x) &
                          row_mask(max(y0 - 64 * b, 0), min(y1 - 64 * b, 63)),
                      x - sx, 64 * b - sy, sy, Wc, rec, cnt, ovf, vmin, vmax);
    }
    // |K - S v| <= 2 W^2 + 2 W rb: below 2^23 the reciprocal estimate is safe
    const bool fast = 2 * W2 + 2 * (long long)W * rb < (1ll << 23);
    c = CellSums{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
    int R2 = 0;
    // rows outward from s, two per pass over the records: up from v = 0, down
    // from v = -1, inside the row limits
    for (int dir = 1; dir >= -1; dir -= 2) {
      const int vend = dir > 0 ? vmax : vmin;
      for (int v = dir > 0 ? max(0, vmin) : min(-1, vmax); dir > 0 ? v <= vend : v >= vend;
           v += 2 * dir) {
        const RowPair p =
            row_bounds2(rec, cnt, ovf, fast, bits, n, sx, sy, x0, x1, b0, b1, y0, y1, Wc, v, dir);
        if (p.lo0 > p.hi0 + 1) break;  // the cell has ended in this direction
        if (p.lo0 <= p.hi0) take_row(a, n, sx, sy, rb2, v, p.lo0, p.hi0, R2, c);
        const int v1 = v + dir;
        if ((dir > 0 ? v1 > vend : v1 < vend) || p.lo1 > p.hi1 + 1) break;
        if (p.lo1 <= p.hi1) take_row(a, n, sx, sy, rb2, v1, p.lo1, p.hi1, R2, c);
      }
    }
    c.r2 = R2;
    // R2 <= rb^2, so a window of 2 rb always passes
    if (whole || 4 * (long long)R2 <= W2) return c;
    W = min(min(2 * isqrt_ceil(R2) + 1, 2 * W), 2 * rb);
  }
}

// Centroid coordinate base + (Sh + Sl) / (Wh + Wl), rounded once to float
// (two-float quotient; W = 0 gives NaN as the reference's 0/0 does).
__device__ __forceinline__ float cell_centroid(int base, float Sh, float Sl, float Wh, float Wl) {
  const float q = __fdiv_rn(Sh, Wh);
  const float rr = __fadd_rn(__fmaf_rn(-q, Wh, Sh), __fmaf_rn(-q, Wl, Sl));
  const float q2 = __fdiv_rn(rr, Wh);
  float s, e;
  tsum_c((float)base, q, s, e);
  return __fadd_rn(s, __fadd_rn(e, q2));
}

// Add one to *counter after every earlier write of this thread is visible
// (an atomic with release semantics): the writer's half of a counter
// handoff, where whoever brings the counter to its target fences and reads
// the others' results.  Cheaper than a full fence before a plain atomic.
__device__ __forceinline__ unsigned add_release(unsigned *counter) {
  unsigned prev;
  asm volatile("atom.add.release.gpu.u32 %0, [%1], 1;" : "=r"(prev) : "l"(counter) : "memory");
  return prev;
}

__device__ __forceinline__ uint64_t *bits_at(const LevelBufs &a, int k) {
  return k == 0 ? a.bits[0] : (k == 1 ? a.bits[1] : a.bits[2]);
}
__device__ __forceinline__ unsigned *counts_at(const LevelBufs &a, int k) {
  return k == 0 ? a.counts[0] : (k == 1 ? a.counts[1] : a.counts[2]);
}

// Warp reduction of (energy two-float, max r2, max move2) in a fixed order.
__device__ __forceinline__ void warp_reduce(float &eh, float &el, unsigned &r2, unsigned &mv) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, eh, o);
    const float ol = __shfl_xor_sync(0xffffffffu, el, o);
    dfa(eh, el, oh, ol);
  }
  r2 = __reduce_max_sync(0xffffffffu, r2);
  mv = __reduce_max_sync(0xffffffffu, mv);
}

// The gCVT schedule after an iteration of energy E (gcvt.cu:1105-1142), the
// next covering bound, and the rotation of the bitmaps.
__device__ void run_schedule(DevState *st, double E, unsigned r2, unsigned mv, int n, int cur) {
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
  if (st->target_energy > 0.0 && E <= st->target_energy) stop = 1;  // time-to-energy runs
  if (stop) st->stopped = 1;
  st->cover = min(isqrt_ceil((int)r2) + isqrt_ceil((int)mv), 2 * n);
  st->cur = cur == 2 ? 0 : cur + 1;
  st->done_blocks = 0;
  __threadfence();
}

// The end of a pass: MODE 0 and 4 (a plain iteration, MODE 4 also writing
// the learned step's features) run the schedule; MODE 5 (the iteration of
// the jumped sites) also judges the jump: it stands if the jumped sites'
// energy is below the energy of the sites it started from (when no jump was
// proposed, MODE 5 is a plain iteration); MODE 2 (features only, nothing
// moves) just closes the pass.
template <int MODE>
__device__ void pass_done(DevState *st, double E, unsigned r2, unsigned mv, int n, int cur) {
  if (MODE == 5 && st->gate_active) {
    st->gate_e1 = E;
    st->gate_accept = E < st->gate_e0 ? 1 : 0;
  }
  if (MODE == 0 || MODE == 4 || MODE == 5) {
    run_schedule(st, E, r2, mv, n, cur);
  } else {
    st->done_blocks = 0;
    __threadfence();
  }
}

// What one chart's iteration reads at its start.
struct IterView {
  const uint64_t *bits;  // current sites
  uint64_t *nxt;         // where the moved sites go
  unsigned *cnt_nxt;     // their per-list-block counts
  float omega;
  int W0, rb, nsites, cur, nxt_i, slack;
  unsigned ngroups;      // 32-site groups of the list
};

__device__ __forceinline__ IterView iter_view(const LevelBufs &a) {
  const DevState *st = a.st;
  IterView v;
  v.cur = st->snap_cur;
  v.nxt_i = v.cur == 2 ? 0 : v.cur + 1;
  v.bits = bits_at(a, v.cur);
  v.nxt = bits_at(a, v.nxt_i);
  v.cnt_nxt = counts_at(a, v.nxt_i);
  v.omega = st->snap_omega;
  v.W0 = st->snap_window;
  v.rb = st->snap_cover;
  v.nsites = st->snap_count;
  v.slack = st->hint_slack;
  v.ngroups = (unsigned)(v.nsites + 31) / 32;
  return v;
}

// The snapshot k_cell reads (k_list, before the iteration; thread 0 of the
// chart's first list block).  A stopped chart records only that it stopped.
__device__ __forceinline__ void take_snapshot(DevState *st) {
  st->snap_stopped = st->stopped;
  st->snap_cur = st->cur;
  st->snap_omega = st->omega;
  st->snap_window = st->window;
  st->snap_cover = st->cover;
}

// Clear the bitmap and counts the next iteration writes (nobody reads them
// in this one); this thread's grid-stride share.
__device__ __forceinline__ void clear_ahead(const LevelBufs &a, int cur, size_t t0,
                                            size_t gthreads) {
  const size_t nwords = (size_t)(a.n / kBand) * a.n;
  uint64_t *zro = bits_at(a, cur == 0 ? 2 : cur - 1);
  unsigned *czro = counts_at(a, cur == 0 ? 2 : cur - 1);
  for (size_t i = t0; i < nwords; i += gthreads) zro[i] = 0ull;
  const size_t nlb = (nwords + kListWords - 1) / kListWords;
  for (size_t i = t0; i < nlb; i += gthreads) czro[i] = 0u;
}

// Features of listed site idx at (sx, sy) with cell sums cs, for the learned
// step, all in units of the mean cell radius (DevState::feat_scale): its
// pending Lloyd displacement (the centroid of its cell minus the site, not
// yet rounded to a pixel; 0 for a cell without density), its last three
// applied moves (newest first) and the density gradient over the density at
// the site.
__device__ __forceinline__ void site_features(const LevelBufs &a, const IterView &v, int idx,
                                              int sx, int sy, const CellSums &cs) {
  const int n = a.n;
  const float r = a.st->feat_scale, ir = 1.0f / r;
  const uint64_t h = a.hist[v.cur][(size_t)sy * n + sx];
  float *f = a.feat + (size_t)idx * 10;
  const bool mass = cs.wh > 0.f;
  const float cx = mass ? cell_centroid(sx, cs.xh, cs.xl, cs.wh, cs.wl) - (float)sx : 0.f;
  const float cy = mass ? cell_centroid(sy, cs.yh, cs.yl, cs.wh, cs.wl) - (float)sy : 0.f;
  f[0] = cx * ir;
  f[1] = cy * ir;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    f[2 + 2 * k] = (float)(int8_t)(h >> (16 * k)) * ir;
    f[3 + 2 * k] = (float)(int8_t)(h >> (16 * k + 8)) * ir;
  }
  const float *d = a.density;
  const float r0 = d[(size_t)sy * n + sx];
  const int xa = max(sx - 1, 0), xb = min(sx + 1, n - 1), ya = max(sy - 1, 0), yb = min(sy + 1, n - 1);
  const float gx = (d[(size_t)sy * n + xb] - d[(size_t)sy * n + xa]) / (float)(xb - xa);
  const float gy = (d[(size_t)yb * n + sx] - d[(size_t)ya * n + sx]) / (float)(yb - ya);
  f[8] = r0 > 0.f ? gx / r0 * r : 0.f;
  f[9] = r0 > 0.f ? gy / r0 * r : 0.f;
}

// Group g of a chart (32 listed sites, one per lane).  MODE 0: cells, moves,
// and the group's share of the energy reduction; the warp that completes the
// chart's last 64-group runs its schedule.  MODE 1: moments only, written as
// doubles (W, X, Y, E) at each site pixel of out4 (four n*n planes).
// The move of listed site e at (sx, sy) with cell sums cs (gcvt.cu:753-781):
// the over-relaxed centroid rounded to float, then to a pixel; fixed sites
// and zero-density targets stay.  The site goes into the next bitmap (the
// first to set a bit counts it for the next list), leaves its window hint and
// (learned steps) its move history and id at its new pixel.  Returns the
// move's squared length.  With centry, the count is left to the caller: the
// list block to count in goes to *centry (-1: the bit was set already), so
// that a warp adds its group's sites with one atomic per list block instead
// of one per site (many sites land in one list block, and same-address
// atomics serialise).
__device__ __forceinline__ unsigned move_site(const LevelBufs &a, const IterView &v, uint32_t e,
                                              int sx, int sy, const CellSums &cs,
                                              int *centry = nullptr) {
  const int n = a.n;
  const size_t pid = (size_t)sy * n + sx;
  const float cx = cell_centroid(sx, cs.xh, cs.xl, cs.wh, cs.wl);
  const float cy = cell_centroid(sy, cs.yh, cs.yl, cs.wh, cs.wl);
  const float fx = __fadd_rn(__fmaf_rn(__fsub_rn(cx, (float)sx), v.omega, (float)sx), 0.5f);
  const float fy = __fadd_rn(__fmaf_rn(__fsub_rn(cy, (float)sy), v.omega, (float)sy), 0.5f);
  int nx = min(max(__float2int_rz(fx), 0), n - 1);
  int ny = min(max(__float2int_rz(fy), 0), n - 1);
  if ((e & 0x8000u) || a.density[(size_t)ny * n + nx] == 0.0f) { nx = sx; ny = sy; }
  const unsigned mv = (unsigned)((nx - sx) * (nx - sx) + (ny - sy) * (ny - sy));
  const size_t widx = (size_t)(ny / kBand) * n + nx;
  const unsigned long long bit = 1ull << (ny % kBand);
  const unsigned long long old =
      atomicOr(reinterpret_cast<unsigned long long *>(v.nxt + widx), bit);
  const int entry = (old & bit) ? -1 : (int)(widx / kListWords);
  if (centry) *centry = entry;
  else if (entry >= 0) atomicAdd(v.cnt_nxt + entry, 1u);
  const size_t npid = (size_t)ny * n + nx;
  a.hint[npid] = (uint8_t)min(2 * isqrt_ceil(cs.r2) + v.slack, 255);
  if (a.hist[0]) {  // this move becomes the newest of the site's last four
    const int mx = min(max(nx - sx, -127), 127), my = min(max(ny - sy, -127), 127);
    a.hist[v.nxt_i][npid] = (a.hist[v.cur][pid] << 16) | (uint64_t)(uint8_t)mx |
                            ((uint64_t)(uint8_t)my << 8);
  }
  if (a.ids[0]) a.ids[v.nxt_i][npid] = a.ids[v.cur][pid];
  return mv;
}

// The energy reduction after group g (lane i holds site 32 g + i's energy
// two-float, max cell radius^2 and move^2): group total -> slot; the warp
// finishing the last group of a 64-group reduces the 64 slots; the warp
// finishing the last 64-group totals them and closes the pass (pass_done).
template <int MODE>
__device__ __forceinline__ void group_tail(const LevelBufs &a, const IterView &v, unsigned g,
                                           int lane, float eh, float el, unsigned r2,
                                           unsigned mv) {
  DevState *st = a.st;
  warp_reduce(eh, el, r2, mv);
  int last = 0;
  const unsigned sg = g / kGroupsPerSlot;
  const unsigned sbase = sg * kGroupsPerSlot;
  const unsigned starget = min((unsigned)kGroupsPerSlot, v.ngroups - sbase);
  if (lane == 0) {
    a.gslot[g] = make_float4(eh, el, __uint_as_float(r2), __uint_as_float(mv));
    last = add_release(a.scnt + sg) == starget - 1;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence();
  eh = el = 0.f;
  r2 = mv = 0;
  for (unsigned k = lane; k < starget; k += 32) {
    const float4 q = __ldcg(a.gslot + sbase + k);
    dfa(eh, el, q.x, q.y);
    r2 = max(r2, __float_as_uint(q.z));
    mv = max(mv, __float_as_uint(q.w));
  }
  warp_reduce(eh, el, r2, mv);
  const unsigned nslots = (v.ngroups + kGroupsPerSlot - 1) / kGroupsPerSlot;
  last = 0;
  if (lane == 0) {
    a.sslot[sg] = make_float4(eh, el, __uint_as_float(r2), __uint_as_float(mv));
    a.scnt[sg] = 0u;
    last = add_release(&st->done_blocks) == nslots - 1;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence();
  eh = el = 0.f;
  r2 = mv = 0;
  for (unsigned k = lane; k < nslots; k += 32) {
    const float4 q = __ldcg(a.sslot + k);
    dfa(eh, el, q.x, q.y);
    r2 = max(r2, __float_as_uint(q.z));
    mv = max(mv, __float_as_uint(q.w));
  }
  warp_reduce(eh, el, r2, mv);
  if (lane == 0) {
    const double E = ((double)eh + (double)el) * st->energy_scale;
    pass_done<MODE>(st, E, r2, mv, a.n, v.cur);
  }
}

// Group g of a chart (32 listed sites, one per lane).  MODE 0: cells, moves,
// and the group's share of the energy reduction.  MODE 1: moments only,
// written as doubles (W, X, Y, E) at each site pixel of out4 (four n*n
// planes).  MODE 2: the learned step's features of the sites (nothing
// moves).  MODE 4: MODE 0 and the features, with each site's window in
// jaux.  MODE 5: MODE 0 for the jumped sites (the pass then judges the jump).
// The next work item of a persistent warp: its first is its block index (no
// atomic), the rest come from the ticket, numbered after that first wave (a
// ticket every warp takes at once is a burst of same-address atomics).
__device__ __forceinline__ unsigned next_item(unsigned *ticket, bool first, int lane) {
  unsigned g = blockIdx.x;
  if (!first) {
    if (lane == 0) g = gridDim.x + atomicAdd(ticket, 1u);
    g = __shfl_sync(0xffffffffu, g, 0);
  }
  return g;
}

template <int MODE>
__device__ void cell_group(const LevelBufs &a, const IterView &v, unsigned g, int lane,
                           double *out4) {
  const int n = a.n;
  float eh = 0.f, el = 0.f;
  unsigned r2 = 0, mv = 0;
  int centry = -1;
  const int idx = (int)g * 32 + lane;
  if (idx < v.nsites) {
    const uint32_t e = a.list[idx];
    const int sx = (int)(e & 0x7fffu), sy = (int)(e >> 16);
    const size_t pid = (size_t)sy * n + sx;
    const int h = a.hint[pid];
    const CellSums cs = cell_sums(a, v.bits, n, sx, sy, h ? h : v.W0, v.rb);
    if (MODE == 1) {
      const size_t nn = (size_t)n * n;
      const double Wd = (double)cs.wh + (double)cs.wl;
      out4[pid] = Wd;
      out4[nn + pid] = (double)sx * Wd + ((double)cs.xh + (double)cs.xl);
      out4[2 * nn + pid] = (double)sy * Wd + ((double)cs.yh + (double)cs.yl);
      out4[3 * nn + pid] = (double)cs.eh + (double)cs.el;
    } else {
      dfa(eh, el, cs.eh, cs.el);
      r2 = (unsigned)cs.r2;
      if (MODE == 2 || MODE == 4) site_features(a, v, idx, sx, sy, cs);
      if (MODE == 4) a.jaux[idx] = (uint32_t)min(2 * isqrt_ceil(cs.r2) + v.slack, 255);
      if (MODE != 2) mv = move_site(a, v, e, sx, sy, cs, &centry);
    }
  }
  __syncwarp();
  // the group's new sites, counted per list block: one atomic per block
  const unsigned want = __ballot_sync(0xffffffffu, centry >= 0);
  if (centry >= 0) {
    const unsigned peers = __match_any_sync(want, centry);
    if (lane == __ffs(peers) - 1) atomicAdd(v.cnt_nxt + centry, (unsigned)__popc(peers));
  }
  if (MODE == 1) return;
  group_tail<MODE>(a, v, g, lane, eh, el, r2, mv);
}

// ---------------------------------------------------------------------------
// One site per warp, for problems with fewer sites than the GPU holds warps
// (a lane-per-site group then runs one site's whole cell serially, and only
// a few groups exist).  The same cell and the same sums, bit for bit: the
// candidates are gathered by the lanes into shared memory, the rows of the
// walk are bounded and summed one per lane, 32 at a time, and lane 0 folds
// the rows' chunk sums into the cell sums in the lane-per-site order.  The
// energy reduction keeps its groups: each site's contribution waits in
// LevelBufs::sitev, and the warp finishing a group's last site reduces it.
// ---------------------------------------------------------------------------

constexpr int kWarpChunks = 4;  // chunk sums per row kept in shared memory

struct WarpScratch {
  int2 rec[kMaxCand];
  float part[32][kWarpChunks][3];  // per row (lane): chunk sums rw, rx, rq
  int2 span[32];                   // per row: summed pixels [da, db]
};

__device__ CellSums cell_sums_warp(const LevelBufs &a, const uint64_t *__restrict__ bits, int n,
                                   int sx, int sy, int W, int rb, int lane, WarpScratch &ws) {
  constexpr unsigned kFull = 0xffffffffu;
  const int2 yr = *a.sup_range;
  const int vlo_sup = max(yr.x, sy - rb) - sy, vhi_sup = min(yr.y - 1, sy + rb) - sy;
  const int rb2 = rb * rb;
  W = max(1, min(W, 2 * rb));
  CellSums c;
  for (;;) {
    const int x0 = max(0, sx - W), x1 = min(n - 1, sx + W);
    const int y0 = max(0, sy - W), y1 = min(n - 1, sy + W);
    const bool whole = x0 == 0 && y0 == 0 && x1 == n - 1 && y1 == n - 1;
    const int b0 = y0 >> 6, b1 = y1 >> 6, nb = b1 - b0 + 1, ncol = x1 - x0 + 1;
    const long long W2 = (long long)W * W;
    const long long Wc = whole ? (1ll << 62) : W2;
    // candidates: lanes over the window's (column, band) words, records
    // compacted into shared memory in word order
    int cnt = 0;
    int vmin = vlo_sup, vmax = vhi_sup;
    for (int t0 = 0; t0 < ncol * nb; t0 += 32) {
      const int t = t0 + lane;
      uint64_t w = 0ull;
      int A = 0, B0 = 0;
      if (t < ncol * nb) {
        const int x = x0 + t / nb, b = b0 + t % nb;
        w = __ldg(bits + (size_t)b * n + x) & row_mask(max(y0 - 64 * b, 0), min(y1 - 64 * b, 63));
        A = x - sx;
        B0 = 64 * b - sy;
      }
      int mine = 0;
      for (uint64_t q = w; q; q &= q - 1ull) {
        const int B = B0 + __ffsll((long long)q) - 1;
        const int K = A * A + B * B;
        if (K == 0 || (long long)K > Wc) continue;
        if (A == 0) same_column_limit(B, sy, vmin, vmax);
        else ++mine;
      }
      int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += u;
      }
      int pos = cnt + incl - mine;
      if (mine) {
        for (uint64_t q = w; q; q &= q - 1ull) {
          const int B = B0 + __ffsll((long long)q) - 1;
          const int K = A * A + B * B;
          if (K == 0 || (long long)K > Wc || A == 0) continue;
          if (pos < kMaxCand) ws.rec[pos] = make_rec(A, B, K);
          ++pos;
        }
      }
      cnt += __shfl_sync(kFull, incl, 31);
    }
    vmin = __reduce_max_sync(kFull, vmin);
    vmax = __reduce_min_sync(kFull, vmax);
    const bool ovf = cnt > kMaxCand;
    __syncwarp();
    const bool fast = 2 * W2 + 2 * (long long)W * rb < (1ll << 23);
    c = CellSums{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};  // lane 0 accumulates
    int R2 = 0;
    // rows outward from s, up from v = 0 then down from v = -1, 32 per step
    // (one per lane); the walk ends at its first row with lo > hi + 1
    for (int dir = 1; dir >= -1; dir -= 2) {
      const int vend = dir > 0 ? vmax : vmin;
      const int vstart = dir > 0 ? max(0, vmin) : min(-1, vmax);
      for (int base = vstart; dir > 0 ? base <= vend : base >= vend; base += 32 * dir) {
        const int vr = base + dir * lane;
        const bool inr = dir > 0 ? vr <= vend : vr >= vend;
        int lo = -sx, hi = n - 1 - sx;
        if (inr) {
          if (!ovf) {
            for (int k = 0; k < cnt; ++k) {
              const int2 r = ws.rec[k];
              const int S = (int)(int16_t)((unsigned)r.y & 0xffffu);
              const int D = (int)(int16_t)((unsigned)r.y >> 16);
              const int aD = abs(D);
              const int N = r.x - S * vr;
              const int q = fast ? floordiv_r(N, aD, rcp_approx((float)aD))
                                 : floordiv_est(N, aD, 0.f, false);
              if (D > 0) hi = min(hi, q);
              else lo = max(lo, q + 1);
            }
          } else {
            for (int x = x0; x <= x1; ++x)
              for (int b = b0; b <= b1; ++b) {
                uint64_t w = __ldg(bits + (size_t)b * n + x) &
                             row_mask(max(y0 - 64 * b, 0), min(y1 - 64 * b, 63));
                while (w) {
                  const int i = __ffsll((long long)w) - 1;
                  w &= w - 1ull;
                  const int A = x - sx, B = 64 * b + i - sy;
                  const int K = A * A + B * B;
                  if (K == 0 || (long long)K > Wc) continue;
                  constrain_rel(A, B, vr, lo, hi);
                }
              }
          }
        }
        const unsigned sb = __ballot_sync(kFull, !inr || lo > hi + 1);
        const int f = sb ? __ffs(sb) - 1 : 32;  // rows 0 .. f-1 of this step are walked
        int da = 1, db = 0;
        if (lane < f && lo <= hi && row_span(a, sx, sy, rb2, vr, lo, hi, da, db)) {
          R2 = max(R2, max(da * da, db * db) + vr * vr);
          const float *row = a.density + (size_t)(sy + vr) * n + sx;
          int k = 0;
          for (int u0 = da; u0 <= db && k < kWarpChunks; u0 += 16, ++k)
            chunk_sums(row, u0, min(db, u0 + 15), ws.part[lane][k][0], ws.part[lane][k][1],
                       ws.part[lane][k][2]);
        }
        ws.span[lane] = make_int2(da, db);
        __syncwarp();
        if (lane == 0) {
          for (int r = 0; r < f; ++r) {
            const int2 sp = ws.span[r];
            if (sp.x > sp.y) continue;
            const int vv = base + dir * r;
            const float fv = (float)vv, fv2 = (float)(vv * vv);
            const float *row = a.density + (size_t)(sy + vv) * n + sx;
            int k = 0;
            for (int u0 = sp.x; u0 <= sp.y; u0 += 16, ++k) {
              float rw, rx, rq;
              if (k < kWarpChunks) {
                rw = ws.part[r][k][0];
                rx = ws.part[r][k][1];
                rq = ws.part[r][k][2];
              } else {
                chunk_sums(row, u0, min(sp.y, u0 + 15), rw, rx, rq);
              }
              fold_chunk(c, rw, rx, rq, fv, fv2);
            }
          }
        }
        __syncwarp();
        if (f < 32) break;
      }
    }
    R2 = __reduce_max_sync(kFull, R2);
    if (lane == 0) c.r2 = R2;
    if (whole || 4 * (long long)R2 <= W2) return c;
    W = min(min(2 * isqrt_ceil(R2) + 1, 2 * W), 2 * rb);
  }
}

// One Lloyd iteration, one listed site per warp from a site ticket.  MODE
// 0, 4 and 5 as in k_cell (MODE 4 also writes the learned step's features,
// MODE 5 judges a jump and does not clear ahead).
template <int MODE>
__global__ void __launch_bounds__(32, 32) k_cell_warp(LevelBufs a) {
  __shared__ WarpScratch ws;
  DevState *st = a.st;
  if (st->snap_stopped) return;
  const int lane = threadIdx.x;
  const IterView v = iter_view(a);
  if (MODE != 5 || !st->gate_active)
    clear_ahead(a, v.cur, (size_t)blockIdx.x * 32 + lane, (size_t)gridDim.x * 32);
  if (v.ngroups == 0) {  // no sites: the schedule still advances
    if (blockIdx.x == 0 && lane == 0) pass_done<MODE>(st, 0.0, 0u, 0u, a.n, v.cur);
    return;
  }
  if (v.nsites > kWarpSites) {  // more sites than LevelBufs::sitev holds: per lane
    for (bool first = true;; first = false) {
      const unsigned g = next_item(&st->ticket, first, lane);
      if (g >= v.ngroups) return;
      cell_group<MODE>(a, v, g, lane, nullptr);
    }
  }
  const int n = a.n;
  for (bool first = true;; first = false) {
    const unsigned idx = next_item(&st->ticket, first, lane);
    if (idx >= (unsigned)v.nsites) break;
    const uint32_t e = a.list[idx];
    const int sx = (int)(e & 0x7fffu), sy = (int)(e >> 16);
    const int h = a.hint[(size_t)sy * n + sx];
    const CellSums cs = cell_sums_warp(a, v.bits, n, sx, sy, h ? h : v.W0, v.rb, lane, ws);
    const unsigned g = idx / 32;
    int last = 0;
    if (lane == 0) {
      float eh = 0.f, el = 0.f;
      dfa(eh, el, cs.eh, cs.el);
      if (MODE == 4) {
        site_features(a, v, (int)idx, sx, sy, cs);
        a.jaux[idx] = (uint32_t)min(2 * isqrt_ceil(cs.r2) + v.slack, 255);
      }
      const unsigned mv = move_site(a, v, e, sx, sy, cs);
      a.sitev[idx] = make_float4(eh, el, __uint_as_float((unsigned)cs.r2), __uint_as_float(mv));
      const unsigned gsize = min(32u, (unsigned)v.nsites - g * 32);
      last = add_release(a.gcnt + g) == gsize - 1;
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) continue;
    // the group's last site: its values in lane order, then the usual tail
    __threadfence();
    float eh = 0.f, el = 0.f;
    unsigned r2 = 0, mv = 0;
    if (g * 32 + lane < (unsigned)v.nsites) {
      const float4 q = __ldcg(a.sitev + g * 32 + lane);
      eh = q.x, el = q.y, r2 = __float_as_uint(q.z), mv = __float_as_uint(q.w);
    }
    if (lane == 0) a.gcnt[g] = 0u;
    group_tail<MODE>(a, v, g, lane, eh, el, r2, mv);
  }
}

// One chart.  MODE 0: one Lloyd iteration (sums, move, energy, schedule).
// MODE 1: moments only (gcvt_ctx_moments); the sites do not move.
// MODE 2: the learned step's features of the sites (LevelBufs::feat);
//         nothing moves.
// MODE 4: MODE 0 and the features, for a jump from these sites.
// MODE 5: MODE 0 for the jumped sites without clearing ahead (the bitmap
//         after next holds the plain step's sites until the gate decides),
//         and the gate's decision (DevState::gate_accept); when no jump was
//         proposed (DevState::gate_active 0), exactly MODE 0.
template <int MODE>
__global__ void __launch_bounds__(32, 32) k_cell(LevelBufs a, double *out4) {
  DevState *st = a.st;
  constexpr bool kMoves = MODE == 0 || MODE == 4 || MODE == 5;
  if (kMoves && st->snap_stopped) return;
  const int lane = threadIdx.x;
  const IterView v = iter_view(a);
  // MODE 5 keeps the bitmap after next (the plain step's sites) while a jump
  // is judged; without a jump it is a plain iteration
  if (MODE == 0 || MODE == 4 || (MODE == 5 && !st->gate_active))
    clear_ahead(a, v.cur, (size_t)blockIdx.x * 32 + lane, (size_t)gridDim.x * 32);
  if (MODE != 1 && v.ngroups == 0) {  // no sites: the schedule still advances
    if (blockIdx.x == 0 && lane == 0) pass_done<MODE>(st, 0.0, 0u, 0u, a.n, v.cur);
    return;
  }
  for (bool first = true;; first = false) {
    const unsigned g = next_item(&st->ticket, first, lane);
    if (g >= v.ngroups) break;
    cell_group<MODE>(a, v, g, lane, out4);
  }
}

// Many charts, one launch: the groups of all charts that have not stopped form
// one sequence (group offsets per chart from k_list_batch, gofs[c] .. gofs[c+1]),
// handed out by one ticket; each chart keeps its own state, reduction and
// schedule, so a chart's iteration is the same as in k_cell.  MODE 0, 4, 5 as
// in k_cell.
template <int MODE>
__global__ void __launch_bounds__(32, 32) k_cell_batch(const LevelBufs *__restrict__ charts,
                                                       int nchart,
                                                       const unsigned *__restrict__ gofs,
                                                       unsigned *ticket) {
  const int lane = threadIdx.x;
  const size_t t0 = (size_t)blockIdx.x * 32 + lane, gthreads = (size_t)gridDim.x * 32;
  for (int c = 0; c < nchart; ++c) {
    const LevelBufs &a = charts[c];
    DevState *st = a.st;
    if (st->snap_stopped) continue;
    const int cur = st->snap_cur;
    if (MODE != 5 || !st->gate_active) clear_ahead(a, cur, t0, gthreads);
    if (st->snap_count == 0 && blockIdx.x == 0 && lane == 0)
      pass_done<MODE>(st, 0.0, 0u, 0u, a.n, cur);
  }
  const unsigned total = gofs[nchart];
  for (bool first = true;; first = false) {
    const unsigned g = next_item(ticket, first, lane);
    if (g >= total) break;
    int lo = 0, hi = nchart - 1;  // the chart c with gofs[c] <= g < gofs[c + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(gofs + mid) <= g) lo = mid;
      else hi = mid - 1;
    }
    const LevelBufs &a = charts[lo];
    const IterView v = iter_view(a);
    cell_group<MODE>(a, v, g - __ldg(gofs + lo), lane, nullptr);
  }
}

// Block `blk` of a chart's site list: the sites of bitmap words
// [blk kListWords, (blk+1) kListWords) in bitmap order (word by word, bits in
// row order) with the fixed flag, at the offset the per-block counts give.
// The chart's last block records the list length.
__device__ void list_block(const LevelBufs &a, unsigned blk, unsigned nblk) {
  constexpr int kPer = kListWords / 256;
  __shared__ unsigned wsum[8];
  __shared__ unsigned base_s;
  DevState *st = a.st;
  const int n = a.n;
  const int cur = st->cur;
  const uint64_t *bits = bits_at(a, cur);
  const unsigned *counts = counts_at(a, cur);
  const size_t nwords = (size_t)(n / kBand) * n;
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  if (blk == 0 && tid == 0) {
    st->done_blocks = 0u;
    take_snapshot(st);
  }
  // offset of this block: the counts of the blocks before it
  unsigned pre = 0;
  for (unsigned k = tid; k < blk; k += 256) pre += counts[k];
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
  // this thread's words and their sites
  const size_t w0 = (size_t)blk * kListWords + (size_t)tid * kPer;
  uint64_t w[kPer];
  unsigned cnt = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    w[k] = (w0 + k < nwords) ? bits[w0 + k] : 0ull;
    cnt += __popcll(w[k]);
  }
  // exclusive scan of cnt over the block
  unsigned incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  __syncthreads();  // every thread has read base_s / wsum
  if (lane == 31) wsum[wib] = incl;
  __syncthreads();
  unsigned woff = 0, total = 0;
  for (int k = 0; k < 8; ++k) {
    const unsigned v = wsum[k];
    if (k < wib) woff += v;
    total += v;
  }
  unsigned pos = base + woff + incl - cnt;
  const unsigned cap = (unsigned)n * (unsigned)n;  // list capacity at this size
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    uint64_t word = w[k];
    if (!word) continue;
    const size_t t = w0 + k;
    const int x = (int)(t % (unsigned)n), band = (int)(t / (unsigned)n);
    const uint64_t fw = a.fixed_bits[t];
    while (word) {
      const int i = __ffsll((long long)word) - 1;
      word &= word - 1ull;
      if (pos < cap)
        a.list[pos] = (uint32_t)x | ((uint32_t)(band * kBand + i) << 16) |
                      ((uint32_t)((fw >> i) & 1ull) << 15);
      ++pos;
    }
  }
  if (blk == nblk - 1 && tid == 0) st->list_count = st->snap_count = (int)min(base + total, cap);
  __syncthreads();  // the shared scratch may be reused by the caller
}

// One chart's site list; also rearms the chart's ticket.  respect_stop = 0
// lists a stopped chart too (moments, point extraction) and marks the
// snapshot running.
__global__ void __launch_bounds__(256) k_list(LevelBufs a, int respect_stop) {
  DevState *st = a.st;
  if (respect_stop && st->stopped) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->snap_stopped = 1;
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st->ticket = 0u;
  list_block(a, blockIdx.x, gridDim.x);
  if (!respect_stop && blockIdx.x == 0 && threadIdx.x == 0) st->snap_stopped = 0;
}

// The site lists of many charts: chart c owns blocks lofs[c] .. lofs[c+1].
// The block that finishes last lays out the group offsets of the charts that
// run (gofs) for k_cell_batch and rearms its ticket.
__global__ void __launch_bounds__(256) k_list_batch(const LevelBufs *__restrict__ charts,
                                                    int nchart,
                                                    const unsigned *__restrict__ lofs,
                                                    unsigned *gofs, unsigned *done,
                                                    unsigned *ticket) {
  __shared__ bool is_last;
  int lo = 0, hi = nchart - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(lofs + mid) <= blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  const LevelBufs &a = charts[lo];
  const unsigned blk = blockIdx.x - __ldg(lofs + lo);
  if (!a.st->stopped) list_block(a, blk, __ldg(lofs + lo + 1) - __ldg(lofs + lo));
  else if (blk == 0 && threadIdx.x == 0) a.st->snap_stopped = 1;
  if (threadIdx.x == 0) {
    __threadfence();
    is_last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last || threadIdx.x != 0) return;
  __threadfence();
  unsigned acc = 0;
  for (int c = 0; c < nchart; ++c) {
    gofs[c] = acc;
    const DevState *st = charts[c].st;
    const int cnt = *((volatile const int *)&st->snap_count);
    if (!*((volatile const int *)&st->snap_stopped)) acc += (unsigned)(cnt + 31) / 32;
  }
  gofs[nchart] = acc;
  *ticket = 0u;
  *done = 0u;
  __threadfence();
}

// Per-block site counts of the current bitmap (for the first k_list of a
// level; afterwards k_cell counts the sites it places).
__global__ void __launch_bounds__(256) k_count(LevelBufs a) {
  constexpr int kPer = kListWords / 256;
  __shared__ unsigned wsum[8];
  const int n = a.n;
  const int cur = a.st->cur;
  const uint64_t *bits = bits_at(a, cur);
  unsigned *counts = counts_at(a, cur);
  const size_t nwords = (size_t)(n / kBand) * n;
  const size_t w0 = (size_t)blockIdx.x * kListWords + (size_t)threadIdx.x * kPer;
  unsigned cnt = 0;
  for (int k = 0; k < kPer; ++k)
    if (w0 + k < nwords) cnt += __popcll(bits[w0 + k]);
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned s = 0;
    for (int k = 0; k < 8; ++k) s += wsum[k];
    counts[blockIdx.x] = s;
  }
}

// Covering bound from a label grid: cover = ceil(sqrt(max |p - label(p)|^2))
// over the pixels of the density's row support.  One block per row.
// hint[pid] = max(hint[pid], b) on the byte inside its 32-bit word.  Each
// failed compare-and-swap means another byte of the word grew, so the loop is
// short; past the limit the hint just stays lower (a wider first window).
__device__ __forceinline__ void hint_max(uint8_t *hint, size_t pid, unsigned b) {
  unsigned *word = reinterpret_cast<unsigned *>(hint + (pid & ~(size_t)3));
  const int sh = (int)(pid & 3) * 8;
  unsigned old = *reinterpret_cast<volatile unsigned *>(word);
  for (int k = 0; k < 64 && ((old >> sh) & 0xffu) < b; ++k) {
    const unsigned prev = atomicCAS(word, old, (old & ~(0xffu << sh)) | (b << sh));
    if (prev == old) break;
    old = prev;
  }
}

// Covering bound of a label grid (max over density pixels of the squared
// distance to their site), and each site's first window: 2 R + slack with R
// the largest distance from the site to a density pixel of its cell (hint at
// the site pixel, zeroed before), so the first iteration after a load needs
// no window retries.
__global__ void __launch_bounds__(256) k_cover(LevelBufs a) {
  const int n = a.n, y = blockIdx.x;
  const int2 yr = *a.sup_range;
  const unsigned slack = (unsigned)a.st->hint_slack;
  const int lane = threadIdx.x & 31;
  unsigned m = 0;
  if (y >= yr.x && y < yr.y) {
    const int2 s = a.support[y];
    const uint32_t *row = a.labels + (size_t)y * n;
    // 32 consecutive pixels per warp step: the lanes holding one site's label
    // (runs along the row) reduce together, one of them updates the hint
    for (int base = s.x + (int)(threadIdx.x & ~31u); base < s.y; base += blockDim.x) {
      const int x = base + lane;
      const uint32_t v = x < s.y ? row[x] : kMarkerWord;
      const int lx = (int16_t)(v & 0xffffu), ly = (int16_t)(v >> 16);
      const bool site = lx != kMarker;
      const unsigned d2 = site ? (unsigned)((x - lx) * (x - lx) + (y - ly) * (y - ly)) : 0u;
      m = max(m, d2);
      const unsigned grp = __match_any_sync(0xffffffffu, site ? v : kMarkerWord);
      const unsigned g2 = __reduce_max_sync(grp, d2);
      if (site && lane == __ffs(grp) - 1) {
        // ceil(sqrt(g2)) from a float square root, one integer correction up
        unsigned r = (unsigned)sqrtf((float)g2);
        if (r * r < g2) ++r;
        const unsigned b = min(2u * r + slack, 255u);
        const size_t pid = (size_t)ly * n + lx;
        if (a.hint[pid] < b) hint_max(a.hint, pid, b);
      }
    }
  }
  // the block's maximum, then one atomic per block (one per warp onto the
  // single accumulator serialised at the L2)
  __shared__ unsigned wmax[8];
  m = __reduce_max_sync(0xffffffffu, m);
  if (lane == 0) wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = max(m, wmax[w]);
    if (m) atomicMax(&a.st->cover_acc, m);
  }
}
__global__ void k_cover_finish(LevelBufs a) {
  DevState *st = a.st;
  st->cover = min(isqrt_ceil((int)st->cover_acc), 2 * a.n);
  st->cover_acc = 0;
}

cudaError_t launch_cover(const LevelBufs &b, cudaStream_t s) {
  k_cover<<<b.n, 256, 0, s>>>(b);
  k_cover_finish<<<1, 1, 0, s>>>(b);
  return cudaGetLastError();
}

size_t list_blocks(int n) {
  const size_t nwords = (size_t)(n / kBand) * n;
  return (nwords + kListWords - 1) / kListWords;
}

size_t cell_groups(int n) { return ((size_t)n * n + 31) / 32; }

cudaError_t launch_list(const LevelBufs &b, int respect_stop, cudaStream_t s) {
  k_list<<<(unsigned)list_blocks(b.n), 256, 0, s>>>(b, respect_stop);
  return cudaGetLastError();
}

cudaError_t launch_count(const LevelBufs &b, cudaStream_t s) {
  k_count<<<(unsigned)list_blocks(b.n), 256, 0, s>>>(b);
  return cudaGetLastError();
}

// Persistent grid of the Lloyd kernel: every warp that fits, per device.
static int g_cell_grid[64] = {};
static int g_warp_grid[64] = {};  // k_cell_warp: its own carveout and occupancy

cudaError_t cells_configure() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (g_cell_grid[dev]) return cudaSuccess;
  int sms = 0, per0 = 0, per1 = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;
  // the candidate records live in local memory: shared memory only for the
  // 1 KB the runtime reserves per block (32 blocks per SM), the rest as L1
  const int carve = 15;
  if ((e = cudaFuncSetAttribute(k_cell<0>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                carve)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_cell<1>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                carve)) != cudaSuccess)
    return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, k_cell<0>, 32, 0)) != cudaSuccess)
    return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, k_cell<1>, 32, 0)) != cudaSuccess)
    return e;
  // every persistent variant shares the grid: the fewest blocks any of them fits
  auto fit = [&](auto fn) -> cudaError_t {
    int per = 0;
    cudaError_t r = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carve);
    if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 32, 0);
    if (r == cudaSuccess) per0 = min(per0, per);
    return r;
  };
  for (auto fn : {k_cell_batch<0>, k_cell_batch<4>, k_cell_batch<5>})
    if ((e = fit(fn)) != cudaSuccess) return e;
  for (auto fn : {k_cell<2>, k_cell<4>, k_cell<5>})
    if ((e = fit(fn)) != cudaSuccess) return e;
  // one site per warp: its shared scratch (candidates, chunk sums) needs about
  // 3.3 KB per block with the reserved 1 KB
  int perw = 0;
  for (auto fn : {k_cell_warp<0>, k_cell_warp<4>, k_cell_warp<5>}) {
    int per = 0;
    if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 50)) !=
        cudaSuccess)
      return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 32, 0)) != cudaSuccess)
      return e;
    perw = perw ? min(perw, per) : per;
  }
  g_warp_grid[dev] = sms * max(1, perw);
  g_cell_grid[dev] = sms * max(1, min(per0, per1));
  return cudaSuccess;
}

cudaError_t launch_list_batch(const LevelBufs *charts, int nchart, const unsigned *lofs,
                              unsigned nblocks, unsigned *gofs, unsigned *done, unsigned *ticket,
                              cudaStream_t s) {
  k_list_batch<<<nblocks, 256, 0, s>>>(charts, nchart, lofs, gofs, done, ticket);
  return cudaGetLastError();
}

cudaError_t launch_cells_batch(const LevelBufs *charts, int nchart, const unsigned *gofs,
                               unsigned *ticket, cudaStream_t s, int mode) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || !g_cell_grid[dev]) return cudaErrorNotReady;
  const int grid = g_cell_grid[dev];
  switch (mode) {
    case 4: k_cell_batch<4><<<grid, 32, 0, s>>>(charts, nchart, gofs, ticket); break;
    case 5: k_cell_batch<5><<<grid, 32, 0, s>>>(charts, nchart, gofs, ticket); break;
    default: k_cell_batch<0><<<grid, 32, 0, s>>>(charts, nchart, gofs, ticket);
  }
  return cudaGetLastError();
}

int cells_default_grid() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  return g_cell_grid[dev];
}

// grid: the persistent grid in blocks (0: every block that fits).
cudaError_t launch_cells(const LevelBufs &b, int moments_only, double *out4, cudaStream_t s,
                         int grid) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || !g_cell_grid[dev]) return cudaErrorNotReady;
  if (grid <= 0 || grid > g_cell_grid[dev]) grid = g_cell_grid[dev];
  if ((moments_only == 0 || moments_only == 4 || moments_only == 5) && b.sitev && b.gcnt) {
    const int wg = min(grid, g_warp_grid[dev]);
    if (moments_only == 4) k_cell_warp<4><<<wg, 32, 0, s>>>(b);
    else if (moments_only == 5) k_cell_warp<5><<<wg, 32, 0, s>>>(b);
    else k_cell_warp<0><<<wg, 32, 0, s>>>(b);
    return cudaGetLastError();
  }
  switch (moments_only) {
    case 1: k_cell<1><<<grid, 32, 0, s>>>(b, out4); break;
    case 2: k_cell<2><<<grid, 32, 0, s>>>(b, out4); break;
    case 4: k_cell<4><<<grid, 32, 0, s>>>(b, out4); break;
    case 5: k_cell<5><<<grid, 32, 0, s>>>(b, out4); break;
    default: k_cell<0><<<grid, 32, 0, s>>>(b, out4);
  }
  return cudaGetLastError();
}

}  // namespace cvtgb
