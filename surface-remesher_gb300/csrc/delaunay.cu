// delaunay.cu -- the Delaunay triangulation of a context's free sites on the
// GPU, in the point order of delaunayInput (delaunay.h:46-57), so that its
// triangles index gcvt_ctx_extract_points' list and feed gcvt_lift.  This is
// the Delaunay part of the reference's CDT stage (gDel2D,
// gDel2D/GPU/GpuDelaunay.cu:46) for the CVT sites; constraint points and
// segments are not inserted.
//
// Sites lie on the integer pixel lattice, so every predicate is exact in
// 64-bit / 128-bit integers.  Co-circular sites (common on a lattice) are
// resolved by symbolic perturbation of the lifting map (simulation of
// simplicity): z(q) = |q|^2 + delta(q), with delta(q) > 0 infinitesimal and
// infinitely larger for a larger rank h(q) = y n + x.  The perturbed lifted
// points are in general position, so their lower hull is one Delaunay
// triangulation of the sites, and every site that evaluates a predicate
// gets the same sign, so all stars agree.
//
// Each site's Delaunay star (its neighbours in angular order) is computed
// by one warp from the sites in a window around it: inverted about the
// site, the star is the part of the candidates' convex hull facing away from
// the site, so the candidates are inserted one by one into a sorted cyclic
// list held in the warp's registers (a candidate inside the current hull
// never becomes a neighbour later; an inserted one removes the neighbours it
// covers).  Certificate, exact: a triangle of the star is final when no site
// outside the window lies in its circumcircle, an open angular gap (>= pi)
// when no site lies strictly inside its cone (then the site is on the
// sites' convex hull); both are searched through a pyramid of tile
// occupancy, and a site found is inserted and the star checked again.  Only
// a star of fewer than two neighbours widens the window (a window covering
// the grid is exact).  Warps take the sites in tile order; a triangle is
// written by its vertex that comes first in delaunayInput's order (x, then
// y), counter-clockwise, so the output does not depend on the scheduling.
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <climits>

namespace cvtgb {

namespace {

constexpr int kStar = 64;  // Delaunay neighbours a site can hold

// (dx, dy) packed in one int: dx in the low 16 bits, dy in the high 16
__device__ __forceinline__ int pk(int dx, int dy) {
  return (int)((unsigned)(dx & 0xffff) | ((unsigned)dy << 16));
}
__device__ __forceinline__ int pdx(int v) { return (int)(int16_t)(v & 0xffff); }
__device__ __forceinline__ int pdy(int v) { return v >> 16; }

__device__ __forceinline__ long long cross(int ax, int ay, int bx, int by) {
  return (long long)ax * by - (long long)ay * bx;
}

// angular order around the site: half 0 = [0, pi), half 1 = [pi, 2 pi)
__device__ __forceinline__ int half_of(int x, int y) {
  return (y > 0 || (y == 0 && x > 0)) ? 0 : 1;
}

// the CCW angle from a to b is >= pi (b not strictly left of a, and not the
// same ray)
__device__ __forceinline__ bool open_gap(int ax, int ay, int bx, int by) {
  const long long c = cross(ax, ay, bx, by);
  if (c > 0) return false;
  if (c < 0) return true;
  return (long long)ax * bx + (long long)ay * by < 0;  // opposite rays: exactly pi
}

// Perturbed incircle: is d strictly inside the circle through the site
// (origin), a and b (counter-clockwise)?  Coordinates relative to the site;
// hp, ha, hb, hd the ranks h(q) = y n + x.  With n <= 8192 every
// coordinate difference is below 2^14, each cofactor and lifted term below
// 2^29 and the determinant below 2^61: exact in 64-bit integers.
__device__ __forceinline__ bool in_circle(int ax, int ay, int bx, int by, int dx, int dy,
                                          long long hp, long long ha, long long hb,
                                          long long hd) {
  // rows: p - d, a - d, b - d (p = origin)
  const int r0x = -dx, r0y = -dy, r1x = ax - dx, r1y = ay - dy, r2x = bx - dx, r2y = by - dy;
  const long long m0 = (long long)r1x * r2y - (long long)r1y * r2x;  // cofactor of row 0
  const long long m1 = (long long)r0x * r2y - (long long)r0y * r2x;
  const long long m2 = (long long)r0x * r1y - (long long)r0y * r1x;
  const long long z0 = (long long)r0x * r0x + (long long)r0y * r0y,
                  z1 = (long long)r1x * r1x + (long long)r1y * r1y,
                  z2 = (long long)r2x * r2x + (long long)r2y * r2y;
  const long long d0 = z0 * m0 - z1 * m1 + z2 * m2;
  if (d0 != 0) return d0 > 0;
  // co-circular: z(q) += delta(q), delta growing (infinitesimally) with
  // h(q); the determinant is linear in the z column, so the sign is that of
  // the top-ranked point's cofactor (none is zero: no three of four
  // co-circular points are collinear)
  if (hp > ha && hp > hb && hp > hd) return m0 > 0;
  if (ha > hb && ha > hd) return m1 < 0;
  if (hb > hd) return m2 > 0;
  return m0 - m1 + m2 < 0;
}

__device__ __forceinline__ long long hkey(int n, int x, int y) { return (long long)y * n + x; }

// Tiles are visited in bricks of 4 x 4 (64 x 64 pixels), so that the sites
// a warp handles lie close together and their windows overlap.
constexpr int kBrick = 4;
__device__ __forceinline__ int brick_of(int tx, int ty, int nt0) {
  return ((ty / kBrick) * (nt0 / kBrick) + tx / kBrick) * (kBrick * kBrick) +
         (ty % kBrick) * kBrick + tx % kBrick;
}

// Is every grid point in the closed circumdisc of (site, u, w) inside the
// window?  Relative to the site: centre (Nx, Ny) / D (D > 0), radius^2
// (Nx^2 + Ny^2) / D^2 (the circle passes through the site).  The grid
// outside the window [x0, x1] x [y0, y1] is up to four strips; the disc
// must stay strictly clear of each (exact in 128-bit integers).
__device__ __forceinline__ __int128 axis_gap(long long N, long long D, int lo, int hi) {
  const __int128 a = (__int128)lo * D - N, b = (__int128)N - (__int128)hi * D;
  return a > 0 ? a : (b > 0 ? b : (__int128)0);
}
__device__ bool clear_of(long long Nx, long long Ny, long long D, int lx, int hx, int ly,
                         int hy) {
  if (lx > hx || ly > hy) return true;  // empty strip
  const __int128 gx = axis_gap(Nx, D, lx, hx), gy = axis_gap(Ny, D, ly, hy);
  return gx * gx + gy * gy > (__int128)Nx * Nx + (__int128)Ny * Ny;
}
__device__ bool disc_in_window(int ux, int uy, int wx, int wy, int sx, int sy, int x0, int x1,
                               int y0, int y1, int n) {
  const long long u2 = (long long)ux * ux + (long long)uy * uy,
                  w2 = (long long)wx * wx + (long long)wy * wy;
  const long long D = 2 * cross(ux, uy, wx, wy);
  const long long Nx = wy * u2 - uy * w2, Ny = ux * w2 - wx * u2;
  const int gx0 = -sx, gx1 = n - 1 - sx, gy0 = -sy, gy1 = n - 1 - sy;  // the grid
  const int wx0 = x0 - sx, wx1 = x1 - sx, wy0 = y0 - sy, wy1 = y1 - sy;  // the window
  return clear_of(Nx, Ny, D, gx0, wx0 - 1, gy0, gy1) &&
         clear_of(Nx, Ny, D, wx1 + 1, gx1, gy0, gy1) &&
         clear_of(Nx, Ny, D, wx0, wx1, gy0, wy0 - 1) &&
         clear_of(Nx, Ny, D, wx0, wx1, wy1 + 1, gy1);
}

// Site occupancy of 16 x 16 pixel tiles and its pyramid (level l: tiles of
// 16 << l pixels, a byte each, nonzero when the tile holds a site).
constexpr int kTile = 16;  // 1 << 4
constexpr int kLevels = 16;
struct Pyr {
  const uint8_t *occ;
  int off[kLevels], nt[kLevels];
  int top;  // the one-node level
};

// Free sites: bits & ~fixed.
__device__ __forceinline__ uint64_t free_word(const uint64_t *bits, const uint64_t *fixed,
                                              size_t i) {
  return fixed ? bits[i] & ~fixed[i] : bits[i];
}

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// The star of one site, held by a warp: neighbour k (packed (dx, dy),
// angular order) in lane k % 32 of `a` (k < 32) or of `b`; m and overflow
// are the same in every lane.  Every function below is called by all 32
// lanes with the same arguments and takes the same branches in each.
struct WStar {
  int a, b;
  int m;
  bool overflow;
};

__device__ __forceinline__ int wget(const WStar &s, int k) {
  return __shfl_sync(kFull, k < 32 ? s.a : s.b, k & 31);
}

__device__ __forceinline__ void wset(WStar &s, int k, int v) {
  if (lane_id() == (k & 31)) {
    if (k < 32) s.a = v;
    else s.b = v;
  }
}

// v becomes neighbour pos; neighbours pos.. move up one
__device__ __forceinline__ void wins(WStar &s, int pos, int v) {
  const int l = lane_id();
  const int aup = __shfl_up_sync(kFull, s.a, 1), bup = __shfl_up_sync(kFull, s.b, 1);
  const int a31 = __shfl_sync(kFull, s.a, 31);
  const int na = l < pos ? s.a : (l == pos ? v : aup);
  const int nb = l + 32 < pos ? s.b : (l + 32 == pos ? v : (l == 0 ? a31 : bup));
  s.a = na;
  s.b = nb;
  ++s.m;
}

// neighbour k leaves; neighbours k+1.. move down one
__device__ __forceinline__ void wdel(WStar &s, int k) {
  const int l = lane_id();
  const int adn = __shfl_down_sync(kFull, s.a, 1), bdn = __shfl_down_sync(kFull, s.b, 1);
  const int b0 = __shfl_sync(kFull, s.b, 0);
  const int na = l < k ? s.a : (l == 31 ? b0 : adn);
  const int nb = l + 32 < k ? s.b : bdn;
  s.a = na;
  s.b = nb;
  --s.m;
}

// Insert candidate q (relative (qx, qy)) into the star of site (sx, sy).
// The star is sorted by angle from the +x axis; inverted about the site, its
// neighbours are the hull vertices facing away from the site, and a
// candidate inside that hull never becomes one later (the hull only grows).
__device__ void winsert(WStar &st, int n, int sx, int sy, int qx, int qy) {
  const long long hp = hkey(n, sx, sy), hq = hkey(n, sx + qx, sy + qy);
  const int qv = pk(qx, qy), l = lane_id();
  int m = st.m;
  // q's position (the neighbours before it in angle form a prefix) and a
  // neighbour on the same ray, each lane for its two entries
  const int hqh = half_of(qx, qy);
  bool ba = false, sa = false, bb = false, sb = false;
  if (l < m) {
    const int ux = pdx(st.a), uy = pdy(st.a), hu = half_of(ux, uy);
    const long long c = cross(ux, uy, qx, qy);
    ba = hu < hqh || (hu == hqh && c > 0);
    sa = c == 0 && hu == hqh;
  }
  if (l + 32 < m) {
    const int ux = pdx(st.b), uy = pdy(st.b), hu = half_of(ux, uy);
    const long long c = cross(ux, uy, qx, qy);
    bb = hu < hqh || (hu == hqh && c > 0);
    sb = c == 0 && hu == hqh;
  }
  const unsigned mba = __ballot_sync(kFull, ba), mbb = __ballot_sync(kFull, bb);
  const unsigned msa = __ballot_sync(kFull, sa), msb = __ballot_sync(kFull, sb);
  const int pos = __popc(mba) + __popc(mbb);
  const int same = msa ? __ffs(msa) - 1 : (msb ? 31 + __ffs(msb) : -1);
  int iq;
  if (same >= 0) {
    // the nearer site on a ray wins (the farther one is strictly inside
    // every circle through the site and the nearer one); a nearer q lies
    // outside the hull, so it takes the neighbour's place
    const int u = wget(st, same), ux = pdx(u), uy = pdy(u);
    if ((long long)qx * qx + (long long)qy * qy >= (long long)ux * ux + (long long)uy * uy) return;
    wset(st, same, qv);
    iq = same;
  } else {
    if (m >= 2) {
      const int u = wget(st, (pos + m - 1) % m), w = wget(st, pos % m);
      const int ux = pdx(u), uy = pdy(u), wx = pdx(w), wy = pdy(w);
      if (!open_gap(ux, uy, wx, wy) &&
          !in_circle(ux, uy, wx, wy, qx, qy, hp, hkey(n, sx + ux, sy + uy),
                     hkey(n, sx + wx, sy + wy), hq))
        return;  // inside the hull: never a neighbour
    }
    if (m >= kStar) {
      st.overflow = true;
      return;
    }
    wins(st, pos, qv);
    m = st.m;
    iq = pos;
  }
  // neighbours q now covers: clockwise of q, then counter-clockwise
  while (m >= 3) {
    const int iu = iq ? iq - 1 : m - 1, iuu = iu ? iu - 1 : m - 1;
    const int u = wget(st, iu), uu = wget(st, iuu);
    const int ax = pdx(uu), ay = pdy(uu), vx = pdx(u), vy = pdy(u);
    if (open_gap(ax, ay, qx, qy) ||
        in_circle(ax, ay, qx, qy, vx, vy, hp, hkey(n, sx + ax, sy + ay), hq,
                  hkey(n, sx + vx, sy + vy)))
      break;
    wdel(st, iu);
    m = st.m;
    if (iu < iq) --iq;
  }
  while (m >= 3) {
    const int iw = iq + 1 < m ? iq + 1 : 0, iww = iw + 1 < m ? iw + 1 : 0;
    const int w = wget(st, iw), ww = wget(st, iww);
    const int bx = pdx(ww), by = pdy(ww), vx = pdx(w), vy = pdy(w);
    if (open_gap(qx, qy, bx, by) ||
        in_circle(qx, qy, bx, by, vx, vy, hp, hq, hkey(n, sx + bx, sy + by),
                  hkey(n, sx + vx, sy + vy)))
      break;
    wdel(st, iw);
    m = st.m;
    if (iw < iq) --iq;
  }
}

// Rows [lo, hi] of band b as a bit mask.
__device__ __forceinline__ uint64_t band_rows(int b, int lo, int hi) {
  lo = max(lo - b * kBand, 0);
  hi = min(hi - b * kBand, kBand - 1);
  if (lo > hi) return 0ull;
  const uint64_t up = hi >= 63 ? ~0ull : ((2ull << hi) - 1ull);
  return up & ~((1ull << lo) - 1ull);
}

// Insert the free sites of the window [nx0, nx1] x [ny0, ny1] that are not
// in the window [x0, x1] x [y0, y1] inserted before; the lanes take 32
// columns at a time, then insert the sites they found one by one.
__device__ void wwindow(WStar &st, const uint64_t *bits, const uint64_t *fixed, int n, int sx,
                        int sy, int nx0, int nx1, int ny0, int ny1, int x0, int x1, int y0,
                        int y1) {
  const int l = lane_id();
  for (int cx = nx0; cx <= nx1; cx += 32) {
    const int x = cx + l;
    for (int b = ny0 / kBand; b <= ny1 / kBand; ++b) {
      uint64_t w = 0;
      if (x <= nx1) {
        w = free_word(bits, fixed, (size_t)b * n + x) & band_rows(b, ny0, ny1);
        if (x >= x0 && x <= x1) w &= ~band_rows(b, y0, y1);
      }
      unsigned pend = __ballot_sync(kFull, w != 0);
      while (pend) {
        const int L = __ffs(pend) - 1;
        pend &= pend - 1u;
        uint64_t wl = __shfl_sync(kFull, (unsigned long long)w, L);
        while (wl) {
          const int i = __ffsll((long long)wl) - 1;
          wl &= wl - 1ull;
          const int qx = cx + L - sx, qy = b * kBand + i - sy;
          if (qx != 0 || qy != 0) winsert(st, n, sx, sy, qx, qy);
        }
      }
    }
  }
}

// The bounding box of the closed disc with centre (Nx, Ny) / D relative to
// the site (radius = |centre|): FP64 with one pixel of slack, clipped to
// the grid, so it holds every grid point of the disc.
__device__ __forceinline__ void disc_box(long long Nx, long long Ny, long long D, int sx, int sy,
                                         int n, int &bx0, int &bx1, int &by0, int &by1) {
  const double cx = (double)Nx / (double)D, cy = (double)Ny / (double)D;
  const double r = sqrt(cx * cx + cy * cy) + 1.0;
  bx0 = (int)fmax(0.0, floor(sx + cx - r));
  bx1 = (int)fmin(n - 1.0, ceil(sx + cx + r));
  by0 = (int)fmax(0.0, floor(sy + cy - r));
  by1 = (int)fmin(n - 1.0, ceil(sy + cy + r));
}

// The sites of the box [bx0, bx1] x [by0, by1] outside the window that lie
// in the circumcircle of the star's triangle (site, u, w), a lane per
// column, are inserted; true when there were any (the triangle is gone).
__device__ bool wbox_scan(WStar &st, const uint64_t *bits, const uint64_t *fixed, int n, int sx,
                          int sy, int ux, int uy, int wx, int wy, int x0, int x1, int y0, int y1,
                          int bx0, int bx1, int by0, int by1) {
  const long long hp = hkey(n, sx, sy), hu = hkey(n, sx + ux, sy + uy),
                  hw = hkey(n, sx + wx, sy + wy);
  const int lane = lane_id();
  bool found = false;
  for (int cx = bx0; cx <= bx1; cx += 32) {
    const int x = cx + lane;
    for (int b = by0 / kBand; b <= by1 / kBand; ++b) {
      uint64_t w = 0;
      if (x <= bx1) {
        w = free_word(bits, fixed, (size_t)b * n + x) & band_rows(b, by0, by1);
        if (x >= x0 && x <= x1) w &= ~band_rows(b, y0, y1);
      }
      uint64_t hit = 0;
      while (w) {
        const int i = __ffsll((long long)w) - 1;
        w &= w - 1ull;
        const int qx = x - sx, qy = b * kBand + i - sy;
        if ((qx == ux && qy == uy) || (qx == wx && qy == wy)) continue;
        if (in_circle(ux, uy, wx, wy, qx, qy, hp, hu, hw, hkey(n, sx + qx, sy + qy)))
          hit |= 1ull << i;
      }
      unsigned pend = __ballot_sync(kFull, hit != 0);
      while (pend) {
        const int L = __ffs(pend) - 1;
        pend &= pend - 1u;
        uint64_t hl = __shfl_sync(kFull, (unsigned long long)hit, L);
        while (hl) {
          const int i = __ffsll((long long)hl) - 1;
          hl &= hl - 1ull;
          winsert(st, n, sx, sy, cx + L - sx, b * kBand + i - sy);
          found = true;
        }
      }
    }
  }
  return found;
}

// What a search of the occupancy pyramid looks for: the sites in the
// closed circumdisc of the star's triangle (site, u, w) -- centre (Nx, Ny) /
// D relative to the site -- or, for an open angular gap from u to w
// (counter-clockwise, >= pi), the sites strictly inside its cone
// {q : u x q > 0 or q x w > 0}.
struct Probe {
  bool cone;
  int ux, uy, wx, wy;
  long long Nx, Ny, D, hp, hu, hw;
};

// Can the tile [px0, px1] x [qy0, qy1] hold a site the probe looks for?
__device__ __forceinline__ bool probe_node(const Probe &pr, int sx, int sy, int px0, int px1,
                                           int qy0, int qy1) {
  if (!pr.cone) return !clear_of(pr.Nx, pr.Ny, pr.D, px0 - sx, px1 - sx, qy0 - sy, qy1 - sy);
  // the cross products are linear: their largest value is at a corner
  long long cu = LLONG_MIN, cw = LLONG_MIN;
  for (int c = 0; c < 4; ++c) {
    const int qx = ((c & 1) ? px1 : px0) - sx, qy = ((c >> 1) ? qy1 : qy0) - sy;
    cu = max(cu, cross(pr.ux, pr.uy, qx, qy));
    cw = max(cw, cross(qx, qy, pr.wx, pr.wy));
  }
  return cu > 0 || cw > 0;
}

// Is site q (relative to the site) one the probe looks for?
__device__ __forceinline__ bool probe_site(const Probe &pr, int n, int sx, int sy, int qx,
                                           int qy) {
  if (pr.cone) return cross(pr.ux, pr.uy, qx, qy) > 0 || cross(qx, qy, pr.wx, pr.wy) > 0;
  if ((qx == pr.ux && qy == pr.uy) || (qx == pr.wx && qy == pr.wy)) return false;
  return in_circle(pr.ux, pr.uy, pr.wx, pr.wy, qx, qy, pr.hp, pr.hu, pr.hw,
                   hkey(n, sx + qx, sy + qy));
}

constexpr int kWarpsPerBlock = 4;  // k_dt_star's blocks: 128 threads
constexpr int kFrontier = 1536;    // pyramid nodes one warp's search holds
enum { kFinal = 0, kInserted = 1, kGaveUp = 2 };

// Warp-parallel search of the occupancy pyramid for the probe's sites
// outside the window.  The nodes still to test form a stack in the warp's
// shared memory (stk, sp of them already there); each step the lanes take up
// to 32 nodes from its top, and an occupied node not wholly inside the
// window that the probe can reach either puts its children on the stack or,
// as a 16 x 16 tile, has its sites tested by its lane.  As soon as a step
// finds sites, the tile nearest the site among those with any decides: for a
// disc every site of it inside the circle is inserted, for a cone the first
// one found (kInserted).  kFinal when no site is found; kGaveUp when the stack
// would overflow (the caller then widens the window instead).  Each step
// pops at least one node and pushes only lower levels, so the search ends;
// a descent adds at most 3 x 32 nodes per level, so 14 levels stay below
// kFrontier.
__device__ int wsearch(WStar &st, const Pyr &py, const uint64_t *bits, const uint64_t *fixed,
                       int n, int sx, int sy, const Probe &pr, int x0, int x1, int y0, int y1,
                       unsigned *stk, int sp) {
  const int lane = lane_id();
  while (sp > 0) {
    const int k = min(sp, 32);
    unsigned v = 0;
    if (lane < k) v = stk[sp - k + lane];
    __syncwarp();
    sp -= k;
    unsigned ch[4];
    int nch = 0, hq = 0;
    unsigned key = 0xffffffffu;  // (distance to the site, lane) of a tile with sites found
    if (lane < k) {
      const int l = (int)(v >> 28), tx = (int)((v >> 14) & 0x3fff), ty = (int)(v & 0x3fff);
      const int S = kTile << l;
      const int px0 = tx * S, px1 = min(px0 + S, n) - 1, qy0 = ty * S, qy1 = min(qy0 + S, n) - 1;
      if (py.occ[py.off[l] + ty * py.nt[l] + tx] &&
          !(px0 >= x0 && px1 <= x1 && qy0 >= y0 && qy1 <= y1) &&
          probe_node(pr, sx, sy, px0, px1, qy0, qy1)) {
        if (l > 0) {
          const int cn = py.nt[l - 1];
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int cx = 2 * tx + (c & 1), cy = 2 * ty + (c >> 1);
            if (cx < cn && cy < cn)
              ch[nch++] = ((unsigned)(l - 1) << 28) | ((unsigned)cx << 14) | (unsigned)cy;
          }
        } else {  // a tile: its sites, column by column, until one is found
          const int b = qy0 / kBand, sh = qy0 % kBand;
          bool found = false;
          for (int x = px0; x <= px1 && !found; ++x) {
            unsigned w = (unsigned)((free_word(bits, fixed, (size_t)b * n + x) >> sh) & 0xffffull);
            while (w) {
              const int i = __ffs(w) - 1;
              w &= w - 1u;
              if (probe_site(pr, n, sx, sy, x - sx, qy0 + i - sy)) {
                found = true;
                hq = pk(x - sx, qy0 + i - sy);
                break;
              }
            }
          }
          if (found) {
            const long long dx = px0 + kTile / 2 - sx, dy = qy0 + kTile / 2 - sy;
            key = (unsigned)min((dx * dx + dy * dy) >> 4, (long long)(1 << 26)) << 5 | lane;
          }
        }
      }
    }
    const unsigned best = __reduce_min_sync(kFull, key);
    if (best != 0xffffffffu) {
      const int L = (int)(best & 31u);
      const unsigned vL = __shfl_sync(kFull, v, L);
      const int qL = __shfl_sync(kFull, hq, L);
      if (pr.cone) {
        winsert(st, n, sx, sy, pdx(qL), pdy(qL));
        return kInserted;
      }
      // the disc: every site of that tile inside the circle, a lane per column
      const int tx = (int)((vL >> 14) & 0x3fff), ty = (int)(vL & 0x3fff);
      const int px0 = tx * kTile, qy0 = ty * kTile, b = qy0 / kBand, sh = qy0 % kBand;
      const int x = px0 + lane;
      unsigned hit = 0;
      if (lane < kTile && x < n) {
        unsigned w = (unsigned)((free_word(bits, fixed, (size_t)b * n + x) >> sh) & 0xffffull);
        while (w) {
          const int i = __ffs(w) - 1;
          w &= w - 1u;
          if (probe_site(pr, n, sx, sy, x - sx, qy0 + i - sy)) hit |= 1u << i;
        }
      }
      unsigned pend = __ballot_sync(kFull, hit != 0);
      while (pend) {
        const int Lc = __ffs(pend) - 1;
        pend &= pend - 1u;
        unsigned hl = __shfl_sync(kFull, hit, Lc);
        while (hl) {
          const int i = __ffs(hl) - 1;
          hl &= hl - 1u;
          winsert(st, n, sx, sy, px0 + Lc - sx, qy0 + i - sy);
        }
      }
      return kInserted;
    }
    // the children onto the stack
    int off = nch;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, off, o);
      if (lane >= o) off += y;
    }
    const int total = __shfl_sync(kFull, off, 31);
    off -= nch;
    if (sp + total > kFrontier) return kGaveUp;
    for (int c = 0; c < nch; ++c) stk[sp + off + c] = ch[c];
    __syncwarp();
    sp += total;
  }
  return kFinal;
}

// Search for the sites in the circumcircle of (site, u, w) outside the
// window, starting at the pyramid level where the disc's bounding box spans
// at most 2 x 2 nodes.
__device__ int wdisc_search(WStar &st, const Pyr &py, const uint64_t *bits, const uint64_t *fixed,
                            int n, int sx, int sy, int ux, int uy, int wx, int wy, int x0, int x1,
                            int y0, int y1, unsigned *stk) {
  Probe pr;
  pr.cone = false;
  pr.ux = ux, pr.uy = uy, pr.wx = wx, pr.wy = wy;
  const long long u2 = (long long)ux * ux + (long long)uy * uy,
                  w2 = (long long)wx * wx + (long long)wy * wy;
  pr.D = 2 * cross(ux, uy, wx, wy);
  pr.Nx = wy * u2 - uy * w2;
  pr.Ny = ux * w2 - wx * u2;
  pr.hp = hkey(n, sx, sy), pr.hu = hkey(n, sx + ux, sy + uy), pr.hw = hkey(n, sx + wx, sy + wy);
  int bx0, bx1, by0, by1;
  disc_box(pr.Nx, pr.Ny, pr.D, sx, sy, n, bx0, bx1, by0, by1);
  int l0 = 0;
  while (l0 < py.top && (((bx1 >> (4 + l0)) - (bx0 >> (4 + l0))) > 1 ||
                         ((by1 >> (4 + l0)) - (by0 >> (4 + l0))) > 1))
    ++l0;
  const int tx0 = bx0 >> (4 + l0), ty0 = by0 >> (4 + l0);
  const int ntx = (bx1 >> (4 + l0)) - tx0 + 1, nty = (by1 >> (4 + l0)) - ty0 + 1;  // <= 2 each
  const int lane = lane_id();
  if (lane < ntx * nty)
    stk[lane] = ((unsigned)l0 << 28) | ((unsigned)(tx0 + lane % ntx) << 14) |
                (unsigned)(ty0 + lane / ntx);
  __syncwarp();
  return wsearch(st, py, bits, fixed, n, sx, sy, pr, x0, x1, y0, y1, stk, ntx * nty);
}

// Search for the sites strictly inside the open gap's cone, from the root.
__device__ int wcone_search(WStar &st, const Pyr &py, const uint64_t *bits, const uint64_t *fixed,
                            int n, int sx, int sy, int ux, int uy, int wx, int wy, int x0, int x1,
                            int y0, int y1, unsigned *stk) {
  Probe pr;
  pr.cone = true;
  pr.ux = ux, pr.uy = uy, pr.wx = wx, pr.wy = wy;
  pr.Nx = pr.Ny = pr.D = pr.hp = pr.hu = pr.hw = 0;
  if (lane_id() == 0) stk[0] = (unsigned)py.top << 28;
  __syncwarp();
  return wsearch(st, py, bits, fixed, n, sx, sy, pr, x0, x1, y0, y1, stk, 1);
}

// Neighbour (k + 1) % m for the lane's entry k (lane l: k = l or l + 32).
__device__ __forceinline__ int wnext(const WStar &s, int k) {
  const int e = k + 1 < s.m ? k + 1 : 0;
  const int va = __shfl_sync(kFull, s.a, e & 31), vb = __shfl_sync(kFull, s.b, e & 31);
  return e < 32 ? va : vb;
}

// The Delaunay star of site (sx, sy), computed by a warp.  The first window
// is sized from the local site density (the 3 x 3 tiles around the site:
// half-width kWindow site spacings, which holds a regular site's neighbours
// and triangles' circles).  When kWiden or more of its triangles reach past
// it (as around irregular sites), the window doubles once before any search
// (inserting a ring costs less than searching); then the certificate
// settles the triangles exactly, and only a star of fewer than two
// neighbours doubles the window again (each time inserting just the new
// ring).  kWindow and kWiden are the fastest of a sweep on converged CVT
// sites and on uniform random ones at 4096^2 and 8192^2.  Returns false
// when the star overflowed.
constexpr float kWindow = 1.4f;
constexpr int kWiden = 1;
constexpr int kBoxCols = 96, kBoxBands = 3;  // largest disc box scanned directly
__device__ bool wsite_star(WStar &st, const uint64_t *bits, const uint64_t *fixed, int n, int sx,
                           int sy, const Pyr &py, const unsigned *tilecnt, unsigned *stk) {
  st.a = st.b = 0;
  st.m = 0;
  st.overflow = false;
  const int tx = sx / kTile, ty = sy / kTile, nt0 = py.nt[0], lane = lane_id();
  unsigned cnt = 0, tiles = 0;
  for (int j = max(ty - 1, 0); j <= min(ty + 1, nt0 - 1); ++j)
    for (int i = max(tx - 1, 0); i <= min(tx + 1, nt0 - 1); ++i) {
      cnt += tilecnt[brick_of(i, j, nt0)];
      ++tiles;
    }
  int W = (int)ceilf(kWindow * sqrtf((float)(tiles * kTile * kTile) / (float)max(cnt, 1u)));
  W = min(max(W, 4), 2 * n);
  int x0 = sx, x1 = sx, y0 = sy, y1 = sy;  // the window so far: the site
  bool first = true;
  for (;;) {
    const int nx0 = max(0, sx - W), nx1 = min(n - 1, sx + W);
    const int ny0 = max(0, sy - W), ny1 = min(n - 1, sy + W);
    wwindow(st, bits, fixed, n, sx, sy, nx0, nx1, ny0, ny1, x0, x1, y0, y1);
    x0 = nx0;
    x1 = nx1;
    y0 = ny0;
    y1 = ny1;
    if (st.overflow) return false;
    if (x0 == 0 && y0 == 0 && x1 == n - 1 && y1 == n - 1) return true;  // every site seen
    // certificate, exact: the sites inside a triangle's circumcircle or an
    // open gap's cone are inserted until there are none.  A triangle (or gap)
    // a search found final stays final while it is in the star (its circle
    // and the window do not change), so its key (u, w) is kept, one per lane,
    // and not searched again after another triangle changed the star.
    long long vkey = 0;
    int nver = 0;
    bool ok, changed;
    int rounds = 0;
    do {
      if (++rounds > (1 << 16)) {  // more insertions than any star needs: give up
        st.overflow = true;
        return false;
      }
      changed = false;
      const int m = st.m;
      ok = m >= 2;  // fewer than two neighbours: a wider window
      if (!ok) break;
      // each lane checks its two triangles against the window; the ones
      // that the window does not settle are searched one by one
      bool need_a = false, need_b = false;
      {
        const int wa = wnext(st, lane), wb = wnext(st, lane + 32);
        if (lane < m) {
          const int ux = pdx(st.a), uy = pdy(st.a), wx = pdx(wa), wy = pdy(wa);
          need_a = open_gap(ux, uy, wx, wy) ||
                   !disc_in_window(ux, uy, wx, wy, sx, sy, x0, x1, y0, y1, n);
        }
        if (lane + 32 < m) {
          const int ux = pdx(st.b), uy = pdy(st.b), wx = pdx(wb), wy = pdy(wb);
          need_b = open_gap(ux, uy, wx, wy) ||
                   !disc_in_window(ux, uy, wx, wy, sx, sy, x0, x1, y0, y1, n);
        }
      }
      unsigned pa = __ballot_sync(kFull, need_a), pb = __ballot_sync(kFull, need_b);
      if (first && rounds == 1 && __popc(pa) + __popc(pb) >= kWiden) {
        ok = false;  // an irregular neighbourhood: a wider window before searching
        break;
      }
      while (pa || pb) {
        int k;
        if (pa) {
          k = __ffs(pa) - 1;
          pa &= pa - 1u;
        } else {
          k = 31 + __ffs(pb);
          pb &= pb - 1u;
        }
        const int u = wget(st, k), w = wget(st, k + 1 < m ? k + 1 : 0);
        const int ux = pdx(u), uy = pdy(u), wx = pdx(w), wy = pdy(w);
        const long long key = ((long long)(unsigned)u << 32) | (unsigned)w;
        if (__ballot_sync(kFull, lane < nver && vkey == key)) continue;  // known final
        int res;
        if (open_gap(ux, uy, wx, wy)) {
          res = wcone_search(st, py, bits, fixed, n, sx, sy, ux, uy, wx, wy, x0, x1, y0, y1, stk);
        } else {
          // a small disc: its bounding box outside the window, column by
          // column; a large one through the occupancy pyramid
          const long long u2 = (long long)ux * ux + (long long)uy * uy,
                          w2 = (long long)wx * wx + (long long)wy * wy;
          const long long D = 2 * cross(ux, uy, wx, wy);
          int bx0, bx1, by0, by1;
          disc_box(wy * u2 - uy * w2, ux * w2 - wx * u2, D, sx, sy, n, bx0, bx1, by0, by1);
          res = bx1 - bx0 < kBoxCols && by1 / kBand - by0 / kBand < kBoxBands
                    ? (wbox_scan(st, bits, fixed, n, sx, sy, ux, uy, wx, wy, x0, x1, y0, y1, bx0,
                                 bx1, by0, by1)
                           ? kInserted
                           : kFinal)
                    : wdisc_search(st, py, bits, fixed, n, sx, sy, ux, uy, wx, wy, x0, x1, y0, y1,
                                   stk);
        }
        if (res == kGaveUp) {  // the search did not fit: a wider window instead
          ok = false;
          break;
        }
        const bool found = res == kInserted;
        if (st.overflow) return false;
        if (found) {
          changed = true;
          break;
        }
        if (nver < 32) {  // final: remembered
          if (lane == nver) vkey = key;
          ++nver;
        }
      }
    } while (changed);
    if (ok) return true;
    first = false;
    W = min(2 * W, 2 * n);
  }
}

// Sites per tile (brick order) and level 0 of the occupancy pyramid: one
// thread per (column, 64-row band).
__global__ void k_dt_tiles(const uint64_t *__restrict__ bits, const uint64_t *__restrict__ fixed,
                           int n, uint8_t *occ0, int nt0, unsigned *tcnt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nb = n / kBand;
  if (i >= (long long)nb * n) return;
  const int b = (int)(i / n), x = (int)(i % n);
  const uint64_t w = free_word(bits, fixed, (size_t)b * n + x);
  for (int q = 0; q < kBand / kTile; ++q) {
    const unsigned c = (unsigned)__popcll((w >> (q * kTile)) & 0xffffull);
    if (c) {
      const int ty = b * (kBand / kTile) + q, tx = x / kTile;
      occ0[ty * nt0 + tx] = 1;
      atomicAdd(&tcnt[brick_of(tx, ty, nt0)], c);
    }
  }
}

// Level l from level l - 1.
__global__ void k_dt_up(const uint8_t *__restrict__ lo, int nlo, uint8_t *hi, int nhi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nhi * nhi) return;
  const int x = i % nhi, y = i / nhi;
  uint8_t v = 0;
  for (int c = 0; c < 4; ++c) {
    const int cx = 2 * x + (c & 1), cy = 2 * y + (c >> 1);
    if (cx < nlo && cy < nlo) v |= lo[cy * nlo + cx];
  }
  hi[i] = v;
}

// Edge tiles first: an occupied tile with an empty tile (or the grid's edge)
// among its eight neighbours holds the sites whose stars reach far (flat
// triangles along the sites' boundary, convex-hull gaps).  Their sites are
// listed before the interior ones so the long stars start first instead of
// finishing last.  cnt2[c * ntiles + i]: the sites of brick-order tile i in
// class c (0 edge, 1 interior).
__global__ void k_dt_class(const uint8_t *__restrict__ occ0, int nt0,
                           const unsigned *__restrict__ tilecnt, unsigned *cnt2, uint8_t *cls) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt0 * nt0) return;
  const int brick = i / (kBrick * kBrick), in = i % (kBrick * kBrick);
  const int tx = (brick % (nt0 / kBrick)) * kBrick + in % kBrick;
  const int ty = (brick / (nt0 / kBrick)) * kBrick + in / kBrick;
  bool edge = false;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      const int x = tx + dx, y = ty + dy;
      edge |= x < 0 || y < 0 || x >= nt0 || y >= nt0 || !occ0[y * nt0 + x];
    }
  const unsigned c = tilecnt[i];
  cnt2[i] = edge ? c : 0u;
  cnt2[nt0 * nt0 + i] = edge ? 0u : c;
  cls[i] = edge ? 0 : 1;
}

// Per column: free sites in the bands before each band, and in the column.
// One warp per 32 columns; the band loop is unrolled so the loads overlap.
__global__ void k_dt_columns(const uint64_t *__restrict__ bits, const uint64_t *__restrict__ fixed,
                             int n, unsigned *colpre, unsigned *colcnt) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  unsigned c = 0;
#pragma unroll 8
  for (int b = 0; b < n / kBand; ++b) {
    colpre[(size_t)b * n + x] = c;
    c += __popcll(free_word(bits, fixed, (size_t)b * n + x));
  }
  colcnt[x] = c;
}

// The sites in tile order, edge tiles first: one thread per tile (brick
// order), its sites by column, then row.
__global__ void k_dt_order(const uint64_t *__restrict__ bits, const uint64_t *__restrict__ fixed,
                           int n, int nt0, const unsigned *__restrict__ toff,
                           const uint8_t *__restrict__ cls, int *order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt0 * nt0) return;
  const int brick = i / (kBrick * kBrick), in = i % (kBrick * kBrick);
  const int tx = (brick % (nt0 / kBrick)) * kBrick + in % kBrick;
  const int ty = (brick / (nt0 / kBrick)) * kBrick + in / kBrick;
  const int y0 = ty * kTile, b = y0 / kBand, sh = y0 % kBand;
  unsigned pos = toff[(size_t)cls[i] * nt0 * nt0 + i];
  for (int x = tx * kTile; x < tx * kTile + kTile; ++x) {
    uint64_t w = (free_word(bits, fixed, (size_t)b * n + x) >> sh) & 0xffffull;
    while (w) {
      const int k = __ffsll((long long)w) - 1;
      w &= w - 1ull;
      order[pos++] = pk(x, y0 + k);
    }
  }
}

__device__ __forceinline__ int site_index(const uint64_t *bits, const uint64_t *fixed, int n,
                                          const unsigned *coloff, const unsigned *colpre, int x,
                                          int y) {
  const int b = y / kBand, i = y % kBand;
  const uint64_t w = free_word(bits, fixed, (size_t)b * n + x);
  const uint64_t below = i ? (w & ((1ull << i) - 1ull)) : 0ull;
  return (int)(coloff[x] + colpre[(size_t)b * n + x] + (unsigned)__popcll(below));
}

// The star of the t-th site in tile order (one warp per site), stored
// under its index in delaunayInput's order with the number of triangles it
// writes.
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_dt_star(const uint64_t *__restrict__ bits, const uint64_t *__restrict__ fixed, int n,
              const int *__restrict__ order, int nsites, Pyr py,
              const unsigned *__restrict__ coloff, const unsigned *__restrict__ colpre,
              const unsigned *__restrict__ tilecnt, int *sitepos, int *stars, int *degree,
              unsigned *tcount, int *err) {
  const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= nsites) return;  // the whole warp
  const int lane = lane_id();
  const int sx = pdx(order[t]) & 0xffff, sy = pdy(order[t]);
  const int xm = site_index(bits, fixed, n, coloff, colpre, sx, sy);
  __shared__ unsigned s_front[kWarpsPerBlock][kFrontier];
  WStar st;
  if (!wsite_star(st, bits, fixed, n, sx, sy, py, tilecnt, s_front[threadIdx.x >> 5])) {
    if (lane == 0) {
      atomicOr(err, 1);
      sitepos[xm] = order[t];
      degree[xm] = 0;
      tcount[xm] = 0;
    }
    return;
  }
  const int m = st.m;
  int *row = stars + (size_t)xm * kStar;
  if (lane < m) row[lane] = st.a;
  if (lane + 32 < m) row[lane + 32] = st.b;
  // triangles (k, k + 1) this site writes: the one of its vertices first in
  // (x, y) order
  auto owns = [&](int u, int w) {
    if (m < 2 || open_gap(pdx(u), pdy(u), pdx(w), pdy(w))) return false;
    const int ux = sx + pdx(u), uy = sy + pdy(u), wx = sx + pdx(w), wy = sy + pdy(w);
    return (sx < ux || (sx == ux && sy < uy)) && (sx < wx || (sx == wx && sy < wy));
  };
  const int wa = wnext(st, lane), wb = wnext(st, lane + 32);
  const bool oa = lane < m && owns(st.a, wa), ob = lane + 32 < m && owns(st.b, wb);
  const int own = __popc(__ballot_sync(kFull, oa)) + __popc(__ballot_sync(kFull, ob));
  if (lane == 0) {
    sitepos[xm] = order[t];
    degree[xm] = m;
    tcount[xm] = own;
  }
}

__global__ void k_dt_emit(const uint64_t *__restrict__ bits, const uint64_t *__restrict__ fixed,
                          int n, const int *__restrict__ sitepos, int nsites,
                          const unsigned *__restrict__ coloff, const unsigned *__restrict__ colpre,
                          const int *__restrict__ stars, const int *__restrict__ degree,
                          const unsigned *__restrict__ toff, int *tris, unsigned cap) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsites) return;
  const int sx = pdx(sitepos[t]) & 0xffff, sy = pdy(sitepos[t]);
  const int m = degree[t];
  unsigned pos = toff[t];
  for (int k = 0; k < m; ++k) {
    const int u = stars[(size_t)t * kStar + k], w = stars[(size_t)t * kStar + (k + 1) % m];
    if (m < 2 || open_gap(pdx(u), pdy(u), pdx(w), pdy(w))) continue;
    const int ux = sx + pdx(u), uy = sy + pdy(u), wx = sx + pdx(w), wy = sy + pdy(w);
    const bool first = (sx < ux || (sx == ux && sy < uy)) && (sx < wx || (sx == wx && sy < wy));
    if (!first) continue;
    if (pos < cap) {
      tris[3 * (size_t)pos] = t;
      tris[3 * (size_t)pos + 1] = site_index(bits, fixed, n, coloff, colpre, ux, uy);
      tris[3 * (size_t)pos + 2] = site_index(bits, fixed, n, coloff, colpre, wx, wy);
    }
    ++pos;
  }
}

// Exclusive scan of large count arrays: blocks of 4096 counts scanned in
// shared memory, the block totals by launch_scan, then the block offsets
// added (offset[n] = total).
constexpr int kScanBlock = 4096;
__global__ void __launch_bounds__(1024) k_scan_local(const unsigned *__restrict__ count, int n,
                                                     unsigned *offset, unsigned *total) {
  __shared__ unsigned v[kScanBlock];
  __shared__ unsigned wsum[32];
  const int base = blockIdx.x * kScanBlock, t = threadIdx.x;
  for (int k = t; k < kScanBlock; k += 1024) v[k] = base + k < n ? count[base + k] : 0u;
  __syncthreads();
  const unsigned a0 = v[4 * t], a1 = v[4 * t + 1], a2 = v[4 * t + 2], a3 = v[4 * t + 3];
  const unsigned sum = a0 + a1 + a2 + a3;
  unsigned inc = sum;  // inclusive scan over the warp
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
    if ((t & 31) >= o) inc += y;
  }
  if ((t & 31) == 31) wsum[t >> 5] = inc;
  __syncthreads();
  if (t < 32) {
    unsigned w = wsum[t], wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, wi, o);
      if (t >= o) wi += y;
    }
    wsum[t] = wi - w;
    if (t == 31) total[blockIdx.x] = wi;
  }
  __syncthreads();
  const unsigned ex = wsum[t >> 5] + inc - sum;
  v[4 * t] = ex;
  v[4 * t + 1] = ex + a0;
  v[4 * t + 2] = ex + a0 + a1;
  v[4 * t + 3] = ex + a0 + a1 + a2;
  __syncthreads();
  for (int k = t; k < kScanBlock; k += 1024)
    if (base + k < n) offset[base + k] = v[k];
}

__global__ void k_scan_add(unsigned *offset, int n, const unsigned *__restrict__ boff, int nblock) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) offset[i] += boff[i / kScanBlock];
  if (i == 0) offset[n] = boff[nblock];
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

#define DCK(call)                                 \
  do {                                            \
    if ((call) != cudaSuccess) return GCVT_ERR_CUDA; \
  } while (0)

// Exclusive scan of count[0..n) into offset[0..n] (n >= 1).
int scan_big(const unsigned *count, int n, unsigned *offset, Scratch &sc, cudaStream_t s) {
  const int nblock = (n + kScanBlock - 1) / kScanBlock;
  unsigned *tot = sc.take<unsigned>(nblock), *boff = sc.take<unsigned>(nblock + 1),
           *cur = sc.take<unsigned>(nblock);
  if (!tot || !boff || !cur) return GCVT_ERR_ALLOC;
  k_scan_local<<<nblock, 1024, 0, s>>>(count, n, offset, tot);
  DCK(cudaGetLastError());
  DCK(launch_scan(reinterpret_cast<const int *>(tot), nblock, reinterpret_cast<int *>(boff),
                  reinterpret_cast<int *>(cur), s));
  k_scan_add<<<nblk(n, 256), 256, 0, s>>>(offset, n, boff, nblock);
  DCK(cudaGetLastError());
  return GCVT_OK;
}

}  // namespace

// The Delaunay triangles of the free sites of `bits` (n x n, n a multiple of
// 64), as indices into delaunayInput's point order; host-synchronous on `s`.
int delaunay_sites(const uint64_t *bits, const uint64_t *fixed, int n, int *tris, unsigned cap,
                   unsigned *ntris, cudaStream_t s) {
  Scratch sc(s);
  return delaunay_sites_in(bits, fixed, n, tris, cap, ntris, s, sc);
}

// The same with the caller's scratch (a caller that holds one already: the
// device's scratch lock is not taken twice).
int delaunay_sites_in(const uint64_t *bits, const uint64_t *fixed, int n, int *tris,
                      unsigned cap, unsigned *ntris, cudaStream_t s, Scratch &sc) {
  *ntris = 0;
  if (n <= 0 || n % kBand) return GCVT_ERR_ARGUMENT;
  const size_t nb = (size_t)(n / kBand) * n;
  const int nt0 = n / kTile, ntiles = nt0 * nt0;
  unsigned *colpre = sc.take<unsigned>(nb), *colcnt = sc.take<unsigned>(n),
           *coloff = sc.take<unsigned>(n + 1), *cur = sc.take<unsigned>(n),
           *tilecnt = sc.take<unsigned>(ntiles), *cnt2 = sc.take<unsigned>(2 * (size_t)ntiles),
           *tileoff = sc.take<unsigned>(2 * (size_t)ntiles + 1);
  uint8_t *cls = sc.take<uint8_t>(ntiles);
  int *err = sc.take<int>(1);
  Pyr py{};
  size_t occ_bytes = 0;
  for (int l = 0, t = nt0;; ++l, t = (t + 1) / 2) {
    if (l >= kLevels) return GCVT_ERR_ARGUMENT;
    py.off[l] = (int)occ_bytes;
    py.nt[l] = t;
    occ_bytes += (size_t)t * t;
    if (t == 1) {
      py.top = l;
      break;
    }
  }
  uint8_t *occ = sc.take<uint8_t>(occ_bytes);
  py.occ = occ;
  if (!colpre || !colcnt || !coloff || !cur || !tilecnt || !cnt2 || !tileoff || !cls || !err ||
      !occ)
    return GCVT_ERR_ALLOC;
  DCK(cudaMemsetAsync(err, 0, sizeof(int), s));
  DCK(cudaMemsetAsync(occ, 0, occ_bytes, s));
  DCK(cudaMemsetAsync(tilecnt, 0, (size_t)ntiles * sizeof(unsigned), s));
  k_dt_columns<<<nblk(n, 64), 64, 0, s>>>(bits, fixed, n, colpre, colcnt);
  DCK(cudaGetLastError());
  k_dt_tiles<<<nblk((long long)nb, 256), 256, 0, s>>>(bits, fixed, n, occ, nt0, tilecnt);
  DCK(cudaGetLastError());
  for (int l = 1; l <= py.top; ++l) {
    k_dt_up<<<nblk((long long)py.nt[l] * py.nt[l], 256), 256, 0, s>>>(
        occ + py.off[l - 1], py.nt[l - 1], occ + py.off[l], py.nt[l]);
    DCK(cudaGetLastError());
  }
  DCK(launch_scan(reinterpret_cast<const int *>(colcnt), n, reinterpret_cast<int *>(coloff),
                  reinterpret_cast<int *>(cur), s));
  k_dt_class<<<nblk(ntiles, 256), 256, 0, s>>>(occ, nt0, tilecnt, cnt2, cls);
  DCK(cudaGetLastError());
  int rc = scan_big(cnt2, 2 * ntiles, tileoff, sc, s);
  if (rc) return rc;
  unsigned nsites_u = 0;
  DCK(cudaMemcpyAsync(&nsites_u, coloff + n, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  DCK(cudaStreamSynchronize(s));
  const int nsites = (int)nsites_u;
  if (nsites < 3) return GCVT_OK;
  int *order = sc.take<int>(nsites), *sitepos = sc.take<int>(nsites),
      *stars = sc.take<int>((size_t)nsites * kStar), *degree = sc.take<int>(nsites);
  unsigned *tcnt = sc.take<unsigned>(nsites), *toff = sc.take<unsigned>(nsites + 1);
  if (!order || !sitepos || !stars || !degree || !tcnt || !toff) return GCVT_ERR_ALLOC;
  k_dt_order<<<nblk(ntiles, 128), 128, 0, s>>>(bits, fixed, n, nt0, tileoff, cls, order);
  DCK(cudaGetLastError());
  k_dt_star<<<nblk(32ll * nsites, 32 * kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
      bits, fixed, n, order, nsites, py, coloff, colpre, tilecnt, sitepos, stars, degree, tcnt,
      err);
  DCK(cudaGetLastError());
  if ((rc = scan_big(tcnt, nsites, toff, sc, s))) return rc;
  if (tris && cap) {
    k_dt_emit<<<nblk(nsites, 128), 128, 0, s>>>(bits, fixed, n, sitepos, nsites, coloff, colpre,
                                                stars, degree, toff, tris, cap);
    DCK(cudaGetLastError());
  }
  unsigned h[2] = {0, 0};
  DCK(cudaMemcpyAsync(&h[0], toff + nsites, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  DCK(cudaMemcpyAsync(&h[1], err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  DCK(cudaStreamSynchronize(s));
  if (h[1]) return GCVT_ERR_INPUT;
  *ntris = h[0];
  return GCVT_OK;
}

}  // namespace cvtgb
