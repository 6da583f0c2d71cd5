// cdt.cu -- the constrained Delaunay triangulation of the CDT stage on the
// GPU: the reference hands gDel2D (gDel2D/GPU/GpuDelaunay.cu:46) the free
// sites and the constraint points (delaunay.h:46-67) with the constraint
// segments between those points (delaunay.h:69-75), and gDel2D triangulates
// them and then inserts the segments by flips (GpuDelaunay.cu:749,
// splitAndFlip).  Here:
//
//   1. the sites' Delaunay triangulation (delaunay.cu, exact on the lattice);
//   2. adjacency from a hash of directed edges;
//   3. the constraint points inserted in rounds: every point locates itself
//      by a walk, claims the triangles its split changes (atomicMin of a
//      priority, a fixed bijective hash of its index: claims by plain index
//      let only the first of a run of neighbours win each round), and the
//      points that won all their claims split (1 -> 3 inside a triangle,
//      2 -> 4 on an edge, a fan over the visible hull edges outside the
//      hull); after each round, two flip rounds over the changed triangles
//      (two rounds with their flips make one CUDA graph and one read-back);
//   4. each segment made an edge by flipping the edges that cross it
//      (Sloan's method, cdt_core.cuh recover_segment) and marked: segments
//      already edges at once, the others in rounds where each claims the
//      triangles around the vertices of its crossing edges and the winners
//      are recovered side by side, the rare long ones (or ones with a vertex
//      inside) by one thread;
//   5. flip rounds that restore the Delaunay property on every edge that is
//      not a constraint: the result is the constrained Delaunay
//      triangulation;
//   6. the triangles written in a fixed order (by their smallest vertex, then
//      the next one), so the output does not depend on scheduling.
//
// A flip round: every changed triangle tests its edges towards
// higher-numbered neighbours (cdt_core.cuh wants_flip); a flip claims its two
// triangles and their four outer neighbours (whose back links it rewrites);
// the flips that won all six claims are applied.  Lawson's flips end (each
// one lowers the lifted surface), so the rounds end; a round limit turns a
// runaway into an error instead of a hang.
//
// Coordinates: sites (x, y) on the pixel lattice scaled by 2^15; a
// constraint point (px, py) maps to ((px - left) / scale, (py - lower) /
// scale) pixels, rounded to the nearest 2^-15 pixel -- the same frame as
// delaunayInput's (x * scale + left, y * scale + lower) for the sites.  All
// predicates are then exact integers (cdt_core.cuh).  Symbolic perturbation
// ranks: a site ranks y n + x (as in the sites' triangulation), constraint
// point j ranks n^2 + j.
#include "gcvt_internal.cuh"
#include "cdt_core.cuh"
#include "../../include/gcvt_gb300.h"

#include <cmath>
#include <utility>

namespace cvtgb {

using cdt::i64;
using cdt::Mesh;

namespace {

constexpr int kWalk = 1 << 20;    // steps of one point location
constexpr int kRotate = 4096;     // triangles around one vertex
constexpr int kChain = 64;        // visible hull edges from one outside point
constexpr int kFlipRounds = 1 << 16;
constexpr int kFlipPoll = 4;      // flip rounds between read-backs
constexpr int kInterimFlips = 2;  // flip rounds after each insertion round
constexpr int kFlipBlocks = 304;  // grid of the grid-stride flip kernels (2 per SM)
constexpr int kInsertRounds = 1 << 12;
constexpr int kSegQueue = 4096;   // crossing edges of one segment
constexpr int kSegStack = 256;    // pieces of one segment split by vertices inside it
constexpr int kCorr = 8;          // crossing edges of a segment recovered in the parallel rounds
constexpr int kClaim = 128;       // triangles one such segment claims
constexpr int kSegWindow = 1 << 15;  // segments per window of parallel rounds
constexpr int kSegRounds = 1 << 12;

enum CdtErr {
  kErrCoord = 1,       // a constraint point beyond the supported coordinate range
  kErrDuplicate = 2,   // a constraint point on a site or another constraint point
  kErrWalk = 4,        // a location, rotation or chain bound ran out
  kErrHash = 8,        // the edge table is inconsistent or full
  kErrSegment = 16,    // a vertex inside a segment, crossing segments, a bad index pair
  kErrSegLimit = 32,   // a segment's recovery ran out of its bounds
  kErrCapacity = 64    // more triangles than the mesh holds
};

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

#define CCK(call)                                   \
  do {                                              \
    if ((call) != cudaSuccess) return GCVT_ERR_CUDA; \
  } while (0)

// ---- coordinates ---------------------------------------------------------

__global__ void k_cdt_coords(const double *__restrict__ sxy, int F, const double *__restrict__ cxy,
                             int C, double scale, double left, double lower, int n, i64 *X,
                             i64 *Y, i64 *R, int *err) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= F + C) return;
  if (v < F) {
    const i64 x = (i64)sxy[2 * (size_t)v], y = (i64)sxy[2 * (size_t)v + 1];
    X[v] = x << 15;
    Y[v] = y << 15;
    R[v] = y * n + x;
    return;
  }
  const int j = v - F;
  const double u = (cxy[2 * j] - left) / scale * 32768.0,
               w = (cxy[2 * j + 1] - lower) / scale * 32768.0;
  const double lim = 536870912.0;  // 2^29
  if (!(fabs(u) < lim) || !(fabs(w) < lim)) {
    atomicOr(err, kErrCoord);
    X[v] = Y[v] = 0;
  } else {
    X[v] = llrint(u);
    Y[v] = llrint(w);
  }
  R[v] = (i64)n * n + j;
}

// ---- adjacency ------------------------------------------------------------

__device__ __forceinline__ unsigned long long ekey(int u, int w) {
  return ((unsigned long long)(unsigned)u << 32) | (unsigned)w;
}
__device__ __forceinline__ unsigned ehash(unsigned long long k, unsigned mask) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (unsigned)k & mask;
}

__global__ void k_edge_insert(const int *__restrict__ tri, int T, unsigned long long *hk, int *hv,
                              unsigned mask, int *err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * T) return;
  const int t = e / 3, i = e % 3;
  const int u = tri[3 * t + cdt::nx3(i)], w = tri[3 * t + cdt::pv3(i)];
  const unsigned long long k = ekey(u, w);
  unsigned h = ehash(k, mask);
  for (unsigned s = 0; s <= mask; ++s, h = (h + 1) & mask) {
    const unsigned long long old = atomicCAS(hk + h, ~0ull, k);
    if (old == ~0ull) {
      hv[h] = cdt::pack_nb(t, i);
      return;
    }
    if (old == k) break;  // a directed edge twice
  }
  atomicOr(err, kErrHash);
}

__global__ void k_edge_link(const int *__restrict__ tri, int T, const unsigned long long *hk,
                            const int *hv, unsigned mask, int *nbr, int *vt, int *err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * T) return;
  const int t = e / 3, i = e % 3;
  const int u = tri[3 * t + cdt::nx3(i)], w = tri[3 * t + cdt::pv3(i)];
  if (i == 0) vt[tri[3 * t]] = t;
  if (i == 1) vt[tri[3 * t + 1]] = t;
  if (i == 2) vt[tri[3 * t + 2]] = t;
  const unsigned long long k = ekey(w, u);
  unsigned h = ehash(k, mask);
  int nb = cdt::kNone;
  for (unsigned s = 0; s <= mask; ++s, h = (h + 1) & mask) {
    const unsigned long long cur = hk[h];
    if (cur == k) {
      nb = hv[h];
      break;
    }
    if (cur == ~0ull) break;
  }
  nbr[3 * t + i] = nb;
}

// ---- constraint point insertion --------------------------------------------

// Where a pending point lies, and (outside the hull) the hull edges it sees
// in counter-clockwise order with the hull triangles just before and after
// them -- recorded while nothing changes, so the insertion never walks a
// mesh that other points are changing.
struct Loc {
  int kind, t, i;
  int cnt, before, after;
  int et[kChain], ei[kChain];
};

// Claims hold priorities (cdt_core.cuh prio): the smallest wins.
__device__ __forceinline__ void claim(unsigned *cl, int t, unsigned pr) { atomicMin(cl + t, pr); }
__device__ __forceinline__ void claim_nbrs(const Mesh &m, unsigned *cl, int t, unsigned pr) {
  claim(cl, t, pr);
  for (int i = 0; i < 3; ++i) {
    const int nb = m.nbr[3 * t + i];
    if (nb >= 0) claim(cl, cdt::nb_tri(nb), pr);
  }
}

// Locate every pending point and claim what its insertion changes.
__global__ void k_ins_locate(Mesh m, const int *__restrict__ pend, const int *npp, int *start,
                             Loc *loc, unsigned *cl, int *err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= *npp) return;
  const int p = pend[q];
  const unsigned pr = cdt::prio((unsigned)p);
  Loc L;
  L.kind = cdt::locate(m, p, start[q], kWalk, &L.t, &L.i);
  L.cnt = 0;
  if (L.kind == cdt::kLocFail) {
    atomicOr(err, kErrWalk);
  } else if (L.kind == cdt::kLocVertex) {
    atomicOr(err, kErrDuplicate);
  } else if (L.kind == cdt::kLocIn) {
    claim_nbrs(m, cl, L.t, pr);
  } else if (L.kind == cdt::kLocEdge) {
    claim_nbrs(m, cl, L.t, pr);
    const int nb = m.nbr[3 * L.t + L.i];
    if (nb >= 0) claim_nbrs(m, cl, cdt::nb_tri(nb), pr);
  } else {  // outside: the visible hull edges around the exit edge
    int ft = L.t, fi = L.i, back = 0, ok = 1;
    int bt[kChain], bi[kChain];  // the edges before the exit edge, nearest first
    L.before = L.after = -1;
    for (;;) {
      int pt, pi;
      if (!cdt::hull_prev(m, ft, fi, kRotate, &pt, &pi)) {
        ok = 0;
        break;
      }
      if (cdt::orient(m, m.tri[3 * pt + cdt::nx3(pi)], m.tri[3 * pt + cdt::pv3(pi)], p) >= 0) {
        L.before = pt;
        break;
      }
      if (back + 1 >= kChain) {
        ok = 0;
        break;
      }
      bt[back] = ft = pt;
      bi[back] = fi = pi;
      ++back;
    }
    int cnt = 0;
    if (ok) {
      for (int k = back - 1; k >= 0; --k, ++cnt) {
        L.et[cnt] = bt[k];
        L.ei[cnt] = bi[k];
      }
      L.et[cnt] = L.t;
      L.ei[cnt] = L.i;
      ++cnt;
      int lt = L.t, li = L.i;
      for (;;) {
        int nt, ni;
        if (!cdt::hull_next(m, lt, li, kRotate, &nt, &ni)) {
          ok = 0;
          break;
        }
        if (cdt::orient(m, m.tri[3 * nt + cdt::nx3(ni)], m.tri[3 * nt + cdt::pv3(ni)], p) >= 0) {
          L.after = nt;
          break;
        }
        if (cnt >= kChain) {
          ok = 0;
          break;
        }
        L.et[cnt] = lt = nt;
        L.ei[cnt] = li = ni;
        ++cnt;
      }
    }
    if (!ok) {
      atomicOr(err, kErrWalk);
      L.kind = cdt::kLocFail;
    } else {
      // claim the chain and the hull edges just before and after it, so that
      // two points never extend the hull next to each other in one round
      L.cnt = cnt;
      for (int k = 0; k < cnt; ++k) claim(cl, L.et[k], pr);
      if (L.before >= 0) claim(cl, L.before, pr);
      if (L.after >= 0) claim(cl, L.after, pr);
    }
  }
  loc[q] = L;
}

__device__ __forceinline__ bool owns(const Mesh &m, const unsigned *cl, int t, unsigned pr) {
  return cl[t] == pr;
}
__device__ bool owns_nbrs(const Mesh &m, const unsigned *cl, int t, unsigned pr) {
  if (!owns(m, cl, t, pr)) return false;
  for (int i = 0; i < 3; ++i) {
    const int nb = m.nbr[3 * t + i];
    if (nb >= 0 && !owns(m, cl, cdt::nb_tri(nb), pr)) return false;
  }
  return true;
}

// Triangle t changed: it and its neighbours are tested by the next flip
// round.  An edge whose opposite vertices changed belongs to a changed
// triangle, so it is tested from whichever of its triangles has the smaller
// index (k_flip_mark).
__device__ __forceinline__ void touch(const Mesh &m, uint8_t *act, int t) {
  act[t] = 1;
  for (int i = 0; i < 3; ++i) {
    const int nb = m.nbr[3 * t + i];
    if (nb >= 0) act[cdt::nb_tri(nb)] = 1;
  }
}

// Insert the points that won every claim; the others stay pending (their
// walk starts next round from the triangle they reached).
__global__ void k_ins_apply(Mesh m, const int *__restrict__ pend, const int *npp, int *start,
                            const Loc *__restrict__ loc, const unsigned *cl, int *ntri, int cap,
                            int *done, uint8_t *act, int *err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= *npp) return;
  const int p = pend[q];
  const unsigned pr = cdt::prio((unsigned)p);
  const Loc &L = loc[q];
  if (L.kind == cdt::kLocFail || L.kind == cdt::kLocVertex) return;
  start[q] = L.t;
  if (L.kind == cdt::kLocIn) {
    if (!owns_nbrs(m, cl, L.t, pr)) return;
    const int s = atomicAdd(ntri, 2);
    if (s + 2 > cap) {
      atomicOr(err, kErrCapacity);
      return;
    }
    cdt::split_in(m, L.t, p, s, s + 1);
    touch(m, act, L.t);
    touch(m, act, s);
    touch(m, act, s + 1);
  } else if (L.kind == cdt::kLocEdge) {
    if (!owns_nbrs(m, cl, L.t, pr)) return;
    const int nb = m.nbr[3 * L.t + L.i];
    if (nb >= 0 && !owns_nbrs(m, cl, cdt::nb_tri(nb), pr)) return;
    const int k = nb >= 0 ? 2 : 1;
    const int s = atomicAdd(ntri, k);
    if (s + k > cap) {
      atomicOr(err, kErrCapacity);
      return;
    }
    cdt::split_edge(m, L.t, L.i, p, s, s + 1);
    touch(m, act, L.t);
    touch(m, act, s);
    if (nb >= 0) {
      touch(m, act, cdt::nb_tri(nb));
      touch(m, act, s + 1);
    }
  } else {
    bool won = (L.before < 0 || owns(m, cl, L.before, pr)) && (L.after < 0 || owns(m, cl, L.after, pr));
    for (int k = 0; k < L.cnt && won; ++k) won = owns(m, cl, L.et[k], pr);
    if (!won) return;
    const int s = atomicAdd(ntri, L.cnt);
    if (s + L.cnt > cap) {
      atomicOr(err, kErrCapacity);
      return;
    }
    int slots[kChain];
    for (int k = 0; k < L.cnt; ++k) slots[k] = s + k;
    cdt::insert_out(m, L.et, L.ei, L.cnt, p, slots);
    for (int k = 0; k < L.cnt; ++k) touch(m, act, slots[k]);
    start[q] = s;
  }
  done[q] = 1;
}

// ---- flips ---------------------------------------------------------------

// Each changed triangle (act) of the *ntri in the mesh: the first of its
// edges towards a higher-numbered neighbour that wants a flip; the flip
// claims both triangles and the four outer neighbours with the priority of
// 3 t + i.  A triangle with none is settled until a change touches it again.
__device__ __forceinline__ void flip_mark_one(const Mesh &m, int t, int *cand, unsigned *cl,
                                              uint8_t *act, int *found) {
  if (!act[t]) {
    cand[t] = 0;
    return;
  }
  int c = 0;
  for (int i = 0; i < 3; ++i) {
    const int nb = m.nbr[3 * t + i];
    if (nb < 0 || cdt::nb_tri(nb) < t) continue;
    if (cdt::wants_flip(m, t, i)) {
      c = i + 1;
      break;
    }
  }
  cand[t] = c;
  if (!c) {
    act[t] = 0;
    return;
  }
  atomicAdd(found, 1);
  const int i = c - 1;
  const unsigned pr = cdt::prio((unsigned)(3 * t + i));
  const int t2 = cdt::nb_tri(m.nbr[3 * t + i]);
  claim_nbrs(m, cl, t, pr);
  claim_nbrs(m, cl, t2, pr);
}

// (grid-stride: a round with few changed triangles costs few blocks)
__global__ void k_flip_mark(Mesh m, const int *ntri, int *cand, unsigned *cl, uint8_t *act,
                            int *found) {
  const int T = *ntri;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
    flip_mark_one(m, t, cand, cl, act, found);
}

__global__ void k_flip_apply(Mesh m, const int *ntri, const int *cand, const unsigned *cl,
                             uint8_t *act, int *flips) {
  const int T = *ntri;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
    if (!cand[t]) continue;
    const int i = cand[t] - 1;
    const unsigned pr = cdt::prio((unsigned)(3 * t + i));
    const int t2 = cdt::nb_tri(m.nbr[3 * t + i]);
    if (!owns_nbrs(m, cl, t, pr) || !owns_nbrs(m, cl, t2, pr)) continue;
    cdt::flip(m, t, i);
    touch(m, act, t);
    touch(m, act, t2);
    atomicAdd(flips, 1);
  }
}

// ---- segments --------------------------------------------------------------

enum SegState { kSegPending = 0, kSegDone = 1, kSegSerial = 2 };

// Segments that are already edges are marked at once (atomic bit sets, the
// mesh is otherwise read-only here); the others wait for the rounds.  Bad
// index pairs set err.
__global__ void k_seg_mark(Mesh m, const int *__restrict__ segs, int S, int V, int *state,
                           int *err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S) return;
  const int a = segs[2 * k], b = segs[2 * k + 1];
  if (a < 0 || b < 0 || a >= V || b >= V || a == b) {
    atomicOr(err, kErrSegment);
    state[k] = kSegDone;
    return;
  }
  state[k] = cdt::mark_constraint(m, a, b, kRotate) ? kSegDone : kSegPending;
}

// A pending segment of the window [base, base + W) claims, with its priority,
// the triangles around its ends and around every end of the edges crossing
// it: all that its recovery reads or writes (Sloan's flips stay inside the
// triangles the segment crosses, whose vertices are those ends, and rewrite
// the back links of their neighbours, which lie around the same vertices).
// The claimed triangles are listed for the apply pass.  A segment that meets
// a vertex or a constraint, or crosses more than kCorr edges, goes to the
// one-thread pass.
__global__ void k_seg_locate(Mesh m, const int *__restrict__ segs, int base, int W, int *state,
                             int *list, int *lcnt, unsigned *cl) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  const int k = base + w;
  if (state[k] != kSegPending) return;
  const int a = segs[2 * k], b = segs[2 * k + 1];
  int q[2 * kCorr], on = -1, cnt = 0;
  if (cdt::collect_crossings(m, a, b, q, kCorr, kWalk, &on, &cnt) != cdt::kSegOk) {
    state[k] = kSegSerial;
    return;
  }
  int *L = list + (size_t)w * kClaim;
  int n = 0;
  for (int e = -2; e < 2 * cnt; ++e) {
    const int v = e == -2 ? a : (e == -1 ? b : q[e]);
    bool seen = false;
    for (int f = -2; f < e && !seen; ++f) seen = (f == -2 ? a : (f == -1 ? b : q[f])) == v;
    if (seen) continue;
    const int c = cdt::fan(m, v, kRotate, L + n, kClaim - n);
    if (c < 0) {
      state[k] = kSegSerial;
      return;
    }
    n += c;
  }
  const unsigned pr = cdt::prio((unsigned)k);
  for (int i = 0; i < n; ++i) claim(cl, L[i], pr);
  lcnt[w] = n;
}

// The segments that won every claim are recovered (cdt_core.cuh
// recover_segment); the others count themselves pending for the next round.
__global__ void k_seg_apply(Mesh m, const int *__restrict__ segs, int base, int W, int *state,
                            const int *__restrict__ list, const int *__restrict__ lcnt,
                            const unsigned *cl, int *pending, int *err) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  const int k = base + w;
  if (state[k] != kSegPending) return;
  const int *L = list + (size_t)w * kClaim;
  const unsigned pr = cdt::prio((unsigned)k);
  for (int i = 0, n = lcnt[w]; i < n; ++i)
    if (cl[L[i]] != pr) {
      atomicAdd(pending, 1);
      return;
    }
  int q[2 * kCorr], on = -1;
  const int r = cdt::recover_segment(m, segs[2 * k], segs[2 * k + 1], q, kCorr, kWalk, &on);
  if (r == cdt::kSegCrosses) atomicOr(err, kErrSegment);
  else if (r != cdt::kSegOk) atomicOr(err, kErrSegLimit);
  state[k] = kSegDone;
}

// The segments left to one thread, one after the other (they may share
// crossing edges): long ones, and those with vertices inside them, which
// become the chain of edges between those vertices (as constrained Delaunay
// triangulations split such segments).  Crossing segments set err.
__global__ void k_segments(Mesh m, const int *__restrict__ segs, int S, const int *state,
                           int *queue, int *stack, int *err) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int k = 0; k < S; ++k) {
    if (state[k] == kSegDone) continue;
    const int a = segs[2 * k], b = segs[2 * k + 1];
    const int r = cdt::recover_chain(m, a, b, queue, kSegQueue, stack, kSegStack, kWalk);
    if (r == cdt::kSegCrosses) atomicOr(err, kErrSegment);
    else if (r != cdt::kSegOk) atomicOr(err, kErrSegLimit);
  }
}

// ---- output ----------------------------------------------------------------

__global__ void k_emit_count(Mesh m, int T, int *cnt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int a, b, c;
  cdt::canon(m.tri + 3 * t, a, b, c);
  atomicAdd(cnt + a, 1);
}

// Triangle t at its owner's offset plus its rank among the owner's
// triangles (cdt_core.cuh owner_rank).
__global__ void k_emit(Mesh m, int T, const int *__restrict__ off, int *out, int cap, int *err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int a, b, c;
  cdt::canon(m.tri + 3 * t, a, b, c);
  const int rank = cdt::owner_rank(m, t, kRotate);
  if (rank < 0) {
    atomicOr(err, kErrWalk);
    return;
  }
  const int pos = off[a] + rank;
  if (pos < cap) {
    out[3 * (size_t)pos] = a;
    out[3 * (size_t)pos + 1] = b;
    out[3 * (size_t)pos + 2] = c;
  }
}

// Start triangles of the constraint points: a site near each (the first
// found in growing squares around its pixel in the site index grid), or any
// triangle.
__global__ void k_ins_start(const i64 *__restrict__ X, const i64 *__restrict__ Y, int F, int C,
                            const int *__restrict__ site_at, int n, const int *vt, int *start) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= C) return;
  const int px = (int)(X[F + j] >> 15), py = (int)(Y[F + j] >> 15);
  int found = -1;
  for (int r = 0; r < 64 && found < 0; ++r) {
    // the ring at Chebyshev distance r: its 8 r cells (1 for r = 0), side by side
    const int cells = r ? 8 * r : 1;
    for (int k = 0; k < cells; ++k) {
      int dx, dy;
      if (r == 0) dx = dy = 0;
      else if (k < 2 * r) dx = -r + k, dy = -r;          // top, left to right
      else if (k < 4 * r) dx = r, dy = -r + (k - 2 * r);  // right, top to bottom
      else if (k < 6 * r) dx = r - (k - 4 * r), dy = r;   // bottom, right to left
      else dx = -r, dy = r - (k - 6 * r);                 // left, bottom to top
      const int x = px + dx, y = py + dy;
      if (x < 0 || y < 0 || x >= n || y >= n) continue;
      const int v = site_at[(size_t)y * n + x];
      if (v >= 0) {
        found = v;
        break;
      }
    }
  }
  start[j] = found >= 0 ? vt[found] : 0;
}

__global__ void k_site_at(const i64 *__restrict__ X, const i64 *__restrict__ Y, int F, int n,
                          int *site_at) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= F) return;
  site_at[(size_t)(Y[v] >> 15) * n + (X[v] >> 15)] = v;
}

__global__ void k_iota(int *a, int count, int base) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) a[i] = base + i;
}

// Drop the inserted points from the pending list (order kept).
__global__ void k_compact(const int *__restrict__ pend, const int *__restrict__ start,
                          const int *__restrict__ done, const int *npp, int *pend2, int *start2,
                          int *count) {
  if (blockIdx.x != 0) return;
  const int np = *npp;
  // one block: a running offset over chunks of blockDim.x
  __shared__ int base;
  __shared__ int wsum[32];
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < np; c0 += blockDim.x) {
    const int q = c0 + threadIdx.x;
    const int keep = q < np && !done[q];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int pre = 0, tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (w < wid) pre += wsum[w];
      tot += wsum[w];
    }
    if (keep) {
      const int pos = base + pre + __popc(bal & ((1u << lane) - 1u));
      pend2[pos] = pend[q];
      start2[pos] = start[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = base;
}

}  // namespace

// The constrained Delaunay triangulation of the free sites of `bits` (point
// indices in gcvt_ctx_extract_points' order) and C constraint points
// (device, 2 C doubles; indices F .. F + C - 1) with S segments (device
// index pairs).  Writes up to cap triangles (3 ints) to out (device) and the
// count to *ntris.
int cdt_compute(const uint64_t *bits, const uint64_t *fixed, int n, unsigned *colcnt,
                const double *cxy, int C, const int *segs, int S, double scale, double left,
                double lower, int *out, unsigned cap, unsigned *ntris, int *detail,
                cudaStream_t s) {
  *ntris = 0;
  if (detail) *detail = 0;
  if (n <= 0 || C < 0 || S < 0 || !(scale > 0)) return GCVT_ERR_ARGUMENT;
  Scratch sc(s);
  // 1. the sites and their Delaunay triangulation
  unsigned F = 0;
  CCK(launch_extract(bits, fixed, n, colcnt, 1.0, 0.0, 0.0, nullptr, 0, colcnt + n, s));
  CCK(cudaMemcpyAsync(&F, colcnt + n, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CCK(cudaStreamSynchronize(s));
  const long long V = (long long)F + C;
  if (V < 3) return GCVT_OK;
  if (V > (1ll << 28)) return GCVT_ERR_SIZE;
  const int cap_t = (int)(2 * V + 16);
  double *sxy = sc.take<double>(2 * (size_t)F + 2);
  i64 *X = sc.take<i64>((size_t)V), *Y = sc.take<i64>((size_t)V), *R = sc.take<i64>((size_t)V);
  int *tri = sc.take<int>(3 * (size_t)cap_t), *nbr = sc.take<int>(3 * (size_t)cap_t);
  unsigned *cons = sc.take<unsigned>((size_t)cap_t);
  int *vt = sc.take<int>((size_t)V);
  unsigned *cl = sc.take<unsigned>((size_t)cap_t);
  int *cand = sc.take<int>((size_t)cap_t);
  uint8_t *act = sc.take<uint8_t>((size_t)cap_t);
  // [0] error bits, [1] triangles, [2] flips wanted, [3] flips made, [4] and
  // [6] points pending (the two lists), [5] segments pending
  int *ctr = sc.take<int>(8);
  if (!sxy || !X || !Y || !R || !tri || !nbr || !cons || !vt || !cl || !cand || !act || !ctr)
    return GCVT_ERR_ALLOC;
  CCK(launch_extract(bits, fixed, n, colcnt, 1.0, 0.0, 0.0, sxy, F, colcnt + n, s));
  CCK(cudaMemsetAsync(ctr, 0, 8 * sizeof(int), s));
  CCK(cudaMemsetAsync(cons, 0, (size_t)cap_t * sizeof(unsigned), s));
  k_cdt_coords<<<nblk(V, 256), 256, 0, s>>>(sxy, (int)F, cxy, C, scale, left, lower, n, X, Y, R,
                                            ctr);
  CCK(cudaGetLastError());
  unsigned T0 = 0;
  int rc = delaunay_sites_in(bits, fixed, n, tri, (unsigned)cap_t, &T0, s, sc);
  if (rc) return rc;
  if (T0 == 0 && C > 0) return GCVT_ERR_INPUT;  // constraint points need triangulated sites
  Mesh m{tri, nbr, cons, vt, X, Y, R};
  // 2. adjacency
  {
    unsigned hsize = 1;
    while (hsize < 6u * T0 + 64u) hsize <<= 1;
    unsigned long long *hk = sc.take<unsigned long long>(hsize);
    int *hv = sc.take<int>(hsize);
    if (!hk || !hv) return GCVT_ERR_ALLOC;
    CCK(cudaMemsetAsync(hk, 0xff, (size_t)hsize * sizeof(unsigned long long), s));
    CCK(cudaMemsetAsync(vt, 0, (size_t)V * sizeof(int), s));  // a vertex in no triangle: 0
    CCK(cudaMemsetAsync(act, 0, (size_t)cap_t, s));           // the sites' triangulation is Delaunay
    k_edge_insert<<<nblk(3ll * T0, 256), 256, 0, s>>>(tri, (int)T0, hk, hv, hsize - 1, ctr);
    k_edge_link<<<nblk(3ll * T0, 256), 256, 0, s>>>(tri, (int)T0, hk, hv, hsize - 1, nbr, vt,
                                                    ctr);
    CCK(cudaGetLastError());
  }
  int T = (int)T0;
  CCK(cudaMemcpyAsync(ctr + 1, &T, sizeof(int), cudaMemcpyHostToDevice, s));
  int h[8] = {};
  auto pull = [&]() -> int {
    CCK(cudaMemcpyAsync(h, ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    return GCVT_OK;
  };
  // Delaunay flip rounds over the changed triangles (their count read on the
  // device: insertions of the same batch add triangles)
  const int fgrid = nblk(cap_t, 256) < kFlipBlocks ? nblk(cap_t, 256) : kFlipBlocks;
  auto flip_rounds = [&](int rounds) -> int {
    for (int i = 0; i < rounds; ++i) {
      CCK(cudaMemsetAsync(cl, 0xff, (size_t)cap_t * sizeof(unsigned), s));
      CCK(cudaMemsetAsync(ctr + 2, 0, 2 * sizeof(int), s));
      k_flip_mark<<<fgrid, 256, 0, s>>>(m, ctr + 1, cand, cl, act, ctr + 2);
      k_flip_apply<<<fgrid, 256, 0, s>>>(m, ctr + 1, cand, cl, act, ctr + 3);
    }
    CCK(cudaGetLastError());
    return GCVT_OK;
  };
  // flip rounds over every triangle until none is left, read back every
  // kFlipPoll rounds (a round that finds nothing to flip changes nothing)
  auto flips = [&]() -> int {
    CCK(cudaMemsetAsync(act, 1, (size_t)cap_t, s));
    for (int r = 0; r < kFlipRounds; r += kFlipPoll) {
      if ((rc = flip_rounds(kFlipPoll)) || (rc = pull())) return rc;
      if (h[0] || h[2] == 0) return GCVT_OK;
    }
    h[0] |= kErrWalk;
    return GCVT_OK;
  };
  // 3. constraint points
  if (C > 0) {
    int *site_at = sc.take<int>((size_t)n * n);
    int *pend = sc.take<int>(C), *pend2 = sc.take<int>(C);
    int *start = sc.take<int>(C), *start2 = sc.take<int>(C), *done = sc.take<int>(C);
    Loc *loc = sc.take<Loc>(C);
    if (!site_at || !pend || !pend2 || !start || !start2 || !done || !loc) return GCVT_ERR_ALLOC;
    CCK(cudaMemsetAsync(site_at, 0xff, (size_t)n * n * sizeof(int), s));
    k_site_at<<<nblk(F, 256), 256, 0, s>>>(X, Y, (int)F, n, site_at);
    k_ins_start<<<nblk(C, 128), 128, 0, s>>>(X, Y, (int)F, C, site_at, n, vt, start);
    k_iota<<<nblk(C, 256), 256, 0, s>>>(pend, C, (int)F);  // point indices F + j
    CCK(cudaGetLastError());
    // one round: the points of list a (count *na) locate, claim and insert;
    // those left go to list b (count *nb); then kInterimFlips flip rounds.  Every
    // count is read on the device, so rounds queue without the host.
    auto ins_round = [&](int *pa, int *sa, int *pb, int *sb, int *na, int *nb) -> int {
      CCK(cudaMemsetAsync(cl, 0xff, (size_t)cap_t * sizeof(unsigned), s));
      CCK(cudaMemsetAsync(done, 0, (size_t)C * sizeof(int), s));
      k_ins_locate<<<nblk(C, 128), 128, 0, s>>>(m, pa, na, sa, loc, cl, ctr);
      k_ins_apply<<<nblk(C, 128), 128, 0, s>>>(m, pa, na, sa, loc, cl, ctr + 1, cap_t, done, act,
                                               ctr);
      k_compact<<<1, 1024, 0, s>>>(pa, sa, done, na, pb, sb, nb);
      CCK(cudaGetLastError());
      return flip_rounds(kInterimFlips);
    };
    // two rounds (list 1 -> 2 -> 1) per read-back, as one CUDA graph where the
    // stream can be captured
    auto ins_pair = [&]() -> int {
      if ((rc = ins_round(pend, start, pend2, start2, ctr + 4, ctr + 6))) return rc;
      return ins_round(pend2, start2, pend, start, ctr + 6, ctr + 4);
    };
    cudaGraphExec_t pair_exec = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int le = ins_pair();
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(s, &g);
      const cudaError_t ie =
          (le == GCVT_OK && ce == cudaSuccess) ? cudaGraphInstantiate(&pair_exec, g, 0) : ce;
      if (g) cudaGraphDestroy(g);
      if (le != GCVT_OK || ce != cudaSuccess || ie != cudaSuccess) {
        if (pair_exec) cudaGraphExecDestroy(pair_exec);
        return GCVT_ERR_CUDA;
      }
    } else {
      cudaGetLastError();  // the legacy default stream: plain launches
    }
    CCK(cudaMemcpyAsync(ctr + 4, &C, sizeof(int), cudaMemcpyHostToDevice, s));
    int np = C;
    for (int r = 0; r < kInsertRounds / 2 && np > 0; ++r) {
      rc = pair_exec ? (cudaGraphLaunch(pair_exec, s) == cudaSuccess ? GCVT_OK : GCVT_ERR_CUDA)
                     : ins_pair();
      if (rc == GCVT_OK) rc = pull();
      if (rc != GCVT_OK) break;
      if (h[0]) break;
      np = h[4];
    }
    if (pair_exec) cudaGraphExecDestroy(pair_exec);
    if (rc != GCVT_OK) return rc;
    if (!h[0] && np > 0) h[0] |= kErrWalk;
  }
  if ((rc = pull())) return rc;
  T = h[1];
  // 4. segments: those already edges marked at once, the others recovered
  // in parallel rounds of claims (window by window), what is left by one
  // thread; 5. flips that keep them
  if (!h[0] && S > 0) {
    const int Wmax = S < kSegWindow ? S : kSegWindow;
    int *state = sc.take<int>((size_t)S), *lcnt = sc.take<int>((size_t)Wmax);
    int *list = sc.take<int>((size_t)Wmax * kClaim);
    int *queue = sc.take<int>(2 * (size_t)kSegQueue), *stack = sc.take<int>(2 * (size_t)kSegStack);
    if (!state || !lcnt || !list || !queue || !stack) return GCVT_ERR_ALLOC;
    k_seg_mark<<<nblk(S, 256), 256, 0, s>>>(m, segs, S, (int)V, state, ctr);
    CCK(cudaGetLastError());
    for (int base = 0; base < S; base += kSegWindow) {
      const int W = S - base < kSegWindow ? S - base : kSegWindow;
      for (int r = 0; r < kSegRounds; ++r) {
        CCK(cudaMemsetAsync(cl, 0xff, (size_t)T * sizeof(unsigned), s));
        CCK(cudaMemsetAsync(ctr + 5, 0, sizeof(int), s));
        k_seg_locate<<<nblk(W, 128), 128, 0, s>>>(m, segs, base, W, state, list, lcnt, cl);
        k_seg_apply<<<nblk(W, 128), 128, 0, s>>>(m, segs, base, W, state, list, lcnt, cl, ctr + 5,
                                                 ctr);
        CCK(cudaGetLastError());
        if ((rc = pull())) return rc;
        if (h[5] == 0) break;
      }
    }
    k_segments<<<1, 32, 0, s>>>(m, segs, S, state, queue, stack, ctr);
    CCK(cudaGetLastError());
    if ((rc = pull())) return rc;
  }
  if (!h[0] && (rc = flips())) return rc;
  if (h[0]) {
    if (detail) *detail = h[0];
    return (h[0] & (kErrCoord | kErrDuplicate | kErrSegment)) ? GCVT_ERR_INPUT : GCVT_ERR_CUDA;
  }
  // 6. output in a fixed order
  int *cnt = sc.take<int>((size_t)V + 1), *off = sc.take<int>((size_t)V + 1),
      *cur = sc.take<int>((size_t)V + 1);
  if (!cnt || !off || !cur) return GCVT_ERR_ALLOC;
  CCK(cudaMemsetAsync(cnt, 0, ((size_t)V + 1) * sizeof(int), s));
  k_emit_count<<<nblk(T, 256), 256, 0, s>>>(m, T, cnt);
  CCK(cudaGetLastError());
  CCK(launch_scan(cnt, (int)V, off, cur, s));
  if (out && cap) {
    k_emit<<<nblk(T, 256), 256, 0, s>>>(m, T, off, out, (int)cap, ctr);
    CCK(cudaGetLastError());
  }
  if ((rc = pull())) return rc;
  if (h[0]) {
    if (detail) *detail = h[0];
    return GCVT_ERR_CUDA;
  }
  *ntris = (unsigned)T;
  return GCVT_OK;
}

}  // namespace cvtgb
