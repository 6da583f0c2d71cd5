// cdt_core.cuh -- the mesh operations of the constrained Delaunay stage
// (cdt.cu): exact predicates, point location, splits, edge flips and the
// recovery of a constraint segment, on a triangle mesh with adjacency.
// Host-and-device functions: the GPU kernels run them in parallel rounds
// (each operation on triangles its point or flip has claimed), and a
// sequential host build of the same functions can replay a run.
//
// Mesh: triangle t has vertices tri[3t .. 3t+2], counter-clockwise, and for
// the edge opposite vertex i the neighbour nbr[3t+i] = (t' << 2) | j, where j
// is the index of the opposite vertex in t' (-1: boundary of the convex
// hull); cons[t] bit i marks that edge a constraint segment; vt[v] is some
// triangle holding vertex v.
//
// Coordinates are integers below 2^29 in magnitude (lattice sites scaled by
// 2^15, constraint points snapped to 2^-15 pixel), so orientations are exact
// in 128-bit integers (products below 2^62) and so is the incircle
// determinant (lifted terms below 2^61, cofactors below 2^61, three products
// below 2^124).  Exactly co-circular points are split by the same symbolic
// perturbation as the sites' Delaunay triangulation (delaunay.cu): z(q) =
// |q|^2 + delta(q), delta infinitesimal and infinitely larger for a larger
// rank R[q].
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define CDT_HD __host__ __device__ __forceinline__
#else
#define CDT_HD inline
#endif

namespace cvtgb {
namespace cdt {

typedef long long i64;
typedef __int128 i128;

constexpr int kNone = -1;

struct Mesh {
  int *tri;
  int *nbr;
  unsigned *cons;
  int *vt;
  const i64 *X, *Y, *R;
};

// The priority of an operation with id x in a round of claims (the
// smallest wins): a bijection of 32-bit words (xor-shift and odd-multiplier
// steps, each invertible; the "lowbias32" constants of C. Wellons' hash
// prospector), so distinct ids never tie and neighbours along a list do not
// win in index order.
CDT_HD unsigned prio(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

CDT_HD int nb_tri(int v) { return v >> 2; }
CDT_HD int nb_idx(int v) { return v & 3; }
CDT_HD int pack_nb(int t, int j) { return (t << 2) | j; }
CDT_HD int nx3(int i) { return i == 2 ? 0 : i + 1; }
CDT_HD int pv3(int i) { return i == 0 ? 2 : i - 1; }

// sign of the orientation of (a, b, c): > 0 counter-clockwise
CDT_HD int orient(const Mesh &m, int a, int b, int c) {
  const i128 d = (i128)(m.X[b] - m.X[a]) * (m.Y[c] - m.Y[a]) -
                 (i128)(m.Y[b] - m.Y[a]) * (m.X[c] - m.X[a]);
  return d > 0 ? 1 : (d < 0 ? -1 : 0);
}

// Is d strictly inside the circle through a, b, c (counter-clockwise),
// under the perturbation?  Rows a - d, b - d, c - d; the determinant is
// linear in the lifted column, so on an exact zero the sign is that of the
// top-ranked point's cofactor.
CDT_HD bool incircle(const Mesh &m, int a, int b, int c, int d) {
  const i64 r0x = m.X[a] - m.X[d], r0y = m.Y[a] - m.Y[d];
  const i64 r1x = m.X[b] - m.X[d], r1y = m.Y[b] - m.Y[d];
  const i64 r2x = m.X[c] - m.X[d], r2y = m.Y[c] - m.Y[d];
  const i128 m0 = (i128)r1x * r2y - (i128)r1y * r2x;
  const i128 m1 = (i128)r0x * r2y - (i128)r0y * r2x;
  const i128 m2 = (i128)r0x * r1y - (i128)r0y * r1x;
  const i128 z0 = (i128)r0x * r0x + (i128)r0y * r0y;
  const i128 z1 = (i128)r1x * r1x + (i128)r1y * r1y;
  const i128 z2 = (i128)r2x * r2x + (i128)r2y * r2y;
  const i128 det = z0 * m0 - z1 * m1 + z2 * m2;
  if (det != 0) return det > 0;
  const i64 ha = m.R[a], hb = m.R[b], hc = m.R[c], hd = m.R[d];
  if (ha > hb && ha > hc && ha > hd) return m0 > 0;
  if (hb > hc && hb > hd) return m1 < 0;
  if (hc > hd) return m2 > 0;
  return m0 - m1 + m2 < 0;
}

enum { kLocIn = 0, kLocEdge = 1, kLocOut = 2, kLocVertex = 3, kLocFail = 4 };

// Walk from triangle t towards point p (straight visibility walk, exact):
// kLocIn (p inside *ot), kLocEdge (p inside the edge opposite vertex *oi of
// *ot), kLocOut (p outside the hull beyond the boundary edge opposite *oi of
// *ot), kLocVertex (p coincides with vertex *oi of *ot), kLocFail (no answer
// within max_steps).  The edges are tried from a rotating start, which keeps
// the walk from cycling.
CDT_HD int locate(const Mesh &m, int p, int t, int max_steps, int *ot, int *oi) {
  for (int s = 0; s < max_steps; ++s) {
    const int *v = m.tri + 3 * t;
    int zeros = 0, zi = -1, next = -1;
    for (int q = 0; q < 3; ++q) {
      const int i = (q + s) % 3;
      const int o = orient(m, v[nx3(i)], v[pv3(i)], p);
      if (o < 0) {
        next = i;
        break;
      }
      if (o == 0) {
        ++zeros;
        zi = i;
      }
    }
    if (next >= 0) {
      const int nb = m.nbr[3 * t + next];
      if (nb < 0) {
        *ot = t;
        *oi = next;
        return kLocOut;
      }
      t = nb_tri(nb);
      continue;
    }
    *ot = t;
    if (zeros == 0) {
      *oi = -1;
      return kLocIn;
    }
    if (zeros == 1) {
      *oi = zi;
      return kLocEdge;
    }
    // two zero orientations: p is the vertex where those edges meet
    for (int i = 0; i < 3; ++i)
      if (m.X[v[i]] == m.X[p] && m.Y[v[i]] == m.Y[p]) *oi = i;
    return kLocVertex;
  }
  return kLocFail;
}

// Set the neighbour of (t, i) to nb and, when nb is a triangle, its
// neighbour back to (t, i).
CDT_HD void link(const Mesh &m, int t, int i, int nb) {
  m.nbr[3 * t + i] = nb;
  if (nb >= 0) m.nbr[3 * nb_tri(nb) + nb_idx(nb)] = pack_nb(t, i);
}

CDT_HD void set_tri(const Mesh &m, int t, int a, int b, int c) {
  m.tri[3 * t] = a;
  m.tri[3 * t + 1] = b;
  m.tri[3 * t + 2] = c;
}

// p strictly inside t = (a, b, c): t becomes (a, b, p), new slots n1 =
// (b, c, p) and n2 = (c, a, p).
CDT_HD void split_in(const Mesh &m, int t, int p, int n1, int n2) {
  const int a = m.tri[3 * t], b = m.tri[3 * t + 1], c = m.tri[3 * t + 2];
  const int na = m.nbr[3 * t], nb = m.nbr[3 * t + 1], nc = m.nbr[3 * t + 2];
  const int ct = m.cons[t];
  set_tri(m, t, a, b, p);
  set_tri(m, n1, b, c, p);
  set_tri(m, n2, c, a, p);
  m.cons[t] = (unsigned)(((ct >> 2) & 1) << 2);  // (a, b)
  m.cons[n1] = (unsigned)((ct & 1) << 2);        // (b, c)
  m.cons[n2] = (unsigned)(((ct >> 1) & 1) << 2); // (c, a)
  m.nbr[3 * t] = pack_nb(n1, 1);
  m.nbr[3 * t + 1] = pack_nb(n2, 0);
  link(m, t, 2, nc);
  m.nbr[3 * n1] = pack_nb(n2, 1);
  m.nbr[3 * n1 + 1] = pack_nb(t, 0);
  link(m, n1, 2, na);
  m.nbr[3 * n2] = pack_nb(t, 1);
  m.nbr[3 * n2 + 1] = pack_nb(n1, 0);
  link(m, n2, 2, nb);
  m.vt[a] = t;
  m.vt[b] = t;
  m.vt[c] = n1;
  m.vt[p] = t;
}

// p inside the edge opposite vertex i of t (edge (b, c), a = the apex).
// With a neighbour t' = (d, c, b) across it: t = (a, b, p), n1 = (a, p, c),
// t' = (d, c, p), n2 = (d, p, b); on the hull: t = (a, b, p), n1 = (a, p, c).
// A constraint on (b, c) passes to both halves.
CDT_HD void split_edge(const Mesh &m, int t, int i, int p, int n1, int n2) {
  const int a = m.tri[3 * t + i], b = m.tri[3 * t + nx3(i)], c = m.tri[3 * t + pv3(i)];
  const int nab = m.nbr[3 * t + pv3(i)], nca = m.nbr[3 * t + nx3(i)];
  const int ct = m.cons[t];
  const int cab = (ct >> pv3(i)) & 1, cca = (ct >> nx3(i)) & 1, cbc = (ct >> i) & 1;
  const int opp = m.nbr[3 * t + i];
  if (opp < 0) {
    set_tri(m, t, a, b, p);
    set_tri(m, n1, a, p, c);
    m.nbr[3 * t] = kNone;
    m.nbr[3 * t + 1] = pack_nb(n1, 2);
    link(m, t, 2, nab);
    m.nbr[3 * n1] = kNone;
    link(m, n1, 1, nca);
    m.nbr[3 * n1 + 2] = pack_nb(t, 1);
    m.cons[t] = (unsigned)(cbc | (cab << 2));
    m.cons[n1] = (unsigned)(cbc | (cca << 1));
    m.vt[a] = t;
    m.vt[b] = t;
    m.vt[c] = n1;
    m.vt[p] = t;
    return;
  }
  const int t2 = nb_tri(opp), j = nb_idx(opp);
  const int d = m.tri[3 * t2 + j];
  const int nbd = m.nbr[3 * t2 + nx3(j)], ndc = m.nbr[3 * t2 + pv3(j)];
  const int c2 = m.cons[t2];
  const int cbd = (c2 >> nx3(j)) & 1, cdc = (c2 >> pv3(j)) & 1;
  set_tri(m, t, a, b, p);
  set_tri(m, n1, a, p, c);
  set_tri(m, t2, d, c, p);
  set_tri(m, n2, d, p, b);
  m.nbr[3 * t] = pack_nb(n2, 0);
  m.nbr[3 * t + 1] = pack_nb(n1, 2);
  link(m, t, 2, nab);
  m.nbr[3 * n1] = pack_nb(t2, 0);
  link(m, n1, 1, nca);
  m.nbr[3 * n1 + 2] = pack_nb(t, 1);
  m.nbr[3 * t2] = pack_nb(n1, 0);
  m.nbr[3 * t2 + 1] = pack_nb(n2, 2);
  link(m, t2, 2, ndc);
  m.nbr[3 * n2] = pack_nb(t, 0);
  link(m, n2, 1, nbd);
  m.nbr[3 * n2 + 2] = pack_nb(t2, 1);
  m.cons[t] = (unsigned)(cbc | (cab << 2));
  m.cons[n1] = (unsigned)(cbc | (cca << 1));
  m.cons[t2] = (unsigned)(cbc | (cdc << 2));
  m.cons[n2] = (unsigned)(cbc | (cbd << 1));
  m.vt[a] = t;
  m.vt[b] = t;
  m.vt[c] = n1;
  m.vt[d] = t2;
  m.vt[p] = t;
}

// The boundary edge after (opposite vertex i of t) in counter-clockwise hull
// order: rotate around the edge's end vertex.  False past max_steps.
CDT_HD bool hull_next(const Mesh &m, int t, int i, int max_steps, int *ot, int *oi) {
  // the edge runs u = v[i+1] -> w = v[i+2]; around w through the interior:
  // the edge (w, v[cw+1]) leaving w is opposite v[cw+2]
  int ct = t, cw = pv3(i);  // w's index in ct
  for (int s = 0; s < max_steps; ++s) {
    const int e = pv3(cw);
    const int nb = m.nbr[3 * ct + e];
    if (nb < 0) {
      *ot = ct;
      *oi = e;
      return true;
    }
    ct = nb_tri(nb);
    cw = pv3(nb_idx(nb));  // the shared edge (x, w) there runs v[j+1] -> v[j+2] = w
  }
  return false;
}

// The boundary edge before (opposite vertex i of t): rotate around the
// edge's start vertex the other way.
CDT_HD bool hull_prev(const Mesh &m, int t, int i, int max_steps, int *ot, int *oi) {
  // around u = v[i+1] the other way: the edge (v[cu+2], u) entering u is
  // opposite v[cu+1]
  int ct = t, cu = nx3(i);
  for (int s = 0; s < max_steps; ++s) {
    const int e = nx3(cu);
    const int nb = m.nbr[3 * ct + e];
    if (nb < 0) {
      *ot = ct;
      *oi = e;
      return true;
    }
    ct = nb_tri(nb);
    cu = nx3(nb_idx(nb));  // the shared edge (u, x) there runs v[j+1] = u -> v[j+2]
  }
  return false;
}

// p outside the hull, seeing the m boundary edges (et[k], ei[k]), k = 0 .. m-1
// in counter-clockwise hull order (edge k runs u_k -> w_k = u_{k+1}): the
// new triangles slots[k] = (w_k, u_k, p), each facing its hull edge's
// triangle and its fan neighbours; their outer edges (u_0, p) and
// (p, w_{m-1}) are the new hull.
CDT_HD void insert_out(const Mesh &m, const int *et, const int *ei, int cnt, int p,
                       const int *slots) {
  for (int k = 0; k < cnt; ++k) {
    const int t = et[k], i = ei[k];
    const int u = m.tri[3 * t + nx3(i)], w = m.tri[3 * t + pv3(i)];
    const int s = slots[k];
    set_tri(m, s, w, u, p);
    m.cons[s] = 0;
    link(m, s, 2, pack_nb(t, i));
    m.nbr[3 * s] = k == 0 ? kNone : pack_nb(slots[k - 1], 1);
    m.nbr[3 * s + 1] = k + 1 == cnt ? kNone : pack_nb(slots[k + 1], 0);
    m.vt[u] = s;
    m.vt[w] = s;
  }
  m.vt[p] = slots[0];
}

// Flip the edge opposite vertex i of t (a = apex, edge (b, c)) with the
// neighbour t' = (d, c, b): t = (a, b, d), t' = (a, d, c).
CDT_HD void flip(const Mesh &m, int t, int i) {
  const int opp = m.nbr[3 * t + i];
  const int t2 = nb_tri(opp), j = nb_idx(opp);
  const int a = m.tri[3 * t + i], b = m.tri[3 * t + nx3(i)], c = m.tri[3 * t + pv3(i)];
  const int d = m.tri[3 * t2 + j];
  const int nab = m.nbr[3 * t + pv3(i)], nca = m.nbr[3 * t + nx3(i)];
  const int nbd = m.nbr[3 * t2 + nx3(j)], ndc = m.nbr[3 * t2 + pv3(j)];
  const int ct = m.cons[t], c2 = m.cons[t2];
  const int cab = (ct >> pv3(i)) & 1, cca = (ct >> nx3(i)) & 1;
  const int cbd = (c2 >> nx3(j)) & 1, cdc = (c2 >> pv3(j)) & 1;
  set_tri(m, t, a, b, d);
  set_tri(m, t2, a, d, c);
  link(m, t, 0, nbd);
  m.nbr[3 * t + 1] = pack_nb(t2, 2);
  link(m, t, 2, nab);
  link(m, t2, 0, ndc);
  link(m, t2, 1, nca);
  m.nbr[3 * t2 + 2] = pack_nb(t, 1);
  m.cons[t] = (unsigned)(cbd | (cab << 2));
  m.cons[t2] = (unsigned)(cdc | (cca << 1));
  m.vt[a] = t;
  m.vt[b] = t;
  m.vt[d] = t;
  m.vt[c] = t2;
}

// Should the edge opposite vertex i of t be flipped for the Delaunay
// property (it has a neighbour, is not a constraint, and the neighbour's
// apex is inside t's circle)?
CDT_HD bool wants_flip(const Mesh &m, int t, int i) {
  const int opp = m.nbr[3 * t + i];
  if (opp < 0 || ((m.cons[t] >> i) & 1)) return false;
  const int d = m.tri[3 * nb_tri(opp) + nb_idx(opp)];
  return incircle(m, m.tri[3 * t], m.tri[3 * t + 1], m.tri[3 * t + 2], d);
}

// The triangle with the directed edge (u, w) (u at index *oi, w next), found
// by rotating around u from vt[u]; false if there is none within max_steps.
CDT_HD bool find_edge(const Mesh &m, int u, int w, int max_steps, int *ot, int *oi) {
  int t = m.vt[u];
  for (int dir = 0; dir < 2; ++dir) {
    int ct = t;
    for (int s = 0; s < max_steps; ++s) {
      const int *v = m.tri + 3 * ct;
      const int k = v[0] == u ? 0 : (v[1] == u ? 1 : 2);
      if (v[nx3(k)] == w) {
        *ot = ct;
        *oi = k;
        return true;
      }
      // counter-clockwise around u: across the edge (u, v[k+2]), opposite
      // v[k+1]; clockwise: across (v[k+1], u)... opposite v[k+2]
      const int nb = m.nbr[3 * ct + (dir == 0 ? nx3(k) : pv3(k))];
      if (nb < 0) break;
      ct = nb_tri(nb);
      if (ct == t) return false;
    }
  }
  return false;
}

// Set constraint bits of a triangle; atomic on the device, where segments
// already present as edges are marked by many threads at once.
CDT_HD void or_bits(unsigned *w, unsigned bits) {
#ifdef __CUDA_ARCH__
  atomicOr(w, bits);
#else
  *w |= bits;
#endif
}

// Mark the edge {u, w} a constraint in both of its triangles; false if it is
// not an edge.
CDT_HD bool mark_constraint(const Mesh &m, int u, int w, int max_steps) {
  int t, k;
  if (!find_edge(m, u, w, max_steps, &t, &k) && !find_edge(m, w, u, max_steps, &t, &k))
    return false;
  // the edge is opposite v[k+2] of t
  or_bits(m.cons + t, 1u << pv3(k));
  const int nb = m.nbr[3 * t + pv3(k)];
  if (nb >= 0) or_bits(m.cons + nb_tri(nb), 1u << nb_idx(nb));
  return true;
}

// The triangles around vertex v (from vt[v], counter-clockwise until the
// start comes back or the hull is reached, then clockwise from the start):
// their count, or -1 when they are more than cap or a rotation runs past
// max_steps.
CDT_HD int fan(const Mesh &m, int v, int max_steps, int *out, int cap) {
  const int t0 = m.vt[v];
  int cnt = 0;
  for (int dir = 0; dir < 2; ++dir) {
    int ct = t0, s = 0;
    for (; s < max_steps; ++s) {
      if (dir == 0 || ct != t0) {
        if (cnt >= cap) return -1;
        out[cnt++] = ct;
      }
      const int *w = m.tri + 3 * ct;
      const int k = w[0] == v ? 0 : (w[1] == v ? 1 : 2);
      const int nb = m.nbr[3 * ct + (dir == 0 ? nx3(k) : pv3(k))];
      if (nb < 0) break;
      ct = nb_tri(nb);
      if (ct == t0) return cnt;  // all the way round
    }
    if (s == max_steps) return -1;
  }
  return cnt;
}

enum { kSegOk = 0, kSegVertexOn = 1, kSegLimit = 2, kSegBroken = 3, kSegCrosses = 4 };

// The edges crossing the segment (a, b), which is not an edge, as vertex
// pairs in queue[0 .. *cnt_out), walking from a towards b; read-only.
// kSegVertexOn (*on = the vertex) when a vertex lies inside the segment,
// kSegCrosses when a crossing edge is a constraint, kSegLimit when qcap or
// max_steps runs out.
CDT_HD int collect_crossings(const Mesh &m, int a, int b, int *queue, int qcap, int max_steps,
                             int *on, int *cnt_out) {
  *cnt_out = 0;
  // the triangle at a whose wedge holds the direction to b
  int t = m.vt[a], k = 0;
  bool got = false;
  for (int dir = 0; dir < 2 && !got; ++dir) {
    int ct = t;
    for (int s = 0; s < max_steps; ++s) {
      const int *v = m.tri + 3 * ct;
      k = v[0] == a ? 0 : (v[1] == a ? 1 : 2);
      const int u = v[nx3(k)], w = v[pv3(k)];
      const int ou = orient(m, a, u, b), ow = orient(m, a, w, b);
      if (ou == 0 && (m.X[u] - m.X[a]) * (m.X[b] - m.X[a]) + (m.Y[u] - m.Y[a]) * (m.Y[b] - m.Y[a]) > 0) {
        *on = u;  // on the ray towards b, before b (b cannot lie inside the edge (a, u))
        return kSegVertexOn;
      }
      if (ou > 0 && ow < 0) {
        t = ct;
        got = true;
        break;
      }
      const int nb = m.nbr[3 * ct + (dir == 0 ? nx3(k) : pv3(k))];
      if (nb < 0) break;
      ct = nb_tri(nb);
      if (ct == t) break;
    }
  }
  if (!got) return kSegBroken;
  // walk to b collecting the crossing edges (left end l, right end r)
  int cnt = 0;
  const int *v = m.tri + 3 * t;
  int r = v[nx3(k)], l = v[pv3(k)];  // b is left of a->r and right of a->l
  int ct = t, ce = k;                // the crossing edge (r, l) is opposite v[ce] of ct
  for (int s = 0; s < max_steps; ++s) {
    if (cnt >= qcap) return kSegLimit;
    if ((m.cons[ct] >> ce) & 1) return kSegCrosses;
    queue[2 * cnt] = r;
    queue[2 * cnt + 1] = l;
    ++cnt;
    const int nb = m.nbr[3 * ct + ce];
    if (nb < 0) return kSegBroken;
    ct = nb_tri(nb);
    const int j = nb_idx(nb);
    const int y = m.tri[3 * ct + j];
    if (y == b) {
      *cnt_out = cnt;
      return kSegOk;
    }
    const int oy = orient(m, a, b, y);
    if (oy == 0) {  // inside the segment: the walk stays between a and b
      *on = y;
      return kSegVertexOn;
    }
    // in ct = (y, l, r) (counter-clockwise), the next crossing edge is the
    // one between y and the end on y's other side
    if (oy < 0) {  // y right of a->b: replaces r; edge (y, l) is opposite r
      r = y;
      ce = pv3(j);
    } else {       // y left: replaces l; edge (r, y) is opposite l
      l = y;
      ce = nx3(j);
    }
  }
  return kSegLimit;
}

// Make (a, b) an edge by flipping the edges that cross it (Sloan's method):
// the crossing edges are collected by walking from a towards b, then taken
// from a queue in turn -- an edge whose quadrilateral is strictly convex is
// flipped (its new diagonal goes back into the queue if it still crosses
// (a, b)), any other goes to the back.  Then (a, b) is marked a constraint.
// queue: scratch of qcap vertex pairs.  kSegVertexOn (*on = the vertex) when
// a vertex lies inside the segment: the caller recovers the two pieces
// instead; kSegCrosses when the segment crosses a constraint already in
// place (invalid input), kSegLimit when a bound runs out.
CDT_HD int recover_segment(const Mesh &m, int a, int b, int *queue, int qcap, int max_steps,
                           int *on) {
  if (mark_constraint(m, a, b, max_steps)) return kSegOk;
  int cnt = 0;
  const int got = collect_crossings(m, a, b, queue, qcap, max_steps, on, &cnt);
  if (got != kSegOk) return got;
  int head = 0, tail = cnt % qcap;
  // Sloan's loop
  for (int s = 0; cnt > 0; ++s) {
    if (s >= max_steps) return kSegLimit;
    const int u = queue[2 * head], w = queue[2 * head + 1];
    head = (head + 1) % qcap;
    --cnt;
    int ct, ck;
    if (!find_edge(m, u, w, max_steps, &ct, &ck)) return kSegBroken;
    // (u, w) in ct = (u, w, x) is opposite x = v[ck+2]; flip(ct, ck+2)
    const int ix = pv3(ck);
    const int x = m.tri[3 * ct + ix];
    const int opp = m.nbr[3 * ct + ix];
    if (opp < 0) return kSegBroken;
    const int y = m.tri[3 * nb_tri(opp) + nb_idx(opp)];
    if (orient(m, x, u, y) > 0 && orient(m, y, w, x) > 0) {
      flip(m, ct, ix);
      const int ox = orient(m, a, b, x), oy = orient(m, a, b, y);
      if ((ox > 0 && oy < 0) || (ox < 0 && oy > 0)) {
        if (cnt >= qcap) return kSegLimit;
        queue[2 * tail] = x;
        queue[2 * tail + 1] = y;
        tail = (tail + 1) % qcap;
        ++cnt;
      }
    } else {
      if (cnt >= qcap) return kSegLimit;
      queue[2 * tail] = u;
      queue[2 * tail + 1] = w;
      tail = (tail + 1) % qcap;
      ++cnt;
    }
  }
  return mark_constraint(m, a, b, max_steps) ? kSegOk : kSegBroken;
}

// Triangle t rotated to start at its smallest vertex (its owner).
CDT_HD void canon(const int *v, int &a, int &b, int &c) {
  if (v[0] < v[1] && v[0] < v[2]) {
    a = v[0]; b = v[1]; c = v[2];
  } else if (v[1] < v[2]) {
    a = v[1]; b = v[2]; c = v[0];
  } else {
    a = v[2]; b = v[0]; c = v[1];
  }
}

// The rank of triangle t among the triangles its owner a owns, by their
// second vertex (they all lie around a: rotate both ways from t); -1 if a
// rotation runs past max_steps.
CDT_HD int owner_rank(const Mesh &m, int t, int max_steps) {
  int a, b, c;
  canon(m.tri + 3 * t, a, b, c);
  int rank = 0;
  for (int dir = 0; dir < 2; ++dir) {
    int ct = t, s = 0;
    bool full = false;
    for (; s < max_steps; ++s) {
      const int *v = m.tri + 3 * ct;
      const int k = v[0] == a ? 0 : (v[1] == a ? 1 : 2);
      const int nb = m.nbr[3 * ct + (dir == 0 ? nx3(k) : pv3(k))];
      if (nb < 0) break;
      ct = nb_tri(nb);
      if (ct == t) {
        full = true;
        break;
      }
      int x, y, z;
      canon(m.tri + 3 * ct, x, y, z);
      if (x == a && y < b) ++rank;
    }
    if (s == max_steps) return -1;
    if (full) break;  // every triangle around a seen in one direction
  }
  return rank;
}

// The segment (a, b) made a chain of constraint edges: recovered whole, or,
// where vertices lie inside it, piece by piece between them (stack: scratch
// of scap pairs).
CDT_HD int recover_chain(const Mesh &m, int a, int b, int *queue, int qcap, int *stack,
                         int scap, int max_steps) {
  int top = 0;
  stack[0] = a;
  stack[1] = b;
  top = 1;
  while (top > 0) {
    --top;
    const int u = stack[2 * top], w = stack[2 * top + 1];
    int v = -1;
    const int r = recover_segment(m, u, w, queue, qcap, max_steps, &v);
    if (r == kSegVertexOn) {
      if (top + 2 > scap) return kSegLimit;
      stack[2 * top] = v;  // (v, w) after (u, v)
      stack[2 * top + 1] = w;
      stack[2 * top + 2] = u;
      stack[2 * top + 3] = v;
      top += 2;
      continue;
    }
    if (r != kSegOk) return r;
  }
  return kSegOk;
}

}  // namespace cdt
}  // namespace cvtgb
