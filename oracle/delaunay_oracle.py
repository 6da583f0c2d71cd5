"""Delaunay checks for lattice sites (TEST INFRASTRUCTURE ONLY).

Only tests/ use this module.  Two parts:

* check(points, tris): restates gDel2D's DelaunayChecker
  (gDel2D/DelaunayChecker.cpp:27-87 checkEuler, :99-144 checkAdjacency,
  :146-169 checkOrientation, :171-213 checkDelaunay) in exact integer
  arithmetic, plus the coverage DelaunayChecker leaves implicit: the
  triangles tile the sites' convex hull (their areas sum to the hull's) and
  every site is a vertex, so the count is 2V - h - 2 (h: sites on the hull).
* check_fast(points, tris): the same checks vectorised with numpy, for the
  full-size workloads (10^5 - 10^6 sites).
* sos_triangulation(points, n): the one Delaunay triangulation that the
  symbolic perturbation z(q) = |q|^2 + delta(q) picks (delta infinitesimal,
  infinitely larger for a larger rank y n + x), by brute force over all
  triples -- small point sets only.

Points are (x, y) lattice coordinates below 2^13, so every determinant fits
in int64 when taken relative to one of its points.
"""
import itertools

import numpy as np


def _orient(a, b, c):
    return (int(b[0]) - int(a[0])) * (int(c[1]) - int(a[1])) - \
        (int(b[1]) - int(a[1])) * (int(c[0]) - int(a[0]))


def _incircle(p, a, b, d):
    """> 0 when d is strictly inside the circle through p, a, b (CCW)."""
    r = [(int(q[0]) - int(d[0]), int(q[1]) - int(d[1])) for q in (p, a, b)]
    m0 = r[1][0] * r[2][1] - r[1][1] * r[2][0]
    m1 = r[0][0] * r[2][1] - r[0][1] * r[2][0]
    m2 = r[0][0] * r[1][1] - r[0][1] * r[1][0]
    z = [x * x + y * y for x, y in r]
    return z[0] * m0 - z[1] * m1 + z[2] * m2, (m0, m1, m2)


def _incircle_many(p, a, b, d):
    """Vectorised _incircle over the rows of d (int64)."""
    r0 = p[None, :] - d
    r1 = a[None, :] - d
    r2 = b[None, :] - d
    m0 = r1[:, 0] * r2[:, 1] - r1[:, 1] * r2[:, 0]
    m1 = r0[:, 0] * r2[:, 1] - r0[:, 1] * r2[:, 0]
    m2 = r0[:, 0] * r1[:, 1] - r0[:, 1] * r1[:, 0]
    z0 = (r0 * r0).sum(1)
    z1 = (r1 * r1).sum(1)
    z2 = (r2 * r2).sum(1)
    return z0 * m0 - z1 * m1 + z2 * m2, m0, m1, m2


def hull_size(points):
    """Sites on the boundary of their convex hull (corners and edge points)."""
    pts = sorted(set(map(tuple, np.asarray(points).tolist())))
    if len(pts) < 3:
        return len(pts), []

    def chain(seq):
        h = []
        for q in seq:
            while len(h) >= 2 and _orient(h[-2], h[-1], q) <= 0:
                h.pop()
            h.append(q)
        return h
    lower, upper = chain(pts), chain(pts[::-1])
    corners = lower[:-1] + upper[:-1]
    if len(corners) < 3:
        return 0, []
    on = 0
    for q in pts:
        for i in range(len(corners)):
            a, b = corners[i], corners[(i + 1) % len(corners)]
            if _orient(a, b, q) == 0 and min(a[0], b[0]) <= q[0] <= max(a[0], b[0]) and \
                    min(a[1], b[1]) <= q[1] <= max(a[1], b[1]):
                on += 1
                break
    return on, corners


def check(points, tris):
    """Raise AssertionError unless tris is a Delaunay triangulation of points
    (integer (V, 2)); returns a dict of the counts."""
    pts = np.asarray(points, np.int64)
    tris = np.asarray(tris, np.int64).reshape(-1, 3)
    v = len(pts)
    h, corners = hull_size(pts)
    if len(corners) < 3:  # collinear or fewer than three sites
        assert len(tris) == 0, "triangles of collinear sites"
        return {"vertices": 0, "edges": 0, "triangles": 0, "hull": 0}
    assert len(tris) == 2 * v - h - 2, f"{len(tris)} triangles, expected {2 * v - h - 2}"
    assert tris.min() >= 0 and tris.max() < v, "index out of range"
    # checkOrientation: every triangle counter-clockwise, none flat
    a, b, c = pts[tris[:, 0]], pts[tris[:, 1]], pts[tris[:, 2]]
    o = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    assert (o > 0).all(), f"{int((o <= 0).sum())} triangles not counter-clockwise"
    # coverage: twice the areas sum to twice the hull's area
    hull2 = sum(_orient(corners[0], corners[i], corners[i + 1]) for i in range(1, len(corners) - 1))
    assert int(o.sum()) == hull2, "triangles do not tile the hull"
    # checkAdjacency: each directed edge once; an edge's two triangles face
    # each other; boundary edges are the hull's
    opp = {}
    for t, (i, j, k) in enumerate(tris.tolist()):
        for e, w in (((i, j), k), ((j, k), i), ((k, i), j)):
            assert e not in opp, f"directed edge {e} twice"
            opp[e] = (t, w)
    edges = {tuple(sorted(e)) for e in opp}
    # checkEuler: V - E + F = 1 (outer face not counted)
    used = np.unique(tris)
    assert len(used) == v, f"{v - len(used)} sites not in any triangle"
    assert v - len(edges) + len(tris) == 1, "Euler characteristic"
    # checkDelaunay: no opposite vertex strictly inside a neighbour's circle
    ties = 0
    for (i, j), (t, w) in opp.items():
        if (j, i) not in opp:
            continue
        _, x = opp[(j, i)]
        det, _ = _incircle(pts[i], pts[j], pts[w], pts[x])
        assert det <= 0, f"edge {(i, j)} not locally Delaunay"
        ties += det == 0
    return {"vertices": v, "edges": len(edges), "triangles": len(tris), "hull": h,
            "cocircular_edges": ties // 2}


def sos_in_circle(p, a, b, d, hp, ha, hb, hd):
    """The perturbed predicate: d inside the circle through p, a, b (CCW)."""
    det, (m0, m1, m2) = _incircle(p, a, b, d)
    if det:
        return det > 0
    top = max(hp, ha, hb, hd)
    if top == hp:
        return m0 > 0
    if top == ha:
        return m1 < 0
    if top == hb:
        return m2 > 0
    return m0 - m1 + m2 < 0


def sos_triangulation(points, n):
    """All CCW triangles (sorted rows, smallest index first) whose perturbed
    circumcircle holds no other site: the triangulation the symbolic
    perturbation picks.  O(V^4): small sets only."""
    pts = np.asarray(points, np.int64)
    rank = pts[:, 1] * n + pts[:, 0]
    v = len(pts)
    out = []
    for i, j, k in itertools.combinations(range(v), 3):
        o = _orient(pts[i], pts[j], pts[k])
        if o == 0:
            continue
        if o < 0:
            j, k = k, j
        others = np.array([q for q in range(v) if q not in (i, j, k)], np.int64)
        if len(others):
            det, m0, m1, m2 = _incircle_many(pts[i], pts[j], pts[k], pts[others])
            if (det > 0).any():
                continue
            bad = False
            for q in others[det == 0].tolist():
                if sos_in_circle(pts[i], pts[j], pts[k], pts[q], rank[i], rank[j], rank[k],
                                 rank[q]):
                    bad = True
                    break
            if bad:
                continue
        out.append(canonical([(i, j, k)])[0])
    return np.array(sorted(out), np.int64).reshape(-1, 3)


def canonical(tris):
    """Rotate each CCW triangle to start at its smallest index; sort rows."""
    rows = []
    for t in np.asarray(tris).reshape(-1, 3).tolist():
        r = t.index(min(t))
        rows.append(tuple(t[r:] + t[:r]))
    return sorted(rows)


def check_fast(points, tris):
    """The checks of check() vectorised with numpy (for 10^5 - 10^6 sites):
    orientation, each directed edge once, every site a vertex, Euler,
    2V - h - 2 triangles, area sum = hull area, and every interior edge
    locally Delaunay (exact int64 incircle).  Returns the same counts."""
    pts = np.asarray(points, np.int64)
    t = np.asarray(tris, np.int64).reshape(-1, 3)
    v = len(pts)
    h, corners = hull_size_fast(pts)
    if len(corners) < 3:
        assert len(t) == 0, "triangles of collinear sites"
        return {"vertices": 0, "edges": 0, "triangles": 0, "hull": 0}
    assert len(t) == 2 * v - h - 2, f"{len(t)} triangles, expected {2 * v - h - 2}"
    assert t.min() >= 0 and t.max() < v, "index out of range"
    a, b, c = pts[t[:, 0]], pts[t[:, 1]], pts[t[:, 2]]
    o = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    assert (o > 0).all(), f"{int((o <= 0).sum())} triangles not counter-clockwise"
    cs = corners.astype(np.int64)
    hull2 = int(((cs[1:-1, 0] - cs[0, 0]) * (cs[2:, 1] - cs[0, 1]) -
                 (cs[1:-1, 1] - cs[0, 1]) * (cs[2:, 0] - cs[0, 0])).sum())
    assert int(o.sum()) == hull2, "triangles do not tile the hull"
    assert len(np.unique(t)) == v, "sites not in any triangle"
    # directed edges (i, j) with the opposite vertex w
    src = np.concatenate([t[:, 0], t[:, 1], t[:, 2]])
    dst = np.concatenate([t[:, 1], t[:, 2], t[:, 0]])
    opp = np.concatenate([t[:, 2], t[:, 0], t[:, 1]])
    key = src * v + dst
    order = np.argsort(key, kind="stable")
    ks = key[order]
    assert (ks[1:] != ks[:-1]).all(), "a directed edge twice"
    edges = np.unique(np.minimum(src, dst) * v + np.maximum(src, dst))
    assert v - len(edges) + len(t) == 1, "Euler characteristic"
    # the reverse of each directed edge, when it exists: interior edges
    rkey = dst * v + src
    pos = np.searchsorted(ks, rkey)
    pos_c = np.minimum(pos, len(ks) - 1)
    found = ks[pos_c] == rkey
    i, j, w = src[found], dst[found], opp[found]
    x = opp[order[pos_c[found]]]
    # x must not be strictly inside the circle through i, j, w (CCW)
    p0, p1, p2, d = pts[i], pts[j], pts[w], pts[x]
    r0, r1, r2 = p0 - d, p1 - d, p2 - d
    m0 = r1[:, 0] * r2[:, 1] - r1[:, 1] * r2[:, 0]
    m1 = r0[:, 0] * r2[:, 1] - r0[:, 1] * r2[:, 0]
    m2 = r0[:, 0] * r1[:, 1] - r0[:, 1] * r1[:, 0]
    det = (r0 * r0).sum(1) * m0 - (r1 * r1).sum(1) * m1 + (r2 * r2).sum(1) * m2
    assert (det <= 0).all(), f"{int((det > 0).sum())} edges not locally Delaunay"
    return {"vertices": v, "edges": int(len(edges)), "triangles": int(len(t)), "hull": h,
            "cocircular_edges": int((det == 0).sum()) // 2}


def hull_size_fast(points):
    """hull_size for large sets: strict monotone chain (Python loop over the
    sorted unique points), then the sites on each hull edge counted exactly
    by a vectorised collinearity test per edge."""
    pts = np.unique(np.asarray(points, np.int64), axis=0)  # sorted by x, then y
    if len(pts) < 3:
        return len(pts), np.zeros((0, 2), np.int64)

    def chain(seq):
        hh = []
        for q in seq:
            while len(hh) >= 2 and _orient(hh[-2], hh[-1], q) <= 0:
                hh.pop()
            hh.append(q)
        return hh
    # only points extreme in their column can be hull corners
    xs = pts[:, 0]
    first = np.r_[True, xs[1:] != xs[:-1]]
    last = np.r_[xs[1:] != xs[:-1], True]
    ext = [tuple(p) for p in pts[first | last].tolist()]
    lower, upper = chain(ext), chain(ext[::-1])
    corners = lower[:-1] + upper[:-1]
    if len(corners) < 3:
        return 0, np.zeros((0, 2), np.int64)
    cs = np.array(corners, np.int64)
    on = np.zeros(len(pts), bool)
    for e in range(len(cs)):
        a, b = cs[e], cs[(e + 1) % len(cs)]
        cr = (b[0] - a[0]) * (pts[:, 1] - a[1]) - (b[1] - a[1]) * (pts[:, 0] - a[0])
        inside = ((np.minimum(a[0], b[0]) <= pts[:, 0]) & (pts[:, 0] <= np.maximum(a[0], b[0])) &
                  (np.minimum(a[1], b[1]) <= pts[:, 1]) & (pts[:, 1] <= np.maximum(a[1], b[1])))
        on |= (cr == 0) & inside
    return int(on.sum()), cs


# ---------------------------------------------------------------------------
# Constrained Delaunay triangulations (the CDT stage's output)
# ---------------------------------------------------------------------------

def check_cdt(points, tris, segments, ranks):
    """Raise AssertionError unless tris is the constrained Delaunay
    triangulation of the integer points (V, 2) with the constraint segments
    (index pairs), under the symbolic perturbation by `ranks` (a larger rank
    perturbs more); returns a dict of counts.  Restates gDel2D's
    DelaunayChecker (gDel2D/DelaunayChecker.cpp:27-87 checkEuler, :99-144
    checkAdjacency, :146-169 checkOrientation, :171-213 checkDelaunay, which
    skips edges facing a constraint, and checkConstraints at :215-330, which
    looks every segment up as an edge; a segment through other points is the
    chain of edges between them) in exact Python integers, plus the
    coverage of the convex hull and the 2V - h - 2 triangle count.  With no
    unconstrained edge failing the perturbed incircle test and every segment
    an edge, the triangulation is the constrained Delaunay one (unique under
    the perturbation)."""
    pts = [(int(x), int(y)) for x, y in np.asarray(points).tolist()]
    T = [tuple(int(v) for v in t) for t in np.asarray(tris).reshape(-1, 3).tolist()]
    v = len(pts)
    h, corners = hull_size(np.asarray(points, np.int64))
    assert len(corners) >= 3, "collinear input"
    assert len(T) == 2 * v - h - 2, f"{len(T)} triangles, expected {2 * v - h - 2}"
    area = 0
    for a, b, c in T:
        assert 0 <= min(a, b, c) and max(a, b, c) < v, "index out of range"
        o = _orient(pts[a], pts[b], pts[c])
        assert o > 0, f"triangle {(a, b, c)} not counter-clockwise"
        area += o
    hull2 = sum(_orient(corners[0], corners[i], corners[i + 1]) for i in range(1, len(corners) - 1))
    assert area == hull2, "triangles do not tile the hull"
    opp = {}
    for t, (i, j, k) in enumerate(T):
        for e, w in (((i, j), k), ((j, k), i), ((k, i), j)):
            assert e not in opp, f"directed edge {e} twice"
            opp[e] = (t, w)
    edges = {tuple(sorted(e)) for e in opp}
    assert len({q for t in T for q in t}) == v, "points not in any triangle"
    assert v - len(edges) + len(T) == 1, "Euler characteristic"
    cons = set()
    for a, b in np.asarray(segments).reshape(-1, 2).tolist():
        # a segment with points exactly inside it is the chain of edges
        # between them
        pa, pb = pts[a], pts[b]
        dx, dy = pb[0] - pa[0], pb[1] - pa[1]
        inner = sorted((((q[0] - pa[0]) * dx + (q[1] - pa[1]) * dy), k) for k, q in enumerate(pts)
                       if k not in (a, b) and _orient(pa, pb, q) == 0
                       and 0 < (q[0] - pa[0]) * dx + (q[1] - pa[1]) * dy < dx * dx + dy * dy)
        chain = [a] + [k for _, k in inner] + [b]
        for u, w in zip(chain, chain[1:]):
            e = (min(u, w), max(u, w))
            assert e in edges, f"constraint segment {(a, b)}: {e} is not an edge"
            cons.add(e)
    ties = 0
    for (i, j), (t, w) in opp.items():
        if (j, i) not in opp or (min(i, j), max(i, j)) in cons:
            continue
        _, x = opp[(j, i)]
        assert not sos_in_circle(pts[i], pts[j], pts[w], pts[x], ranks[i], ranks[j], ranks[w],
                                 ranks[x]), f"edge {(i, j)} not locally Delaunay"
        det, _ = _incircle(pts[i], pts[j], pts[w], pts[x])
        ties += det == 0
    return {"vertices": v, "edges": len(edges), "triangles": len(T), "hull": h,
            "constraints": len(cons), "cocircular_edges": ties // 2}
