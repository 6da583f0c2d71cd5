"""The Delaunay oracle on the CPU: the perturbed brute-force triangulation
equals scipy's Qhull where the triangulation is unique, passes the restated
DelaunayChecker where it is not, and the restated checks reject planted mistakes."""
import numpy as np
import pytest

import delaunay_oracle as dorc


def _random(seed, count=40, n=4096):
    pts = np.unique(np.random.default_rng(seed).integers(0, n, (count, 2)), axis=0)
    return pts[np.lexsort((pts[:, 1], pts[:, 0]))]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_brute_force_equals_qhull_on_random_sites(seed):
    spatial = pytest.importorskip("scipy.spatial")
    pts = _random(seed)
    got = dorc.sos_triangulation(pts, 4096)
    assert dorc.check(pts, got)["cocircular_edges"] == 0
    q = spatial.Delaunay(pts.astype(np.float64)).simplices
    a, b, c = pts[q[:, 0]], pts[q[:, 1]], pts[q[:, 2]]
    o = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    q[o < 0] = q[o < 0][:, [0, 2, 1]]
    assert dorc.canonical(q) == [tuple(r) for r in got.tolist()]


def test_lattice_block_is_one_valid_triangulation():
    pts = np.array([(x, y) for x in range(0, 12, 2) for y in range(3, 15, 2)])
    got = dorc.sos_triangulation(pts, 256)
    info = dorc.check(pts, got)
    assert info["triangles"] == 2 * 36 - 20 - 2 and info["cocircular_edges"] == 25


def test_delaunay_checks_reject_planted_mistakes():
    pts = _random(5)
    good = dorc.sos_triangulation(pts, 4096)
    dorc.check(pts, good)
    with pytest.raises(AssertionError):  # a triangle missing
        dorc.check(pts, good[1:])
    bad = good.copy()
    bad[0] = bad[0][[0, 2, 1]]
    with pytest.raises(AssertionError):  # clockwise
        dorc.check(pts, bad)
    # flip one interior edge: still a triangulation, no longer Delaunay
    tris = [tuple(t) for t in good.tolist()]
    edge = {}
    for t, (i, j, k) in enumerate(tris):
        for e, w in (((i, j), k), ((j, k), i), ((k, i), j)):
            edge[e] = (t, w)
    for (i, j), (t, w) in edge.items():
        if (j, i) not in edge:
            continue
        u, x = edge[(j, i)]
        if dorc._orient(pts[w], pts[i], pts[x]) > 0 and dorc._orient(pts[x], pts[j], pts[w]) > 0:
            flipped = [tr for q, tr in enumerate(tris) if q not in (t, u)]
            flipped += [(w, i, x), (x, j, w)]
            with pytest.raises(AssertionError, match="locally Delaunay"):
                dorc.check(pts, flipped)
            return
    pytest.fail("no flippable edge")


@pytest.mark.parametrize("seed", [7, 8, 9])
def test_vectorised_checks_agree_and_reject(seed):
    rng = np.random.default_rng(seed)
    pts = np.unique(rng.integers(0, 30, (50, 2)), axis=0)  # dense: many ties
    pts = pts[np.lexsort((pts[:, 1], pts[:, 0]))]
    good = dorc.sos_triangulation(pts, 64)
    assert dorc.check_fast(pts, good) == dorc.check(pts, good)
    with pytest.raises(AssertionError):
        dorc.check_fast(pts, good[1:])
    bad = good.copy()
    bad[0] = bad[0][[0, 2, 1]]
    with pytest.raises(AssertionError):
        dorc.check_fast(pts, bad)
