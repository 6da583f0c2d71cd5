"""The GPU Delaunay triangulation of a context's free sites
(gcvt_ctx_delaunay) against the oracle: on small site sets the very
triangles of the symbolic perturbation (brute force over all triples), on
CVT-sized sets the checks of gDel2D's DelaunayChecker restated in exact
integers (orientation, adjacency, Euler, local Delaunay, hull coverage,
2V - h - 2 triangles), and against scipy's Qhull where no four sites of
adjacent triangles are co-circular (the triangulation is then unique)."""
import numpy as np
import pytest

import delaunay_oracle as dorc
from workloads import MARKER, disk_mask, small_case

pytestmark = pytest.mark.gpu


def _grid(n, pts):
    g = np.full((n, n, 2), MARKER, np.int16)
    for x, y in pts:
        g[y, x] = (x, y)
    return g


def _triangulate(gcvt_lib, sites, mask=None, rho=None, iters=0):
    n = sites.shape[0]
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, np.ones((n, n), np.float32) if rho is None else rho,
             np.zeros((n, n), np.uint8) if mask is None else mask)
    if iters:
        ctx.iterate(iters)
    pts = ctx.extract_points().astype(np.int64)
    tris = ctx.delaunay()
    part = ctx.delaunay(capacity=5)
    ctx.close()
    assert np.array_equal(part, tris[:5])
    return pts, tris


def _small_sets():
    rng = np.random.default_rng(7)
    sets = []
    for s in range(4):  # random
        sets.append(("random%d" % s, [tuple(p) for p in rng.integers(20, 230, (45, 2))]))
    # lattice blocks: every square's four corners co-circular
    sets.append(("grid", [(x, y) for x in range(40, 100, 10) for y in range(50, 110, 10)]))
    sets.append(("grid_dense", [(x, y) for x in range(100, 107) for y in range(3, 10)]))
    # twelve sites on one circle (radius 5) and its centre
    ring = [(5, 0), (0, 5), (-5, 0), (0, -5), (3, 4), (4, 3), (-3, 4), (-4, 3), (3, -4),
            (4, -3), (-3, -4), (-4, -3), (0, 0)]
    sets.append(("ring", [(128 + x, 128 + y) for x, y in ring]))
    # rectangle border with collinear sites on every edge, a few inside
    border = [(x, 30) for x in range(30, 200, 17)] + [(x, 180) for x in range(30, 200, 17)]
    border += [(30, y) for y in range(47, 180, 19)] + [(183, y) for y in range(47, 180, 19)]
    sets.append(("border", border + [(90, 90), (120, 140), (60, 150)]))
    # three sites, a near-degenerate sliver, the grid's corners
    sets.append(("three", [(0, 0), (255, 0), (0, 255)]))
    sets.append(("sliver", [(10, 10), (240, 11), (125, 12), (60, 200)]))
    sets.append(("corners", [(0, 0), (255, 0), (0, 255), (255, 255), (128, 128)]))
    return sets


@pytest.mark.parametrize("name,pts", _small_sets(), ids=lambda v: v if isinstance(v, str) else "")
def test_small_sets_match_the_perturbed_triangulation(gcvt_lib, cuda_device, name, pts):
    n = 256
    pts = sorted(set(pts))
    got_pts, tris = _triangulate(gcvt_lib, _grid(n, pts))
    assert [tuple(p) for p in got_pts.tolist()] == pts  # x-major, then y
    want = dorc.sos_triangulation(got_pts, n)
    assert dorc.canonical(tris) == [tuple(r) for r in want.tolist()]
    dorc.check(got_pts, tris)


def test_random_small_sets_match_the_perturbed_triangulation(gcvt_lib, cuda_device):
    """Forty seeded small sets: uniform, clustered in the grid's corners and
    on a coarse lattice (many co-circular quadruples)."""
    rng = np.random.default_rng(12)
    for trial in range(40):
        n = int(rng.choice([256, 512]))
        m = int(rng.integers(3, 45))
        kind = trial % 3
        if kind == 0:
            pts = rng.integers(0, n, (m, 2))
        elif kind == 1:
            pts = np.concatenate([rng.integers(0, 6, (m // 2, 2)),
                                  rng.integers(n - 6, n, (m - m // 2, 2))])
        else:
            pts = rng.integers(0, 8, (m, 2)) * (n // 8)
        pts = sorted(set((int(x), int(y)) for x, y in pts))
        got_pts, tris = _triangulate(gcvt_lib, _grid(n, pts))
        want = dorc.sos_triangulation(got_pts, n)
        assert dorc.canonical(tris) == [tuple(r) for r in want.tolist()], (trial, n, kind)


@pytest.mark.parametrize("pts", [[], [(5, 5)], [(5, 5), (200, 7)],
                                 [(x, 2 * x + 3) for x in range(0, 120, 7)],
                                 [(77, y) for y in range(0, 256, 5)]])
def test_fewer_than_three_or_collinear_sites_give_no_triangles(gcvt_lib, cuda_device, pts):
    _, tris = _triangulate(gcvt_lib, _grid(256, pts))
    assert tris.shape == (0, 3)


@pytest.mark.parametrize("n,m,iters", [(256, 500, 0), (512, 3000, 10), (1024, 12000, 20)])
def test_cvt_sites_pass_the_delaunay_checks(gcvt_lib, cuda_device, n, m, iters):
    sites, rho, mask = small_case(n, m, seed=41)
    pts, tris = _triangulate(gcvt_lib, sites, mask, rho, iters)
    info = dorc.check(pts, tris)
    assert info["vertices"] == len(pts) > 0
    if info["cocircular_edges"] == 0:
        spatial = pytest.importorskip("scipy.spatial")
        q = spatial.Delaunay(pts.astype(np.float64)).simplices
        a, b, c = pts[q[:, 0]], pts[q[:, 1]], pts[q[:, 2]]
        o = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
        q[o < 0] = q[o < 0][:, [0, 2, 1]]
        assert dorc.canonical(tris) == dorc.canonical(q)


def test_fixed_sites_are_left_out(gcvt_lib, cuda_device):
    n = 512
    sites, rho, mask = small_case(n, 2000, seed=43)
    ys, xs = np.nonzero(sites[..., 0] != MARKER)
    mask[ys[:200], xs[:200]] = 1
    pts, tris = _triangulate(gcvt_lib, sites, mask, rho, 5)
    assert 0 < len(pts) <= 2000 - 200  # free sites only (moved ones may merge)
    dorc.check(pts, tris)


def test_every_pixel_a_site(gcvt_lib, cuda_device):
    """65,536 sites on the full lattice: every unit square co-circular."""
    n = 256
    X, Y = np.meshgrid(np.arange(n), np.arange(n))
    sites = np.stack([X, Y], -1).astype(np.int16)
    pts, tris = _triangulate(gcvt_lib, sites)
    assert len(tris) == 2 * n * n - (4 * n - 4) - 2
    dorc.check(pts, tris)


def test_disk_of_sites_with_wide_gaps(gcvt_lib, cuda_device):
    """Sites inside a disk and a few far outside it: long thin triangles
    whose circumcircles need windows much wider than the site spacing."""
    n = 1024
    rng = np.random.default_rng(44)
    inside = np.argwhere(disk_mask(n, 0.2))
    pick = inside[rng.choice(len(inside), 3000, replace=False)]
    pts = [(int(x), int(y)) for y, x in pick] + [(3, 1000), (1020, 4), (1010, 1015), (2, 2)]
    pts_got, tris = _triangulate(gcvt_lib, _grid(n, pts))
    dorc.check(pts_got, tris)


def test_star_overflow_is_an_input_error(gcvt_lib, cuda_device):
    """A site with more than 64 Delaunay neighbours (the centre of 108
    co-circular lattice sites, radius 1105) fails with GCVT_ERR_INPUT and
    leaves the context usable."""
    n = 4096
    r2 = 1105 ** 2
    ring = set()
    for x in range(-1105, 1106):
        y = int(round((r2 - x * x) ** 0.5))
        if x * x + y * y == r2:
            ring |= {(x, y), (x, -y)}
    assert len(ring) == 108
    pts = [(2048 + x, 2048 + y) for x, y in ring] + [(2048, 2048)]
    ctx = gcvt_lib.Context(n)
    ctx.load(_grid(n, pts), np.ones((n, n), np.float32), np.zeros((n, n), np.uint8))
    with pytest.raises(gcvt_lib.GcvtError) as e:
        ctx.delaunay()
    assert e.value.code == 4  # GCVT_ERR_INPUT
    ctx.load(_grid(n, [(10, 10), (300, 40), (100, 500)]), np.ones((n, n), np.float32),
             np.zeros((n, n), np.uint8))
    assert ctx.delaunay().shape == (1, 3)
    ctx.close()


def test_device_output_equals_host_output(gcvt_lib, cuda_device):
    import ctypes
    import torch
    sites, rho, mask = small_case(512, 2500, seed=45)
    ctx = gcvt_lib.Context(512)
    ctx.load(sites, rho, mask)
    ctx.iterate(6)
    host = ctx.delaunay()
    d = torch.full((len(host) + 7, 3), -1, dtype=torch.int32, device="cuda")
    cnt = ctypes.c_int(0)
    rc = gcvt_lib.load_library().gcvt_ctx_delaunay(ctx.h, d.data_ptr(), len(d), ctypes.byref(cnt),
                                                    gcvt_lib.MEM_DEVICE)
    assert rc == 0 and cnt.value == len(host)
    assert np.array_equal(d[:len(host)].cpu().numpy(), host)
    assert (d[len(host):] == -1).all()
    ctx.close()


@pytest.mark.parametrize("workload", ["plain_4096", "plain_8192"])
def test_full_size_workloads_pass_the_checks(gcvt_lib, cuda_device, workload):
    """The benchmark workloads at full size (262,144 and 1,048,576 sites after
    their Lloyd iterations): every property of the restated DelaunayChecker,
    vectorised."""
    from workloads import config_inputs
    sites, rho, mask, iters = config_inputs(workload)
    n = sites.shape[0]
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    ctx.iterate(iters)
    pts = ctx.extract_points().astype(np.int64)
    tris = ctx.delaunay()
    ctx.close()
    info = dorc.check_fast(pts, tris)
    assert info["vertices"] == len(pts) and info["triangles"] == len(tris)
