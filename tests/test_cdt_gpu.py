"""The constrained Delaunay stage on the GPU (gcvt_ctx_cdt), built as the
reference's pipeline builds its CDT input (main.cpp:211-236): a disk mesh is
rasterised into the density, its boundary vertices are the constraint points
-- fixed sites of the CVT at their pixels (generateMask, gcvt.h:141-158) and
left out of the free sites (delaunayInput, delaunay.h:46-67) -- and its
boundary edges are the constraint segments (delaunay.h:69-75).  The result
must pass the restated DelaunayChecker with its constraint check
(oracle/delaunay_oracle.py check_cdt) exactly, on the coordinates the
library's predicates use (sites on their pixel lattice, constraint points
rounded to 2^-15 pixel)."""
import re

import numpy as np
import pytest

import delaunay_oracle as D
from workloads import (area_weights, disk_sites, disk_surface, mesh_constraints, raster_inputs,
                       small_case)

pytestmark = pytest.mark.gpu


def exact_points(ctx, n, cpoints, scale, left, lower):
    """The integer coordinates and perturbation ranks the library uses."""
    sp = ctx.extract_points().astype(np.int64)
    cx = np.rint((cpoints[:, 0] - left) / scale * 32768.0).astype(np.int64)
    cy = np.rint((cpoints[:, 1] - lower) / scale * 32768.0).astype(np.int64)
    X = np.concatenate([sp[:, 0] << 15, cx])
    Y = np.concatenate([sp[:, 1] << 15, cy])
    R = np.concatenate([sp[:, 1] * n + sp[:, 0], n * n + np.arange(len(cpoints))])
    return np.stack([X, Y], 1), R, len(sp)


def mesh_case(gcvt_lib, nv, n, m, iters, seed=2):
    uv, xyz, tris = disk_surface(nv, seed=seed)
    Q, scale, left, lower = raster_inputs(uv, n)
    rho = gcvt_lib.rasterize(Q, area_weights(uv, xyz, tris), tris, scale, n)
    bv, be, px, py = mesh_constraints(uv, tris, scale, left, lower)
    mask = np.zeros((n, n), np.uint8)
    mask[py, px] = 1
    sites = disk_sites(n, m, seed, rho)
    sites[py, px, 0] = px
    sites[py, px, 1] = py
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    ctx.iterate(iters)
    return ctx, uv[bv], be, bv, scale, left, lower


@pytest.mark.parametrize("nv,n,m,iters", [(24, 256, 500, 10), (64, 512, 3000, 20),
                                          (128, 1024, 12000, 30),
                                          # the mesh workload's size: a 256^2-vertex disk
                                          # mesh on a 2048^2 grid, 65,536 sites
                                          (256, 2048, 65536, 100)])
def test_mesh_boundary_cdt_is_constrained_delaunay(gcvt_lib, cuda_device, nv, n, m, iters):
    ctx, cpts, be, bv, scale, left, lower = mesh_case(gcvt_lib, nv, n, m, iters)
    pts, R, F = exact_points(ctx, n, cpts, scale, left, lower)
    pos = {int(v): k for k, v in enumerate(bv)}
    segs = np.array([(F + pos[int(a)], F + pos[int(b)]) for a, b in be], np.int64)
    tri, detail = ctx.cdt(scale, left, lower, cpts, segs)
    assert detail == 0
    info = D.check_cdt(pts, tri, segs, R.tolist())
    assert info["vertices"] == F + len(cpts)
    assert info["constraints"] >= len(segs)
    # the output order is fixed: triangles start at their smallest index,
    # sorted by it and then the second
    assert (tri[:, 0] < tri[:, 1]).all() and (tri[:, 0] < tri[:, 2]).all()
    key = tri[:, 0].astype(np.int64) * len(pts) + tri[:, 1]
    assert (np.diff(key) > 0).all()
    again, _ = ctx.cdt(scale, left, lower, cpts, segs)
    assert np.array_equal(again, tri)
    ctx.close()


def test_cdt_without_constraints_is_the_delaunay_triangulation(gcvt_lib, cuda_device):
    sites, rho, mask = small_case(512, 2500, 71)
    ctx = gcvt_lib.Context(512)
    ctx.load(sites, rho, mask)
    ctx.iterate(15)
    dt = D.canonical(ctx.delaunay())
    tri, _ = ctx.cdt(1.0, 0.0, 0.0, np.zeros((0, 2)), np.zeros((0, 2), np.int32))
    assert D.canonical(tri) == dt
    ctx.close()


def test_cdt_rejects_crossing_segments(gcvt_lib, cuda_device):
    sites, rho, mask = small_case(256, 400, 72)
    ctx = gcvt_lib.Context(256)
    ctx.load(sites, rho, mask)
    F = len(ctx.extract_points())
    c = np.array([(60.5, 128.3), (190.5, 127.7), (128.4, 60.2), (127.6, 190.1)])
    with pytest.raises(gcvt_lib.GcvtError) as e:
        ctx.cdt(1.0, 0.0, 0.0, c, np.array([(F, F + 1), (F + 2, F + 3)]))
    assert e.value.code == 4 and detail_of(e.value) == 16
    ctx.close()


def detail_of(err):
    m = re.search(r"detail (\d+)", str(err))
    return int(m.group(1)) if m else None


def loaded(gcvt_lib, n, m, seed, iters=5):
    sites, rho, mask = small_case(n, m, seed)
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    ctx.iterate(iters)
    return ctx, ctx.extract_points()


@pytest.mark.parametrize("case", ["on_site", "twice", "far", "bad_pair", "same_pair"])
def test_cdt_rejects_invalid_input(gcvt_lib, cuda_device, case):
    # each reason of the detail mask: a constraint point on a site (2) or on
    # another constraint point (2), beyond the coordinate range (1), a segment
    # index out of range or a segment from a point to itself (16)
    ctx, sp = loaded(gcvt_lib, 256, 400, 73)
    F = len(sp)
    c = np.array([(100.3, 120.7), (150.6, 130.2)])
    s = np.array([(F, F + 1)])
    want = 2
    if case == "on_site":
        c[0] = sp[len(sp) // 2]
    elif case == "twice":
        c[1] = c[0]
    elif case == "far":
        c[1] = (40000.0, 128.0)
        want = 1
    elif case == "bad_pair":
        s = np.array([(F, F + 2)])
        want = 16
    else:
        s = np.array([(F + 1, F + 1)])
        want = 16
    with pytest.raises(gcvt_lib.GcvtError) as e:
        ctx.cdt(1.0, 0.0, 0.0, c, s)
    assert e.value.code == 4 and detail_of(e.value) == want
    # the context stays usable: valid input afterwards gives a valid result
    good = np.array([(100.3, 120.7), (150.6, 130.2)])
    tri, detail = ctx.cdt(1.0, 0.0, 0.0, good, np.array([(F, F + 1)]))
    pts, R, _ = exact_points(ctx, 256, good, 1.0, 0.0, 0.0)
    assert detail == 0 and D.check_cdt(pts, tri, np.array([(F, F + 1)]), R.tolist())
    ctx.close()


def test_cdt_counts_without_writing_past_the_capacity(gcvt_lib, cuda_device):
    ctx, sp = loaded(gcvt_lib, 256, 300, 74)
    F = len(sp)
    c = np.array([(60.25, 70.5), (190.75, 180.25)])
    full, _ = ctx.cdt(1.0, 0.0, 0.0, c, np.array([(F, F + 1)]))
    part, _ = ctx.cdt(1.0, 0.0, 0.0, c, np.array([(F, F + 1)]), capacity=10)
    assert len(part) == 10 and np.array_equal(part, full[:10])
    ctx.close()


def test_cdt_of_segments_between_sites_and_across_the_hull(gcvt_lib, cuda_device):
    # segments between free sites (not Delaunay edges), and constraint points
    # outside the sites' hull joined to sites inside it
    ctx, sp = loaded(gcvt_lib, 256, 500, 75, iters=10)
    F = len(sp)
    rng = np.random.default_rng(75)
    c = np.array([(-20.3, 128.1), (276.4, 127.6), (128.2, -15.7), (127.9, 271.3)])
    pairs = []
    for _ in range(6):  # site pairs about 40 px apart: many crossing edges
        a = int(rng.integers(F))
        d = np.hypot(*(sp - sp[a]).T)
        b = int(np.argmin(np.abs(d - 40.0)))
        pairs.append((a, b))
    near = [int(np.argmin(np.hypot(*(sp - q).T))) for q in c]
    segs = np.array(pairs + [(F + k, near[k]) for k in range(4)])
    try:
        tri, detail = ctx.cdt(1.0, 0.0, 0.0, c, segs)
    except gcvt_lib.GcvtError as e:  # random pairs may cross each other
        assert e.code == 4 and detail_of(e) == 16
        segs = segs[6:]
        tri, detail = ctx.cdt(1.0, 0.0, 0.0, c, segs)
    pts, R, _ = exact_points(ctx, 256, c, 1.0, 0.0, 0.0)
    info = D.check_cdt(pts, tri, segs, R.tolist())
    assert info["vertices"] == F + 4 and info["constraints"] >= len(segs)
    ctx.close()


def test_cdt_of_too_few_points_is_empty(gcvt_lib, cuda_device):
    n = 256
    sites = np.full((n, n, 2), -32768, np.int16)
    for x, y in ((10, 20), (200, 30)):
        sites[y, x] = (x, y)
    rho = np.ones((n, n), np.float32)
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, np.zeros((n, n), np.uint8))
    tri, detail = ctx.cdt(1.0, 0.0, 0.0, np.zeros((0, 2)), np.zeros((0, 2), np.int32))
    assert len(tri) == 0 and detail == 0
    ctx.close()
