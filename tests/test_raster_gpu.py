"""GPU rasteriser parity: gcvt_rasterize (binned, min-index first hit) against
the oracle's restatement of kernelDiscretization and against the reference's
own kernel (compiled from discretization.cu).  Densities are compared bit for
bit: the first-hit decision and the FP64 interpolation follow the reference's
expressions."""
import numpy as np
import pytest

import oracle as orc
from workloads import disk_mesh, raster_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nv,n,seed,jitter", [(24, 256, 1, 0.3), (40, 256, 2, 0.45),
                                              (64, 512, 3, 0.3), (17, 512, 4, 0.0)])
def test_raster_equals_oracle(gcvt_lib, oracle, cuda_device, nv, n, seed, jitter):
    P, w, T = disk_mesh(nv, jitter=jitter, seed=seed)
    Q, scale, _, _ = raster_inputs(P, n)
    got = gcvt_lib.rasterize(Q, w, T, scale, n)
    want = oracle.rasterize(Q, w, T, scale, n)
    bad = np.argwhere(got.view(np.int32) != want.view(np.int32))
    assert bad.size == 0, (len(bad), bad[:3], got[tuple(bad[0])], want[tuple(bad[0])])


@pytest.mark.skipif(not orc.ref_available(), reason="reference cubins not built")
@pytest.mark.parametrize("nv,n,seed", [(24, 256, 5), (48, 512, 6)])
def test_raster_equals_reference_kernel(gcvt_lib, cuda_device, nv, n, seed):
    P, w, T = disk_mesh(nv, seed=seed)
    Q, scale, _, _ = raster_inputs(P, n)
    got = gcvt_lib.rasterize(Q, w, T, scale, n)
    ref, _ = orc.ref_rasterize(Q, w, T, scale, n)
    bad = np.argwhere(got.view(np.int32) != ref.view(np.int32))
    assert bad.size == 0, (len(bad), got[tuple(bad[0])], ref[tuple(bad[0])])


def test_raster_edge_cases(gcvt_lib, cuda_device):
    # shared edges and vertices exactly on pixel samples: the lower index wins
    n = 64
    pts = np.array([[0, 0], [63, 0], [0, 63], [63, 63], [31.5, 31.5]], np.float64)
    w = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    T = np.array([[0, 1, 4], [1, 3, 4], [3, 2, 4], [2, 0, 4], [0, 1, 3]], np.int32)
    got = gcvt_lib.rasterize(pts, w, T, 1.0, n)
    want = orc.rasterize(pts, w, T, 1.0, n)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
    # degenerate (zero-area) and empty inputs
    T2 = np.array([[0, 0, 1], [0, 1, 2]], np.int32)
    assert np.array_equal(gcvt_lib.rasterize(pts, w, T2, 1.0, n).view(np.int32),
                          orc.rasterize(pts, w, T2, 1.0, n).view(np.int32))
    z = gcvt_lib.rasterize(pts, w, np.zeros((0, 3), np.int32), 1.0, n)
    assert (z == 0).all()


def _same_f32(a, b):
    nan = np.isnan(a)
    return bool((nan == np.isnan(b)).all() and
                (a[~nan].view(np.int32) == b[~nan].view(np.int32)).all())


def test_raster_triangles_the_boxes_cannot_place(gcvt_lib, cuda_device):
    """Slivers whose rounded weights pass outside them, nearly collinear and
    negative-denominator triangles, a triangle larger than the tile limit, and
    one with a NaN vertex (its weights are NaN, which pass the test, so it
    takes every pixel no earlier triangle holds): all as the reference."""
    n = 2048
    rng = np.random.default_rng(8)
    base = [[100.0, 100.0], [1900.0, 100.0], [1000.0, 100.0 + 1e-7],      # sliver
            [200.0, 300.0], [1800.0, 300.0 + 1e-9], [1000.0, 300.0],      # near-collinear
            [0.0, 0.0], [2047.0, 0.0], [0.0, 2047.0],                     # whole-grid
            [np.nan, 50.0], [10.0, 20.0], [30.0, 40.0],                    # NaN vertex
            [500.0, 500.0], [1500.0, 700.0], [900.0, 1600.0]]              # ordinary
    pts = np.array(base, np.float64)
    w = rng.uniform(0.5, 2.0, len(pts))
    tris = np.array([[0, 1, 2], [3, 4, 5], [12, 13, 14], [6, 7, 8], [9, 10, 11]], np.int32)
    for order in (tris, tris[::-1].copy(), tris[[4, 0, 1, 2, 3]].copy()):
        got = gcvt_lib.rasterize(pts, w, order, 1.0, n)
        want = orc.rasterize(pts, w, order, 1.0, n)
        assert _same_f32(got, want)
    bad = tris.copy()
    bad[1, 2] = len(pts)
    with pytest.raises(RuntimeError):
        gcvt_lib.rasterize(pts, w, bad, 1.0, n)


def test_raster_slivers_across_conditioning(gcvt_lib, cuda_device):
    """Flat triangles whose height goes from 1e-1 to 1e-10 pixels (conditioning
    up to about 1e26), both orientations, over a regular background mesh."""
    n = 256
    rng = np.random.default_rng(12)
    pts, tris = [], []
    for k, h in enumerate(10.0 ** -np.arange(1, 11)):
        y0 = 10.0 + 23.0 * k
        b = len(pts)
        a, c = np.array([5.0, y0]), np.array([250.0, y0 + 0.37 * k])
        m = a + (0.45 + 0.01 * k) * (c - a) + np.array([0.0, h])   # h above the long edge
        pts += [a.tolist(), c.tolist(), m.tolist()]
        tris += [[b, b + 1, b + 2], [b + 1, b, b + 2]]
    b = len(pts)
    g = np.linspace(0, 255, 9)
    X, Y = np.meshgrid(g, g)
    pts += np.stack([X.ravel(), Y.ravel()], 1).tolist()
    for r in range(8):
        for c in range(8):
            a = b + r * 9 + c
            tris += [[a, a + 1, a + 10], [a, a + 10, a + 9]]
    pts = np.array(pts, np.float64)
    tris = np.array(tris, np.int32)
    w = rng.uniform(0.5, 2.0, len(pts))
    got = gcvt_lib.rasterize(pts, w, tris, 1.0, n)
    want = orc.rasterize(pts, w, tris, 1.0, n)
    assert _same_f32(got, want)
