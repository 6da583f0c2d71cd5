"""CDT input points (delaunay.h:46-57) extracted on the GPU equal the host
loop over the label grid: free sites, x-major then y order, FP64
(x * scale + left, y * scale + lower)."""
import numpy as np
import pytest

from workloads import MARKER, small_case

pytestmark = pytest.mark.gpu


def host_points(labels, mask, scale, left, lower):
    n = labels.shape[0]
    pts = []
    for i in range(n):          # x outer, y inner, as delaunayInput loops
        col = labels[:, i]
        for j in np.nonzero((col[:, 0] == i) & (col[:, 1] == np.arange(n)) & (mask[:, i] == 0))[0]:
            pts.append((i * scale + left, int(j) * scale + lower))
    return np.array(pts, np.float64).reshape(-1, 2)


@pytest.mark.parametrize("n,m,iters,fixed", [(256, 300, 5, 0), (512, 3000, 12, 50)])
def test_extract_matches_host_loop(gcvt_lib, cuda_device, n, m, iters, fixed):
    sites, rho, mask = small_case(n, m, seed=21)
    if fixed:
        ys, xs = np.nonzero(sites[..., 0] != MARKER)
        mask[ys[:fixed], xs[:fixed]] = 1
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    ctx.iterate(iters)
    labels = ctx.label()
    scale, left, lower = 0.0123456789, -0.31, 0.017
    got = ctx.extract_points(scale, left, lower)
    want = host_points(labels, mask, scale, left, lower)
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    # truncated output reports the full count
    part = ctx.extract_points(scale, left, lower, capacity=10)
    assert np.array_equal(part, want[:10])
    ctx.close()
