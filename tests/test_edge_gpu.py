"""Edge cases of the gCVT loop on the GPU against the oracle's exact mode:
no sites, one site, zero density, sites on the density's edge, maxIter = 0
(the reference's do-while still runs one iteration), two sites moving to one
pixel (they merge), and every pixel a site."""
import numpy as np
import pytest

from workloads import MARKER, disk_mask, small_case

pytestmark = pytest.mark.gpu


def _grid(n, pts):
    g = np.full((n, n, 2), MARKER, np.int16)
    for x, y in pts:
        g[y, x] = (x, y)
    return g


def _compare(gcvt_lib, oracle, sites, rho, mask, iters):
    n = sites.shape[0]
    want, st = oracle.gcvt(sites, rho, mask, 1, iters, mode=oracle.EXACT, fixed_iters=iters)
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    ctx.iterate(iters)
    got = ctx.label()
    info = ctx.info()
    ctx.close()
    return got, want, info


def test_no_sites(gcvt_lib, oracle, cuda_device):
    n = 256
    sites = np.full((n, n, 2), MARKER, np.int16)
    rho = np.ones((n, n), np.float32)
    mask = np.zeros((n, n), np.uint8)
    got, want, info = _compare(gcvt_lib, oracle, sites, rho, mask, 5)
    assert (got == MARKER).all() and np.array_equal(got, want)
    out = gcvt_lib.gcvt(sites.copy(), rho, mask, 1, 20)
    assert (out == MARKER).all()


def test_one_site_oscillates_across_the_centroid(gcvt_lib, oracle, cuda_device):
    """One site owns the whole disk; with the first iterations' omega = 2 it
    jumps to the mirror image of its position about the centroid and back."""
    n = 256
    rho = disk_mask(n).astype(np.float32)
    sites = _grid(n, [(40, 200)])
    mask = np.zeros((n, n), np.uint8)
    for iters, where in ((5, (215, 55)), (6, (40, 200))):
        got, want, _ = _compare(gcvt_lib, oracle, sites, rho, mask, iters)
        assert np.array_equal(got, want)
        assert tuple(int(v) for v in got[0, 0]) == where


def test_zero_density_keeps_sites(gcvt_lib, oracle, cuda_device):
    n = 256
    sites, _, mask = small_case(n, 100, seed=31)
    rho = np.zeros((n, n), np.float32)
    got, want, _ = _compare(gcvt_lib, oracle, sites, rho, mask, 4)
    assert np.array_equal(got, want)
    assert np.array_equal(got, oracle.pba_label(sites))


def test_sites_on_the_support_edge(gcvt_lib, oracle, cuda_device):
    """Sites on the last density pixels of their rows and columns: their
    cells are open towards the empty region (the covering bound limits them)."""
    n = 512
    rho = disk_mask(n).astype(np.float32) * 2.0
    ys, xs = np.nonzero(rho)
    edge = []
    for y in range(0, n, 23):
        row = xs[ys == y]
        if len(row):
            edge += [(int(row.min()), y), (int(row.max()), y)]
    sites = _grid(n, edge + [(256, 256), (200, 300)])
    got, want, _ = _compare(gcvt_lib, oracle, sites, rho, np.zeros((n, n), np.uint8), 12)
    assert (got == want).all(-1).mean() > 0.999


def test_max_iter_zero_runs_one_iteration(gcvt_lib, oracle, cuda_device):
    sites, rho, mask = small_case(256, 300, seed=32)
    want, st = oracle.gcvt(sites, rho, mask, 1, 0, mode=oracle.EXACT)
    ctx = gcvt_lib.Context(256)
    ctx.load(sites, rho, mask)
    info = ctx.run(1, 0)
    assert info["iterations"] == st["iterations"] == 1
    assert (ctx.label() == want).all(-1).mean() > 0.999
    ctx.close()


def test_colliding_moves_merge(gcvt_lib, oracle, cuda_device):
    """A site grid where two sites move to one pixel in the first iteration:
    they merge, as the reference's scatter does (one site less)."""
    n = 256
    sites, rho, mask = small_case(n, 527, seed=101)
    got, want, _ = _compare(gcvt_lib, oracle, sites, rho, mask, 1)
    assert np.array_equal(got, want)
    assert len(np.unique(got.reshape(-1, 2), axis=0)) == 526


def test_every_pixel_a_site(gcvt_lib, oracle, cuda_device):
    n = 256
    X, Y = np.meshgrid(np.arange(n), np.arange(n))
    sites = np.stack([X, Y], -1).astype(np.int16)
    rho = np.ones((n, n), np.float32)
    mask = np.zeros((n, n), np.uint8)
    got, want, _ = _compare(gcvt_lib, oracle, sites, rho, mask, 2)
    assert np.array_equal(got, want)
