"""Jump-flooding labels (gcvt_ctx_jfa_label) equal a numpy restatement of the
same schedule (n/2 ... 1 plus 1, nine neighbours at offset k, ties to the
smaller x then y) bit for bit -- large steps with 128-bit accesses and the
fused TMA tail included -- and their error against the exact labels is
reported: pixels with a different label and pixels with a strictly farther
site."""
import numpy as np
import pytest

from workloads import MARKER, disk_sites, gaussian_density, small_case

pytestmark = pytest.mark.gpu

NONE = np.uint32(0x80008000)


def jfa_numpy(sites):
    n = sites.shape[0]
    lab = np.ascontiguousarray(sites).view(np.uint32).reshape(n, n).copy()
    Y, X = np.mgrid[0:n, 0:n]
    ks, k = [], 1
    while 2 * k <= n // 2:
        k *= 2
    while k >= 1:
        ks.append(k)
        k //= 2
    ks.append(1)
    for k in ks:
        best = np.full((n, n), NONE, np.uint32)
        bd = np.full((n, n), np.iinfo(np.int64).max, np.int64)
        bx = np.zeros((n, n), np.int64)
        by = np.zeros((n, n), np.int64)
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.full((n, n), NONE, np.uint32)
                ys, yd = slice(max(0, dy * k), n + min(0, dy * k)), slice(max(0, -dy * k), n + min(0, -dy * k))
                xs, xd = slice(max(0, dx * k), n + min(0, dx * k)), slice(max(0, -dx * k), n + min(0, -dx * k))
                sh[yd, xd] = lab[ys, xs]
                cx = (sh & 0xffff).astype(np.uint16).view(np.int16).astype(np.int64)
                cy = (sh >> 16).astype(np.uint16).view(np.int16).astype(np.int64)
                d = (cx - X) ** 2 + (cy - Y) ** 2
                ok = sh != NONE
                better = ok & ((d < bd) | ((d == bd) & ((cx < bx) | ((cx == bx) & (cy < by)))))
                best = np.where(better, sh, best)
                bd = np.where(better, d, bd)
                bx = np.where(better, cx, bx)
                by = np.where(better, cy, by)
        lab = best
    return lab.view(np.int16).reshape(n, n, 2)


@pytest.mark.parametrize("n,m,seed", [(256, 300, 1), (512, 4000, 2), (1024, 20000, 3), (768, 1500, 4)])
def test_jfa_matches_numpy(gcvt_lib, cuda_device, n, m, seed):
    if n & (n - 1):  # not a power of two: uniform sites, unit density
        sites = np.full((n, n, 2), MARKER, np.int16)
        rng = np.random.default_rng(seed)
        pick = rng.choice(n * n, m, replace=False)
        ys, xs = np.divmod(pick, n)
        sites[ys, xs, 0], sites[ys, xs, 1] = xs, ys
        rho = np.ones((n, n), np.float32)
    else:
        sites, rho, _ = small_case(n, m, seed)
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, np.zeros((n, n), np.uint8))
    got, (diff, far, px) = ctx.jfa_label()
    want = jfa_numpy(sites)
    assert np.array_equal(got, want)
    exact = ctx.label()
    assert px == n * n
    assert diff == int((got != exact).any(-1).sum())
    assert far <= diff and far < 0.01 * px
    ctx.close()


@pytest.mark.parametrize("halo", [0, 8, 32])
@pytest.mark.parametrize("n,m,seed", [(512, 4000, 6), (768, 1500, 7)])
def test_every_fusion_depth_matches_numpy(gcvt_lib, cuda_device, halo, n, m, seed):
    # the fused tail (halo 8 / 32) and one launch per step (halo 0) give the same labels
    rng = np.random.default_rng(seed)
    sites = np.full((n, n, 2), MARKER, np.int16)
    pick = rng.choice(n * n, m, replace=False)
    ys, xs = np.divmod(pick, n)
    sites[ys, xs, 0], sites[ys, xs, 1] = xs, ys
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, np.ones((n, n), np.float32), np.zeros((n, n), np.uint8))
    ctx.set_tuning(jfa_tail_halo=halo)
    got, _ = ctx.jfa_label()
    assert np.array_equal(got, jfa_numpy(sites))
    ctx.close()


def test_jfa_error_on_clustered_sites(gcvt_lib, cuda_device):
    # dense clusters are where jump flooding errs; the count stays small
    n = 512
    rho = gaussian_density(n, 4, 8.0, 0.01, 0.03, seed=5)
    sites = disk_sites(n, 8000, 5, rho)
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, np.zeros((n, n), np.uint8))
    got, (diff, far, px) = ctx.jfa_label()
    assert np.array_equal(got, jfa_numpy(sites))
    assert far < 0.01 * px
    ctx.close()
