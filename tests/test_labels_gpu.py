"""GPU labelling parity: the CUDA labeller against the oracle's literal PBA+
restatement (and the pointwise rule at sizes where the restatement is slow).
Labels are integer work: equality is bit-exact."""
import numpy as np
import pytest

from test_oracle import cases, grid
from workloads import MARKER, config_inputs, disk_sites, gaussian_density

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_labels_equal_pba_random_and_lattices(gcvt_lib, oracle, cuda_device, seed):
    for n, pts in cases(seed, 24):
        g = grid(n, pts)
        got = gcvt_lib.label_grid(g)
        want = oracle.pba_label(g)
        bad = np.argwhere((got != want).any(-1))
        assert bad.size == 0, (n, len(pts), bad[:3], got[tuple(bad[0])], want[tuple(bad[0])])


def test_labels_equal_pba_1024_dense(gcvt_lib, oracle, cuda_device):
    rng = np.random.default_rng(11)
    for m in (1, 3, 50, 4096, 60000):
        n = 1024
        pick = rng.choice(n * n, size=m, replace=False)
        ys, xs = np.divmod(pick, n)
        g = gcvt_lib.sites_from_points(n, xs, ys)
        assert np.array_equal(gcvt_lib.label_grid(g), oracle.pba_label(g)), m


@pytest.mark.parametrize("n", [2048, 4096])
def test_labels_large_against_pointwise_rule(gcvt_lib, oracle, cuda_device, n):
    rho = gaussian_density(n, 8, 4.0, 0.02, 0.15, seed=n)
    g = disk_sites(n, n * n // 64, seed=n, density=rho)
    assert np.array_equal(gcvt_lib.label_grid(g), oracle.spec_label(g))


def test_labels_non_power_of_two(gcvt_lib, oracle, cuda_device):
    rng = np.random.default_rng(3)
    n = 768
    pick = rng.choice(n * n, size=3000, replace=False)
    ys, xs = np.divmod(pick, n)
    g = gcvt_lib.sites_from_points(n, xs, ys)
    assert np.array_equal(gcvt_lib.label_grid(g), oracle.spec_label(g))


def test_full_row_and_full_column(gcvt_lib, oracle, cuda_device):
    n = 512
    pts = [(x, 77) for x in range(n)] + [(300, y) for y in range(n)]
    g = grid(n, sorted(set(pts)))
    assert np.array_equal(gcvt_lib.label_grid(g), oracle.pba_label(g))


def test_no_sites_gives_marker(gcvt_lib, cuda_device):
    g = np.full((256, 256, 2), MARKER, np.int16)
    out = gcvt_lib.label_grid(g)
    assert (out == MARKER).all()


def test_rejects_bad_grids(gcvt_lib, cuda_device):
    g = np.full((256, 256, 2), MARKER, np.int16)
    g[5, 6] = (7, 5)  # site pixel holding someone else's coordinates
    with pytest.raises(gcvt_lib.GcvtError) as e:
        gcvt_lib.label_grid(g)
    assert e.value.code == 4
    with pytest.raises(gcvt_lib.GcvtError) as e:
        gcvt_lib.label_grid(np.full((200, 200, 2), MARKER, np.int16))
    assert e.value.code == 2


def test_context_label_device_buffers(gcvt_lib, oracle, cuda_device):
    import torch
    sites, rho, mask, _ = config_inputs("plain_1024", seed=2)
    want = oracle.pba_label(sites)
    ctx = gcvt_lib.Context(1024)
    ctx.load(torch.from_numpy(sites).to(cuda_device), torch.from_numpy(rho).to(cuda_device),
             torch.from_numpy(mask).to(cuda_device))
    out = torch.empty((1024, 1024, 2), dtype=torch.int16, device=cuda_device)
    ctx.label(out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want)
    ctx.close()
