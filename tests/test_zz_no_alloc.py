"""The allocation-free labelling entry point (gcvt_label_grid_static).

It serves callers that cannot call cudaMalloc (code handed pre-allocated
device buffers by a host that owns the device memory, or a loop that must not
allocate after start-up): its scratch is one static device array, so the
caller passes only the site grid and the label grid.  Checked through the C
ABI against the allocating entry point (gcvt_label_grid) on two calls in a
row; labels are integer results, compared exactly.  This file is collected
last so that a stop-at-first-failure run has already run every other test."""
import ctypes

import numpy as np
import pytest

from workloads import disk_sites, gaussian_density

pytestmark = pytest.mark.gpu


def _static_label(lib, d_sites, d_out, n, stream=None):
    return lib.gcvt_label_grid_static(ctypes.c_void_p(d_sites.data_ptr()),
                                      ctypes.c_void_p(d_out.data_ptr()), n, stream)


def test_static_entry_matches_allocating_entry(gcvt_lib, cuda_device):
    import torch
    lib = gcvt_lib.load_library()
    for call, (n, seed) in enumerate(((2048, 3), (1024, 4))):
        rho = gaussian_density(n, 8, 4.0, 0.02, 0.15, seed=seed)
        sites = disk_sites(n, n * n // 64, seed=seed, density=rho)
        want = gcvt_lib.label_grid(sites)
        d_sites = torch.from_numpy(sites).to(cuda_device)
        d_out = torch.full_like(d_sites, 7)
        assert _static_label(lib, d_sites, d_out, n) == 0, call
        torch.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy(), want), call


def test_static_entry_limits(gcvt_lib, cuda_device):
    import torch
    lib = gcvt_lib.load_library()
    n = 4096
    d = torch.zeros((n, n, 2), dtype=torch.int16, device=cuda_device)
    assert _static_label(lib, d, d, n) == 2  # beyond the 2048 maximum
    assert lib.gcvt_label_grid_static(None, None, 256, None) == 1
    bad = torch.full((256, 256, 2), -32768, dtype=torch.int16, device=cuda_device)
    bad[5, 6, 0], bad[5, 6, 1] = 7, 5  # a site pixel holding foreign coordinates
    out = torch.empty_like(bad)
    assert _static_label(lib, bad, out, 256) == 4
