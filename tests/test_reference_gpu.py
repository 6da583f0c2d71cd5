"""Pins the oracle to the reference itself: the reference's kernels, compiled
from its own sources into oracle/_ref/*.cubin and driven by the host sequence
of gcvt.cu (oracle/ref_harness.c), against the oracle's restatement -- and so,
transitively, against the CUDA library."""
import numpy as np
import pytest

import oracle as orc
from test_oracle import cases, grid
from workloads import small_case

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not orc.ref_available(), reason="reference cubins not built")]


@pytest.mark.parametrize("seed", [0, 3])
def test_reference_labels_equal_oracle(oracle, cuda_device, seed):
    for n, pts in cases(seed, 18):
        g = grid(n, pts)
        assert np.array_equal(orc.ref_pba_label(g), oracle.pba_label(g)), (n, len(pts))


def test_reference_labels_equal_library(gcvt_lib, cuda_device):
    sites, rho, mask = small_case(1024, 5000, seed=31)
    assert np.array_equal(orc.ref_pba_label(sites), gcvt_lib.label_grid(sites))


def test_reference_energy_equals_faithful_oracle(oracle, cuda_device):
    for n, m, seed in ((256, 300, 1), (1024, 4096, 2)):
        sites, rho, mask = small_case(n, m, seed)
        lab = oracle.pba_label(sites)
        assert orc.ref_energy(lab, rho) == oracle.faithful_energy(lab, rho)


def test_reference_trajectory_close_to_oracle(oracle, cuda_device):
    sites, rho, mask = small_case(256, 300, seed=5)
    r, info = orc.ref_gcvt(sites, rho, mask, 1, 30, fixed_iters=30)
    f, st = oracle.gcvt(sites, rho, mask, 1, 30, mode=oracle.FAITHFUL, fixed_iters=30)
    assert info["iterations"] == st["iterations"] == 30
    assert (r == f).all(-1).mean() > 0.9
