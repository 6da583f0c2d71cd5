"""Site seeding (gcvt.h:56-122) is host code of the library: its initial
sites equal the oracle's restatement of putConstrains + randomPoints with the
reference's generator, bit for bit, and the generator state carries over
between calls as the reference's unseeded globals do.  Both are pinned to the
reference's own gcvt.h, compiled from the checkout (oracle/ref_seed.cpp),
where that build exists.  No GPU needed."""
import numpy as np
import pytest

import oracle as orc
from workloads import MARKER, disk_mask, gaussian_density


@pytest.mark.parametrize("n,num,fixed", [(64, 50, 0), (256, 2000, 0), (256, 500, 40), (512, 4096, 0)])
def test_seed_matches_oracle(gcvt_lib, oracle, n, num, fixed):
    rho = gaussian_density(n, 6, 4.0, 0.03, 0.2, seed=n + num)
    mask = np.zeros((n, n), np.uint8)
    if fixed:
        rng = np.random.default_rng(fixed)
        ys, xs = np.nonzero(rho > 0)
        k = rng.choice(len(xs), fixed, replace=False)
        mask[ys[k], xs[k]] = 1
    state = np.zeros(4, np.uint64)
    got = gcvt_lib.seed_sites(rho, mask, num, state)
    want = oracle.seed_sites(rho, mask, num, 0)
    assert np.array_equal(got, want)
    assert int((got[..., 0] != MARKER).sum()) == num + fixed
    assert state.any()  # the generator advanced


def test_state_carries_over(gcvt_lib):
    n = 128
    rho = gaussian_density(n, 4, 4.0, 0.05, 0.2, seed=3)
    mask = np.zeros((n, n), np.uint8)
    s = np.zeros(4, np.uint64)
    a = gcvt_lib.seed_sites(rho, mask, 100, s)
    b = gcvt_lib.seed_sites(rho, mask, 100, s)
    assert not np.array_equal(a, b)
    s2 = np.zeros(4, np.uint64)
    assert np.array_equal(gcvt_lib.seed_sites(rho, mask, 100, s2), a)
    assert np.array_equal(gcvt_lib.seed_sites(rho, mask, 100, s2), b)
    assert np.array_equal(s, s2)


def test_seed_rejects_impossible_counts(gcvt_lib):
    n = 64
    rho = np.zeros((n, n), np.float32)
    rho[:2, :2] = 1.0
    mask = np.zeros((n, n), np.uint8)
    lib = gcvt_lib.load_library()
    v = np.empty((n, n, 2), np.int16)
    st = np.zeros(4, np.uint64)
    assert lib.gcvt_seed_sites(v.ctypes.data, rho.ctypes.data, mask.ctypes.data, 5, n,
                               st.ctypes.data) == 1
    assert lib.gcvt_seed_sites(v.ctypes.data, rho.ctypes.data, mask.ctypes.data, 4, n,
                               st.ctypes.data) == 0
    assert lib.gcvt_seed_sites(None, rho.ctypes.data, None, 4, n, None) == 1


@pytest.mark.skipif(not orc.seed_ref_available(), reason="reference seeding not built here")
@pytest.mark.parametrize("n,num,fixed", [(64, 50, 0), (256, 2000, 0), (256, 500, 40),
                                         (512, 4096, 0), (1024, 4096, 7)])
def test_seed_matches_reference_gcvt_h(gcvt_lib, n, num, fixed):
    rho = gaussian_density(n, 6, 4.0, 0.03, 0.2, seed=n + num + 1)
    mask = np.zeros((n, n), np.uint8)
    if fixed:
        rng = np.random.default_rng(fixed)
        ys, xs = np.nonzero(rho > 0)
        k = rng.choice(len(xs), fixed, replace=False)
        mask[ys[k], xs[k]] = 1
    want, want_state = orc.ref_seed_sites(rho, mask, num)
    state = np.zeros(4, np.uint64)
    got = gcvt_lib.seed_sites(rho, mask, num, state)
    assert np.array_equal(got, want)
    assert np.array_equal(state, want_state)
    # and again from the state the first call left (the reference's globals
    # carry over between calls)
    want2, want_state2 = orc.ref_seed_sites(rho, mask, num, want_state)
    got2 = gcvt_lib.seed_sites(rho, mask, num, state)
    assert np.array_equal(got2, want2) and np.array_equal(state, want_state2)


@pytest.mark.skipif(not orc.seed_ref_available(), reason="reference seeding not built here")
def test_oracle_seed_matches_reference_gcvt_h():
    n = 256
    rho = gaussian_density(n, 5, 4.0, 0.03, 0.2, seed=77)
    mask = np.zeros((n, n), np.uint8)
    want, _ = orc.ref_seed_sites(rho, mask, 1500)
    assert np.array_equal(orc.seed_sites(rho, mask, 1500, 0), want)
