"""The autotuner and the launch choices change speed only: a tuned context,
and one set to each extreme choice by hand, give the same sites, labels and
energies as an untuned one, bit for bit; the search leaves the state as it
found it."""
import numpy as np
import pytest

from workloads import small_case

pytestmark = pytest.mark.gpu


def run(gcvt_lib, sites, rho, mask, iters, tune=None):
    n = sites.shape[0]
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    t = None
    if tune == "auto":
        ctx.iterate(3)
        t = ctx.autotune()
        ctx.iterate(iters - 3)
    else:
        if tune is not None:
            ctx.set_tuning(**tune)
        ctx.iterate(iters)
    out = (ctx.sites(), ctx.label(), ctx.info()["energy"], ctx.jfa_label()[0])
    ctx.close()
    return out, t


@pytest.mark.parametrize("case", [(512, 3000, 41), (1024, 8000, 42)])
def test_tuning_changes_nothing(gcvt_lib, cuda_device, case):
    n, m, seed = case
    sites, rho, mask = small_case(n, m, seed)
    base, _ = run(gcvt_lib, sites, rho, mask, 15)
    tuned, t = run(gcvt_lib, sites, rho, mask, 15, "auto")
    assert t["cell_blocks_per_sm"] in (16, 24, 32)
    assert t["hint_slack"] in (1, 2, 3)
    assert t["jfa_tail_halo"] in (0, 8, 16, 32)
    assert t["lloyd_ms"] > 0 and t["jfa_ms"] > 0
    assert t["cell_mode"] in (1, 2)
    for a, b in zip(base, tuned):
        assert np.array_equal(a, b)
    # one site per lane and one per warp (both sizes have at most 8192 sites)
    for choice in ({"cell_blocks_per_sm": 16, "hint_slack": 1, "jfa_tail_halo": 8,
                    "cell_mode": 1},
                   {"cell_blocks_per_sm": 32, "hint_slack": 3, "jfa_tail_halo": 32,
                    "cell_mode": 1},
                   {"cell_blocks_per_sm": 24, "hint_slack": 2, "jfa_tail_halo": 16,
                    "cell_mode": 2},
                   {"cell_blocks_per_sm": 24, "hint_slack": 2, "jfa_tail_halo": 0,
                    "cell_mode": 2}):
        other, _ = run(gcvt_lib, sites, rho, mask, 15, choice)
        for a, b in zip(base, other):
            assert np.array_equal(a, b)


def test_set_tuning_rejects_bad_values(gcvt_lib, cuda_device):
    ctx = gcvt_lib.Context(256)
    with pytest.raises(gcvt_lib.GcvtError):
        ctx.set_tuning(jfa_tail_halo=12)
    with pytest.raises(gcvt_lib.GcvtError):
        ctx.set_tuning(cell_blocks_per_sm=40)
    with pytest.raises(gcvt_lib.GcvtError):
        ctx.set_tuning(cell_mode=3)
    ctx.close()


@pytest.mark.parametrize("case", [(256, 300, 51, 30), (1024, 4096, 52, 50), (512, 8192, 53, 12)])
def test_one_site_per_warp_equals_one_per_lane(gcvt_lib, cuda_device, case):
    """The two ways of running the cells give the same trajectory bit for
    bit: sites, labels, energy and the schedule's iteration count."""
    n, m, seed, iters = case
    sites, rho, mask = small_case(n, m, seed)
    out = []
    for mode in (1, 2):
        ctx = gcvt_lib.Context(n)
        ctx.set_tuning(cell_mode=mode)
        ctx.load(sites, rho, mask)
        ctx.iterate(iters)
        info = ctx.info()
        out.append((ctx.sites(), ctx.label(), info["energy"], info["iterations"]))
        ctx.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    # and the full schedule through gcvt_ctx_run
    runs = []
    for mode in (1, 2):
        ctx = gcvt_lib.Context(n)
        ctx.set_tuning(cell_mode=mode)
        ctx.load(sites, rho, mask)
        info = ctx.run(1, 300)
        runs.append((ctx.label(), info["iterations"], info["energy"]))
        ctx.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)
