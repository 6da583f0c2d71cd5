"""Batched charts (config 3 family): charts of uneven sizes iterated together
in one launch pair per iteration give, chart by chart, the same sites, labels
and schedule state as each chart iterated alone -- bit for bit, since every
chart's cells, moves and energy order are the same computation."""
import numpy as np
import pytest

from workloads import small_case

pytestmark = pytest.mark.gpu

CHARTS = [(256, 300, 31), (512, 2500, 32), (256, 120, 33), (1024, 6000, 34), (512, 900, 35)]


def load(gcvt_lib, n, m, seed):
    sites, rho, mask = small_case(n, m, seed)
    ctx = gcvt_lib.Context(n)
    ctx.load(sites, rho, mask)
    return ctx


def test_batch_iterate_equals_solo(gcvt_lib, cuda_device):
    iters = 23
    solo = []
    for n, m, seed in CHARTS:
        c = load(gcvt_lib, n, m, seed)
        c.iterate(iters)
        solo.append((c.sites(), c.label(), c.info()))
        c.close()
    ctxs = [load(gcvt_lib, n, m, seed) for n, m, seed in CHARTS]
    batch = gcvt_lib.Batch(ctxs)
    batch.iterate(iters)
    for c, (s, lab, info) in zip(ctxs, solo):
        assert np.array_equal(c.sites(), s)
        assert np.array_equal(c.label(), lab)
        got = c.info()
        assert got["iterations"] == info["iterations"] == iters
        assert got["energy"] == info["energy"]
        assert got["omega"] == info["omega"]
    # a second call continues every chart
    batch.iterate(7)
    assert all(c.info()["iterations"] == iters + 7 for c in ctxs)
    batch.close()
    for c in ctxs:
        c.close()


def test_batch_run_equals_solo(gcvt_lib, cuda_device):
    charts = CHARTS[:3]
    solo = []
    for n, m, seed in charts:
        c = load(gcvt_lib, n, m, seed)
        info = c.run(1, 400)
        solo.append((c.label(), info))
        c.close()
    ctxs = [load(gcvt_lib, n, m, seed) for n, m, seed in charts]
    batch = gcvt_lib.Batch(ctxs)
    infos = batch.run(400)
    for c, info, (lab, want) in zip(ctxs, infos, solo):
        assert info["iterations"] == want["iterations"]
        assert info["energy"] == want["energy"]
        assert np.array_equal(c.label(), lab)
    # the charts stop at different iterations
    assert len({i["iterations"] for i in infos}) > 1
    batch.close()
    for c in ctxs:
        c.close()


def test_batch_rejects_duplicates(gcvt_lib, cuda_device):
    c = load(gcvt_lib, 256, 100, 1)
    with pytest.raises(gcvt_lib.GcvtError):
        gcvt_lib.Batch([c, c])
    c.close()
