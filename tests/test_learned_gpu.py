"""Learned steps: the MLP kernels against numpy and the host oracle
(oracle/mlp_oracle.py: forward bit for bit, gradients, Adam), training
against a known function, the energy gate (a jump that does not lower the
energy is undone without a trace), and the training features (histories,
ids)."""
import numpy as np
import pytest

import mlp_oracle as M
from workloads import MARKER, small_case

pytestmark = pytest.mark.gpu


def bf16(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward_numpy(p, f):
    W1 = bf16(p[:640]).reshape(10, 64).astype(np.float64)
    b1 = bf16(p[640:704]).astype(np.float64)
    W2 = bf16(p[704:4800]).reshape(64, 64).astype(np.float64)
    b2 = bf16(p[4800:4864]).astype(np.float64)
    W3 = bf16(p[4864:4992]).reshape(64, 2).astype(np.float64)
    b3 = bf16(p[4992:4994]).astype(np.float64)
    x = bf16(f).astype(np.float64)
    h1 = bf16(np.maximum(x @ W1 + b1, 0).astype(np.float32)).astype(np.float64)
    h2 = bf16(np.maximum(h1 @ W2 + b2, 0).astype(np.float32)).astype(np.float64)
    return h2 @ W3 + b3


@pytest.mark.parametrize("tensor_cores", [False, True])
def test_mlp_forward_matches_numpy(gcvt_lib, cuda_device, tensor_cores):
    assert gcvt_lib.mlp_param_count() == 4994
    p = gcvt_lib.mlp_init(3)
    p[640:704] = 0.1
    f = np.random.default_rng(4).normal(0, 1.5, (5000, 10)).astype(np.float32)
    got = gcvt_lib.mlp_forward(p, f, tensor_cores)
    want = forward_numpy(p, f)
    # FP32 accumulation vs FP64: the bfloat16 rounding of a hidden value can
    # flip on a tie-close sum, so compare with a loose bound on the few such
    assert np.median(np.abs(got - want)) < 1e-4
    assert np.mean(np.abs(got - want) > 1e-2 * (1 + np.abs(want))) < 0.01


def test_tensor_core_forward_equals_cuda_cores(gcvt_lib, cuda_device):
    p = gcvt_lib.mlp_init(9)
    f = np.random.default_rng(10).normal(0, 1.0, (100003, 10)).astype(np.float32)
    a = gcvt_lib.mlp_forward(p, f, True)
    b = gcvt_lib.mlp_forward(p, f, False)
    assert np.mean(np.abs(a - b) <= 1e-3 * (1 + np.abs(b))) > 0.99


def test_training_fits_a_known_step(gcvt_lib, cuda_device):
    rng = np.random.default_rng(5)
    f = rng.normal(0, 1, (200000, 10)).astype(np.float32)
    y = np.stack([0.8 * f[:, 0] - 0.3 * f[:, 2] + 0.2 * np.abs(f[:, 8]),
                  0.5 * f[:, 1] + 0.4 * f[:, 3] - 0.1 * f[:, 9]], 1).astype(np.float32)
    samples = np.concatenate([f, y], 1)
    p0 = gcvt_lib.mlp_init(6)
    p, loss = gcvt_lib.mlp_train(samples, p0, steps=1500, batch=2048, lr=2e-3, seed=7)
    assert np.all(np.isfinite(loss))
    assert loss[-50:].mean() < 0.05 * loss[:10].mean()
    pred = gcvt_lib.mlp_forward(p, f[:2000])
    assert np.mean((pred - y[:2000]) ** 2) < 0.02


def test_rejected_jumps_leave_no_trace(gcvt_lib, cuda_device):
    # a zero MLP proposes no move: the jumped sites are the sites, the energy
    # does not drop, every jump is undone and the run is the plain run
    sites, rho, mask = small_case(512, 2500, 51)
    plain = gcvt_lib.Context(512)
    plain.load(sites, rho, mask)
    plain.iterate(30)
    ctx = gcvt_lib.Context(512)
    ctx.learning(True)
    ctx.load(sites, rho, mask)
    ctx.set_mlp(np.zeros(gcvt_lib.mlp_param_count(), np.float32))
    tried, kept = ctx.iterate_learned(30, jump_every=5)
    assert (tried, kept) == (5, 0)  # the 30th iteration ends the run before a sixth
    assert np.array_equal(ctx.sites(), plain.sites())
    assert ctx.info()["energy"] == plain.info()["energy"]
    assert np.array_equal(ctx.label(), plain.label())
    plain.close()
    ctx.close()


def test_kept_jumps_lower_the_energy(gcvt_lib, cuda_device):
    sites, rho, mask = small_case(512, 2500, 52)
    ctx = gcvt_lib.Context(512)
    ctx.learning(True)
    ctx.load(sites, rho, mask)
    p = gcvt_lib.mlp_init(8) * 0.1
    ctx.set_mlp(p)
    ctx.iterate(10)
    e0 = ctx.info()["energy"]
    tried, kept = ctx.iterate_learned(40, jump_every=4)
    # rounds of three plain iterations and a learned step of two iterations
    # (kept) or one (rejected), proposed only while omega is 2: at most 10
    # steps in 40 iterations, some before the schedule first lowers omega
    # (after iteration 30)
    assert 1 <= tried <= 10 and 0 <= kept <= tried
    assert ctx.info()["iterations"] == 50
    e1 = ctx.info()["energy"]
    assert np.isfinite(e1) and e1 < e0
    s = ctx.sites()
    ys, xs = np.nonzero(s[..., 0] != MARKER)
    assert np.array_equal(s[ys, xs, 0], xs) and np.array_equal(s[ys, xs, 1], ys)
    ctx.close()


def test_features_track_moves_and_ids(gcvt_lib, cuda_device):
    sites, rho, mask = small_case(512, 2000, 53)
    m0 = int((sites[..., 0] != MARKER).sum())
    ctx = gcvt_lib.Context(512)
    ctx.learning(True, track_ids=True)
    ctx.load(sites, rho, mask)
    f0, ids0, xy0 = ctx.features(with_ids=True)
    assert len(f0) == m0 and np.array_equal(np.sort(ids0), np.arange(m0))
    assert np.all(f0[:, 2:8] == 0)  # no moves yet
    assert np.count_nonzero(f0[:, :2]) > 0.9 * m0  # pending displacements: centroid - site
    prev = {int(i): tuple(p) for i, p in zip(ids0, xy0)}
    ctx.iterate(1)
    f1, ids1, xy1 = ctx.features(with_ids=True)
    s = ctx.sites()
    ys, xs = np.nonzero(s[..., 0] != MARKER)
    assert set(zip(xs.tolist(), ys.tolist())) == set(map(tuple, xy1.tolist()))
    assert len(np.unique(ids1)) == len(ids1) and ids1.min() >= 0 and ids1.max() < m0
    # the newest applied move of each site is its displacement in this
    # iteration: the over-relaxed pending displacement of the features before
    r = None
    for f, i, p in zip(f1, ids1, xy1):
        dx, dy = p[0] - prev[int(i)][0], p[1] - prev[int(i)][1]
        if dx or dy:
            r = dx / f[2] if f[2] else dy / f[3]
            break
    assert r is not None and r > 0
    moves = np.rint(f1[:, 2:4] * r).astype(int)
    disp = np.array([(p[0] - prev[int(i)][0], p[1] - prev[int(i)][1]) for i, p in zip(ids1, xy1)])
    assert np.mean(np.all(moves == disp, 1)) > 0.99  # merges may hand an id on
    ctx.close()


def _params(seed, bias=0.05):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.N_PARAMS, np.float32)
    for sl, fan_in in ((M.SL_W1, 10), (M.SL_W2, 64), (M.SL_W3, 64)):
        p[sl] = rng.normal(0, np.sqrt(2.0 / fan_in), sl.stop - sl.start)
    for sl in (M.SL_B1, M.SL_B2, M.SL_B3):
        p[sl] = rng.normal(bias, 0.05, sl.stop - sl.start)
    return p


def _samples(seed, rows):
    rng = np.random.default_rng(seed)
    f = rng.normal(0, 1, (rows, 10)).astype(np.float32)
    y = np.stack([0.8 * f[:, 0] - 0.3 * f[:, 2] + 0.2 * np.abs(f[:, 8]),
                  0.5 * f[:, 1] + 0.4 * f[:, 3] - 0.1 * f[:, 9]], 1)
    y += rng.normal(0, 0.1, y.shape)
    return np.concatenate([f, y.astype(np.float32)], 1)


def test_cuda_core_forward_is_the_oracle_bit_for_bit(gcvt_lib, cuda_device):
    # the CUDA-core forward runs the same FP32 fma chains as the oracle's
    # "fp32" mode, so every bfloat16 rounding and the outputs agree exactly
    p = _params(11)
    f = np.random.default_rng(12).normal(0, 1.5, (20000, 10)).astype(np.float32)
    got = gcvt_lib.mlp_forward(p, f, False)
    want = M.forward(p, f, "fp32")["O"].astype(np.float32)
    assert np.mean(got == want) > 0.9999
    assert np.max(np.abs(got - want)) < 1e-3


def test_mlp_gradient_matches_fp64_oracle(gcvt_lib, cuda_device):
    p = _params(13)
    s = _samples(14, 5000)
    batch, seed, step = 2048, 3, 5
    g, loss = gcvt_lib.mlp_gradient(s, p, batch, seed, step)
    idx = M.sample_indices(seed, step, batch, len(s))
    want_loss, want, scale = M.loss_and_gradient(p, s[idx, :10], s[idx, 10:])
    # FP32 sums of 2048 terms per parameter (64 per block, then 32 block
    # partials added by atomics): within 1e-4 of the sum of |terms|
    assert abs(loss - want_loss) <= 1e-5 * want_loss
    assert np.all(np.abs(g - want) <= 1e-4 * scale + 1e-7 * np.abs(want).max())
    assert np.linalg.norm(g - want) <= 1e-5 * np.linalg.norm(want)
    assert np.count_nonzero(want) > 0.8 * M.N_PARAMS  # most units see gradient


def test_last_layer_gradient_matches_finite_differences(gcvt_lib, cuda_device):
    # the loss is exactly quadratic in a last-layer weight or bias; with
    # bfloat16-exact values and steps (multiples of 2^-6 below 4) the central
    # difference of the kernel's own losses is its derivative
    p = _params(15)
    w3 = np.clip(np.rint(p[M.SL_W3] * 64), -200, 200) / 64
    p[M.SL_W3] = w3
    p[M.SL_B3] = 0.0
    s = _samples(16, 3000)
    batch, seed, step, h = 2048, 5, 0, 2.0 ** -6
    g, _ = gcvt_lib.mlp_gradient(s, p, batch, seed, step)
    for e in list(range(M.SL_W3.start, M.SL_W3.start + 16)) + [4992, 4993]:
        q = p.copy()
        q[e] += h
        _, lp = gcvt_lib.mlp_gradient(s, q, batch, seed, step)
        q[e] -= 2 * h
        _, lm = gcvt_lib.mlp_gradient(s, q, batch, seed, step)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[e]) <= 2e-3 * abs(g[e]) + 2e-5, (e, fd, g[e])


def test_adam_steps_match_oracle(gcvt_lib, cuda_device):
    p0 = _params(17)
    s = _samples(18, 20000)
    lr, batch, seed = 1e-3, 1024, 4
    p1, _ = gcvt_lib.mlp_train(s, p0, steps=1, batch=batch, lr=lr, seed=seed)
    idx = M.sample_indices(seed, 0, batch, len(s))
    _, g, _ = M.loss_and_gradient(p0, s[idx, :10], s[idx, 10:])
    want = M.adam(p0.astype(np.float64), g, 0.0, 0.0, lr, 1)[0]
    # first step: lr * g / (|g| + eps) per parameter; a sign can differ only
    # where the gradient is at the level of its FP32 rounding
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    assert big.mean() > 0.5
    assert np.all(np.abs(p1 - want)[big] <= 1e-3 * lr + 1e-6)
    assert np.all(np.abs(p1 - want) <= 2 * lr + 1e-6)
    p3, loss3 = gcvt_lib.mlp_train(s, p0, steps=3, batch=batch, lr=lr, seed=seed)
    w3, wloss = M.train(s, p0, 3, batch, lr, seed)
    assert np.allclose(loss3, wloss, rtol=1e-3)
    assert np.mean(np.abs(p3 - w3) <= 1e-2 * lr) > 0.99


def _trained_or_analytic(gcvt_lib):
    """A network whose jumps are taken: the pending displacement itself (a
    jump to the centroid of the cell, the omega = 1 Lloyd step) written as
    MLP weights -- layer 1 splits the first two features into positive and
    negative parts, layer 2 passes them on, layer 3 recombines them."""
    p = np.zeros(gcvt_lib.mlp_param_count(), np.float32)
    W1 = p[:640].reshape(10, 64)
    W2 = p[704:4800].reshape(64, 64)
    W3 = p[4864:4992].reshape(64, 2)
    W1[0, 0], W1[0, 1], W1[1, 2], W1[1, 3] = 1, -1, 1, -1
    for j in range(4):
        W2[j, j] = 1
    W3[0, 0], W3[1, 0], W3[2, 1], W3[3, 1] = 1, -1, 1, -1
    return p


def test_batched_learned_runs_equal_solo_learned_runs(gcvt_lib, cuda_device):
    cases = [small_case(512, 2500, 61), small_case(256, 600, 62), small_case(512, 1500, 63)]
    p = _trained_or_analytic(gcvt_lib)
    solo = []
    for sites, rho, mask in cases:
        c = gcvt_lib.Context(sites.shape[0])
        c.learning(True)
        c.set_mlp(p)
        c.load(sites, rho, mask)
        tk = c.iterate_learned(23, jump_every=3)
        solo.append((c.sites(), c.info(), tk))
        c.close()
    assert sum(t[2][1] for t in solo) > 0  # some jumps stand
    ctxs = []
    for sites, rho, mask in cases:
        c = gcvt_lib.Context(sites.shape[0])
        c.learning(True)
        c.load(sites, rho, mask)
        ctxs.append(c)
    b = gcvt_lib.Batch(ctxs)
    b.set_mlp(p)
    tried, kept = b.iterate_learned(23, jump_every=3)
    assert (tried, kept) == (sum(t[2][0] for t in solo), sum(t[2][1] for t in solo))
    for c, (s_sites, s_info, _) in zip(ctxs, solo):
        assert np.array_equal(c.sites(), s_sites)
        info = c.info()
        assert info["iterations"] == s_info["iterations"] == 23
        assert info["energy"] == s_info["energy"] and info["omega"] == s_info["omega"]
    b.close()
    for c in ctxs:
        c.close()


def test_target_energy_stops_at_the_first_iteration_below(gcvt_lib, cuda_device):
    sites, rho, mask = small_case(512, 2500, 64)
    ctx = gcvt_lib.Context(512)
    ctx.load(sites, rho, mask)
    energies = []
    for _ in range(40):
        ctx.iterate(1)
        energies.append(ctx.info()["energy"])
    target = energies[24] * (1 + 1e-12)
    first = next(i for i, e in enumerate(energies) if e <= target) + 1
    ctx.set_target_energy(target)
    ctx.load(sites, rho, mask)
    ctx.iterate(40)
    info = ctx.info()
    assert info["iterations"] == first and info["energy"] == energies[first - 1]
    # learned steps stop the same way, at an energy at or below the target
    # (one every run meets early)
    target = energies[5] * (1 + 1e-12)
    ctx.set_target_energy(target)
    ctx.learning(True)
    ctx.set_mlp(_trained_or_analytic(gcvt_lib))
    ctx.load(sites, rho, mask)
    ctx.iterate_learned(60, jump_every=3)
    info = ctx.info()
    assert info["energy"] <= target and info["iterations"] < 60
    ctx.set_target_energy(0)
    ctx.close()


def test_trained_network_gains_over_plain_lloyd(gcvt_lib, cuda_device):
    """What the shipped network (surface-remesher_gb300/data/step_mlp.npy) gains
    over the method without it, on held-out runs of its training family
    (1024^2, 8 Gaussians, 4096 sites; seeds the training never saw):
    iterations until E <= (1 + 1e-4) E_conv, E_conv the energy after 1000
    plain iterations, the device stopping each run there.  Measured on a
    GB300: plain 42-43 iterations, learned (three plain iterations, then a
    learned step) 24-26.  A zero network gains nothing: every jump is
    rejected and the run is the plain run."""
    import os
    from train_step_mlp import DATA
    from workloads import disk_sites, gaussian_density
    p = np.load(os.path.join(DATA, "step_mlp.npy"))
    plain_it, learned_it = [], []
    for seed in (7001, 7002, 7003):
        rho = gaussian_density(1024, 8, 4.0, 0.02, 0.15, seed)
        sites = disk_sites(1024, 4096, seed, rho)
        mask = np.zeros((1024, 1024), np.uint8)
        ctx = gcvt_lib.Context(1024)
        ctx.load(sites, rho, mask)
        ctx.iterate(1000)
        target = ctx.info()["energy"] * (1 + 1e-4)
        ctx.set_target_energy(target)
        ctx.load(sites, rho, mask)
        ctx.iterate(400)
        plain_it.append(ctx.info()["iterations"])
        ctx.close()
        lc = gcvt_lib.Context(1024)
        lc.learning(True)
        lc.set_target_energy(target)
        lc.set_mlp(p)
        lc.load(sites, rho, mask)
        _, kept = lc.iterate_learned(400, 4)
        learned_it.append(lc.info()["iterations"])
        assert lc.info()["energy"] <= target and kept > 0
        lc.set_mlp(np.zeros_like(p))
        lc.load(sites, rho, mask)
        assert lc.iterate_learned(400, 4)[1] == 0
        assert lc.info()["iterations"] == plain_it[-1]
        lc.close()
    assert max(learned_it) <= 0.7 * min(plain_it), (learned_it, plain_it)
