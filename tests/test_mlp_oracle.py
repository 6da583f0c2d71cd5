"""The step MLP's host oracle on the CPU: its backward formulas against
central finite differences of the unrounded FP64 network, its sample hash
against splitmix64's published first output, and its two forward
accumulation modes against each other.  The GPU kernels are checked against
this oracle in tests/test_learned_gpu.py."""
import numpy as np

import mlp_oracle as M


def params(seed, bias=0.05):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.N_PARAMS, np.float32)
    for sl, fan_in in ((M.SL_W1, 10), (M.SL_W2, 64), (M.SL_W3, 64)):
        p[sl] = rng.normal(0, np.sqrt(2.0 / fan_in), sl.stop - sl.start)
    for sl in (M.SL_B1, M.SL_B2, M.SL_B3):
        p[sl] = rng.normal(bias, 0.05, sl.stop - sl.start)
    return p


def batch(seed, rows=256):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (rows, 10))
    y = rng.normal(0, 0.5, (rows, 2))
    return x, y


def test_backward_matches_central_differences():
    p = params(1).astype(np.float64)
    x, y = batch(2)
    g = M.smooth_gradient(p, x, y)
    rng = np.random.default_rng(3)
    # a few parameters of every layer, weights and biases
    for sl in (M.SL_W1, M.SL_B1, M.SL_W2, M.SL_B2, M.SL_W3, M.SL_B3):
        for e in rng.choice(np.arange(sl.start, sl.stop), size=min(12, sl.stop - sl.start),
                            replace=False):
            h = 1e-6
            q = p.copy()
            q[e] += h
            lp = M.smooth_loss(q, x, y)
            q[e] -= 2 * h
            lm = M.smooth_loss(q, x, y)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[e]) <= 1e-6 + 1e-5 * abs(g[e]), (e, fd, g[e])


def test_straight_through_gradient_equals_smooth_one_without_rounding():
    # with bfloat16-exact parameters and inputs and no activation rounding
    # the oracle's gradient is the smooth network's
    p = M.bf16(params(4))
    x, y = batch(5, 64)
    x = M.bf16(x.astype(np.float32)).astype(np.float64)
    loss, g, s = M.loss_and_gradient(p, x, y, accumulate="fp64")
    g2 = M.smooth_gradient(p.astype(np.float64), x, y)
    # activations are rounded in the oracle, not in the smooth network:
    # agreement to bfloat16 precision
    assert np.linalg.norm(g - g2) <= 2e-2 * np.linalg.norm(g2)
    assert np.all(s >= np.abs(g) - 1e-12)


def test_fp32_and_fp64_forward_agree():
    p = params(6)
    x, _ = batch(7, 2000)
    a = M.forward(p, x, "fp32")["O"]
    b = M.forward(p, x, "fp64")["O"]
    assert np.median(np.abs(a - b)) < 1e-5
    assert np.mean(np.abs(a - b) > 1e-2 * (1 + np.abs(b))) < 0.01


def test_sample_hash_is_splitmix64():
    # splitmix64 from state 0: first output 0xE220A8397B1DCDAF
    assert int(M.mix64(np.uint64(0))) == 0xE220A8397B1DCDAF
    idx = M.sample_indices(seed=7, step=3, batch=4096, count=1000)
    assert idx.min() >= 0 and idx.max() < 1000
    assert len(np.unique(idx)) > 900
    assert np.array_equal(idx, M.sample_indices(7, 3, 4096, 1000))
    assert not np.array_equal(idx, M.sample_indices(7, 4, 4096, 1000))


def test_oracle_training_fits_a_linear_map():
    rng = np.random.default_rng(8)
    f = rng.normal(0, 1, (4000, 10)).astype(np.float32)
    y = np.stack([0.6 * f[:, 0] - 0.3 * f[:, 2], 0.5 * f[:, 1] + 0.2 * f[:, 9]], 1)
    s = np.concatenate([f, y.astype(np.float32)], 1)
    p, loss = M.train(s, params(9, bias=0.0), steps=150, batch=256, lr=3e-3, seed=1)
    assert loss[-10:].mean() < 0.2 * loss[:5].mean()
