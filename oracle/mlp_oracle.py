"""Host oracle of the learned step's MLP (TEST INFRASTRUCTURE ONLY).

The step MLP has no counterpart in the reference (Surface-Remesher's gCVT,
source/gcvt.cu:1087-1156, moves sites by plain over-relaxed Lloyd steps
only); this module restates the library's own network so that its GPU
forward, backward and Adam kernels can be checked on the CPU:

  * forward  -- 10 -> 64 -> 64 -> 2 with ReLU.  Weights and the inputs are
    rounded to bfloat16, every hidden activation is rounded to bfloat16 after
    the ReLU, accumulation is FP32.  `forward(..., accumulate="fp32")`
    replays the kernels' FP32 fused multiply-add chains in their order
    (bias first, then the inputs in index order), so the bfloat16 rounding
    decisions are the kernels' own; "fp64" accumulates in double.
  * backward -- the gradient of the mean of 0.5 |out - target|^2 over a
    batch with respect to the FP32 master parameters, in FP64, through the
    bfloat16 roundings as the identity (straight-through: the kernels'
    rule), ReLU'(z) = [h > 0].
  * adam     -- one Adam step (beta1 0.9, beta2 0.999, eps 1e-8, bias
    corrected) on the master parameters.
  * sample_indices -- the batch the training kernel draws at a step: slot i
    takes sample mix64(seed ^ (step << 32) ^ i) mod count (splitmix64's
    finaliser).

Parameter layout (4994 floats): W1[10][64], b1[64], W2[64][64], b2[64],
W3[64][2], b3[2]; W[i][j] maps input i to output j.
"""
import numpy as np

N_IN, N_HID, N_OUT = 10, 64, 2
SL_W1 = slice(0, 640)
SL_B1 = slice(640, 704)
SL_W2 = slice(704, 4800)
SL_B2 = slice(4800, 4864)
SL_W3 = slice(4864, 4992)
SL_B3 = slice(4992, 4994)
N_PARAMS = 4994


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float32)
    return (p[SL_W1].reshape(N_IN, N_HID), p[SL_B1], p[SL_W2].reshape(N_HID, N_HID), p[SL_B2],
            p[SL_W3].reshape(N_HID, N_OUT), p[SL_B3])


def _fma32(a, b, c):
    """float32 fma(a, b, c): the product of two floats is exact in double, the
    sum is rounded once to double and then to float (a second rounding that
    can differ from a single one only on a double-rounding boundary)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def forward(params, x, accumulate="fp32"):
    """Forward pass of feature rows x (B x 10): dict with the bfloat16 inputs
    X, hidden activations H1, H2 (after ReLU and rounding) and the output O
    (B x 2), all as float64 arrays holding the kernels' values."""
    W1, b1, W2, b2, W3, b3 = (bf16(a) for a in unpack(params))
    X = bf16(np.asarray(x, np.float32))
    B = X.shape[0]
    if accumulate == "fp64":
        h1 = bf16(np.maximum(X.astype(np.float64) @ W1 + b1, 0).astype(np.float32))
        h2 = bf16(np.maximum(h1.astype(np.float64) @ W2 + b2, 0).astype(np.float32))
        o = h2.astype(np.float64) @ W3 + b3
        return {"X": X.astype(np.float64), "H1": h1.astype(np.float64),
                "H2": h2.astype(np.float64), "O": o}
    acc = np.broadcast_to(b1, (B, N_HID)).astype(np.float32)
    for i in range(N_IN):
        acc = _fma32(X[:, i:i + 1], W1[i][None, :], acc)
    h1 = bf16(np.maximum(acc, np.float32(0)))
    acc = np.broadcast_to(b2, (B, N_HID)).astype(np.float32)
    for k in range(N_HID):
        acc = _fma32(h1[:, k:k + 1], W2[k][None, :], acc)
    h2 = bf16(np.maximum(acc, np.float32(0)))
    o = np.broadcast_to(b3, (B, N_OUT)).astype(np.float32)
    for j in range(N_HID):
        o = _fma32(h2[:, j:j + 1], W3[j][None, :], o)
    return {"X": X.astype(np.float64), "H1": h1.astype(np.float64),
            "H2": h2.astype(np.float64), "O": o.astype(np.float64)}


def loss_and_gradient(params, x, y, accumulate="fp32"):
    """Mean loss 0.5 |O - y|^2 over the rows and its gradient with respect to
    the master parameters (N_PARAMS float64), and the per-parameter sums of
    |term| (the scale an FP32 sum of the terms is accurate to)."""
    W1, b1, W2, b2, W3, b3 = (bf16(a).astype(np.float64) for a in unpack(params))
    f = forward(params, x, accumulate)
    X, H1, H2, O = f["X"], f["H1"], f["H2"], f["O"]
    B = X.shape[0]
    D = O - np.asarray(y, np.float64)                  # dL/dO per row
    loss = 0.5 * np.sum(D * D) / B
    D2 = (D @ W3.T) * (H2 > 0)                         # dL/dz2
    D1 = (D2 @ W2.T) * (H1 > 0)                        # dL/dz1
    # the same chain on absolute values bounds every partial sum
    A = np.abs(D)
    A2 = (A @ np.abs(W3).T) * (H2 > 0)
    A1 = (A2 @ np.abs(W2).T) * (H1 > 0)
    g = np.empty(N_PARAMS, np.float64)
    s = np.empty(N_PARAMS, np.float64)
    g[SL_W1] = (X.T @ D1).ravel() / B
    s[SL_W1] = (np.abs(X).T @ A1).ravel() / B
    g[SL_B1] = D1.sum(0) / B
    s[SL_B1] = A1.sum(0) / B
    g[SL_W2] = (H1.T @ D2).ravel() / B
    s[SL_W2] = (H1.T @ A2).ravel() / B
    g[SL_B2] = D2.sum(0) / B
    s[SL_B2] = A2.sum(0) / B
    g[SL_W3] = (H2.T @ D).ravel() / B
    s[SL_W3] = (H2.T @ A).ravel() / B
    g[SL_B3] = D.sum(0) / B
    s[SL_B3] = A.sum(0) / B
    return loss, g, s


def smooth_loss(params, x, y):
    """The same network without any bfloat16 rounding, FP64 throughout: the
    function whose derivative the straight-through gradient is, used for the
    finite-difference check of loss_and_gradient's formulas."""
    p = np.asarray(params, np.float64)
    W1, b1 = p[SL_W1].reshape(N_IN, N_HID), p[SL_B1]
    W2, b2 = p[SL_W2].reshape(N_HID, N_HID), p[SL_B2]
    W3, b3 = p[SL_W3].reshape(N_HID, N_OUT), p[SL_B3]
    h1 = np.maximum(np.asarray(x, np.float64) @ W1 + b1, 0)
    h2 = np.maximum(h1 @ W2 + b2, 0)
    d = h2 @ W3 + b3 - np.asarray(y, np.float64)
    return 0.5 * np.sum(d * d) / len(d)


def smooth_gradient(params, x, y):
    """Analytic gradient of smooth_loss (FP64, no rounding)."""
    p = np.asarray(params, np.float64)
    W1, b1 = p[SL_W1].reshape(N_IN, N_HID), p[SL_B1]
    W2, b2 = p[SL_W2].reshape(N_HID, N_HID), p[SL_B2]
    W3, b3 = p[SL_W3].reshape(N_HID, N_OUT), p[SL_B3]
    X = np.asarray(x, np.float64)
    h1 = np.maximum(X @ W1 + b1, 0)
    h2 = np.maximum(h1 @ W2 + b2, 0)
    D = h2 @ W3 + b3 - np.asarray(y, np.float64)
    B = len(D)
    D2 = (D @ W3.T) * (h2 > 0)
    D1 = (D2 @ W2.T) * (h1 > 0)
    g = np.empty(N_PARAMS, np.float64)
    g[SL_W1] = (X.T @ D1).ravel() / B
    g[SL_B1] = D1.sum(0) / B
    g[SL_W2] = (h1.T @ D2).ravel() / B
    g[SL_B2] = D2.sum(0) / B
    g[SL_W3] = (h2.T @ D).ravel() / B
    g[SL_B3] = D.sum(0) / B
    return g


def mix64(z):
    """splitmix64's finaliser on uint64 values (wrapping arithmetic)."""
    z = np.asarray(z, np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def sample_indices(seed, step, batch, count):
    """Sample rows the training kernel uses at `step`, one per batch slot."""
    slots = np.arange(batch, dtype=np.uint64)
    z = np.uint64(seed) ^ (np.uint64(step) << np.uint64(32)) ^ slots
    return (mix64(z) % np.uint64(count)).astype(np.int64)


def adam(master, g, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns (master, m, v), float64."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return master - lr * mh / (np.sqrt(vh) + eps), m, v


def train(samples, params, steps, batch, lr, seed):
    """The training loop of the GPU trainer restated: Adam on the mean loss of
    the batch each step draws; returns (master parameters, losses)."""
    samples = np.asarray(samples, np.float32)
    master = np.asarray(params, np.float32).astype(np.float64)
    m = np.zeros(N_PARAMS)
    v = np.zeros(N_PARAMS)
    losses = []
    for st in range(steps):
        idx = sample_indices(seed, st, batch, len(samples))
        rows = samples[idx]
        loss, g, _ = loss_and_gradient(master.astype(np.float32), rows[:, :N_IN], rows[:, N_IN:])
        losses.append(loss)
        master, m, v = adam(master, g, m, v, lr, st + 1)
        master = master.astype(np.float32).astype(np.float64)  # FP32 master weights
    return master.astype(np.float32), np.array(losses)
