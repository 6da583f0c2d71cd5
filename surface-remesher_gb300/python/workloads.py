"""Seeded synthetic workloads for the CVT hot path.

The reference ships no benchmark inputs; these generators produce the density
grids, domains and initial site grids of the benchmark configurations:

  * ``gaussian_density``: rho(x) = 1 + sum_k a_k exp(-|x - mu_k|^2 / (2 s_k^2))
    on pixel centres x = (i + 0.5)/n of [0,1]^2, rho = 0 outside the disk of
    centre (0.5, 0.5) and radius 0.48 (the domain), mu_k uniform in the disk;
  * ``disk_sites``: distinct integer site pixels uniform in the disk;
  * ``CONFIGS``: the parameters of the five benchmark configurations.

All randomness comes from numpy's PCG64 with the seed given, so a (config,
seed) pair names one input exactly.
"""
import numpy as np

MARKER = -32768

CONFIGS = {
    # name: (n, gaussians, a_max, sigma_lo, sigma_hi, sites, iterations)
    "plain_1024": dict(n=1024, k=8, a_max=4.0, s_lo=0.02, s_hi=0.15, sites=4096, iters=50),
    "plain_4096": dict(n=4096, k=32, a_max=8.0, s_lo=0.005, s_hi=0.1, sites=262144, iters=100),
    "plain_8192": dict(n=8192, k=64, a_max=8.0, s_lo=0.005, s_hi=0.1, sites=1048576, iters=100),
}


def disk_mask(n, radius=0.48):
    c = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(c, c)
    return (X - 0.5) ** 2 + (Y - 0.5) ** 2 <= radius * radius


def gaussian_density(n, k, a_max, s_lo, s_hi, seed, radius=0.48):
    """float32 (n, n) density: 1 + k seeded Gaussians inside the disk, 0 outside."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.0, a_max, k)
    # mu uniform in the disk (polar with sqrt radius)
    rr = radius * np.sqrt(rng.uniform(0.0, 1.0, k))
    th = rng.uniform(0.0, 2 * np.pi, k)
    mu = np.stack([0.5 + rr * np.cos(th), 0.5 + rr * np.sin(th)], 1)
    s = rng.uniform(s_lo, s_hi, k)
    c = (np.arange(n, dtype=np.float64) + 0.5) / n
    rho = np.ones((n, n), np.float64)
    for j in range(k):
        gx = np.exp(-((c - mu[j, 0]) ** 2) / (2 * s[j] ** 2))
        gy = np.exp(-((c - mu[j, 1]) ** 2) / (2 * s[j] ** 2))
        rho += a[j] * np.outer(gy, gx)
    rho[~disk_mask(n, radius)] = 0.0
    return rho.astype(np.float32)


def disk_sites(n, m, seed, density=None, radius=0.48):
    """Site grid (n, n, 2) int16 with m distinct sites uniform in the domain."""
    rng = np.random.default_rng(seed + 7919)
    inside = disk_mask(n, radius) if density is None else density > 0
    idx = np.flatnonzero(inside.ravel())
    if m > idx.size:
        raise ValueError("more sites than domain pixels")
    pick = rng.choice(idx, size=m, replace=False)
    ys, xs = np.divmod(pick, n)
    g = np.full((n, n, 2), MARKER, np.int16)
    g[ys, xs, 0] = xs
    g[ys, xs, 1] = ys
    return g


def config_inputs(name, seed=1):
    """(sites, density, mask, iterations) of a named configuration."""
    c = CONFIGS[name]
    rho = gaussian_density(c["n"], c["k"], c["a_max"], c["s_lo"], c["s_hi"], seed)
    sites = disk_sites(c["n"], c["sites"], seed, rho)
    mask = np.zeros((c["n"], c["n"]), np.uint8)
    return sites, rho, mask, c["iters"]


def small_case(n, m, seed, k=6, a_max=4.0):
    """A small Gaussian-density case for parity tests."""
    rho = gaussian_density(n, k, a_max, 0.03, 0.2, seed)
    return disk_sites(n, m, seed, rho), rho, np.zeros((n, n), np.uint8)
