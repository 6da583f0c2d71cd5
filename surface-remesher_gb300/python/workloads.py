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


# Batched uneven charts: 64 charts, side drawn from SIDES, config-0 density
# family (8 Gaussians), sites = domain pixels / 64, 100 iterations.
BATCH = dict(charts=64, sides=(256, 512, 1024, 2048), k=8, a_max=4.0, s_lo=0.02, s_hi=0.15,
             px_per_site=64, iters=100)


def batched_inputs(seed=1, charts=None):
    """[(sites, density, mask)] of the batched configuration: chart i has a
    seeded side from BATCH['sides'] and density seed seed * 1000 + i."""
    c = BATCH
    count = c["charts"] if charts is None else charts
    rng = np.random.default_rng(seed)
    sides = rng.choice(c["sides"], size=count)
    out = []
    for i, n in enumerate(sides.tolist()):
        rho = gaussian_density(n, c["k"], c["a_max"], c["s_lo"], c["s_hi"], seed * 1000 + i)
        m = int((rho > 0).sum()) // c["px_per_site"]
        out.append((disk_sites(n, m, seed * 1000 + i, rho), rho, np.zeros((n, n), np.uint8)))
    return out


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
    # each Gaussian is separable: the sum over k is one (n x k) (k x n)
    # product in float64 (the float32 grid equals the term-by-term sum's on
    # the benchmark configurations; checked at 1024^2, 4096^2 and 8192^2)
    gx = np.exp(-((c[:, None] - mu[None, :, 0]) ** 2) / (2 * s ** 2))
    gy = np.exp(-((c[:, None] - mu[None, :, 1]) ** 2) / (2 * s ** 2))
    rho = 1.0 + (gy * a) @ gx.T
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


def mesh_inputs(nv=256, n=2048, seed=2):
    """Mesh-driven configuration inputs before rasterisation: the jittered
    disk mesh of disk_mesh with its per-vertex area-ratio weights, shifted and
    scaled as discretization.h marshals them.  Returns ((points, weight,
    triangles, scale), mask); the density comes from rasterising the mesh
    and the sites from disk_sites over that density."""
    P, w, T = disk_mesh(nv, seed=seed)
    Q, scale, _, _ = raster_inputs(P, n)
    return (Q, w, T, scale), np.zeros((n, n), np.uint8)


def config_inputs(name, seed=1):
    """(sites, density, mask, iterations) of a named configuration."""
    c = CONFIGS[name]
    rho = gaussian_density(c["n"], c["k"], c["a_max"], c["s_lo"], c["s_hi"], seed)
    sites = disk_sites(c["n"], c["sites"], seed, rho)
    mask = np.zeros((c["n"], c["n"]), np.uint8)
    return sites, rho, mask, c["iters"]


def disk_surface(nv=256, jitter=0.3, seed=2, waves=6, radius=0.48):
    """Triangulated unit-disk parameterisation of a height-field surface.

    A regular nv x nv grid on [0,1]^2 (two triangles per cell) keeps the
    triangles whose vertices all lie in the disk of centre (0.5, 0.5); vertices
    get seeded Gaussian in-plane jitter of jitter x edge; the surface point of
    parameter (u, v) is (u, v, z), z = 0.1 sum_j sin(f_j u + g_j v + phi_j),
    f, g ~ U(2, 20).
    Returns (uv (V, 2) float64, xyz (V, 3) float64, triangles (T, 3) int32)."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (nv - 1)
    g = np.arange(nv) * h
    X, Y = np.meshgrid(g, g)
    P = np.stack([X.ravel(), Y.ravel()], 1)
    inside = (P[:, 0] - 0.5) ** 2 + (P[:, 1] - 0.5) ** 2 <= radius * radius
    P = P + rng.normal(0.0, jitter * h, P.shape)
    idx = np.arange(nv * nv).reshape(nv, nv)
    a, b, c, d = idx[:-1, :-1], idx[:-1, 1:], idx[1:, :-1], idx[1:, 1:]
    tris = np.concatenate([np.stack([a, b, d], -1).reshape(-1, 3),
                           np.stack([a, d, c], -1).reshape(-1, 3)])
    tris = tris[inside[tris].all(1)]
    used = np.unique(tris)
    remap = -np.ones(nv * nv, np.int64)
    remap[used] = np.arange(len(used))
    P = P[used]
    tris = remap[tris]
    f = rng.uniform(2, 20, waves)
    gg = rng.uniform(2, 20, waves)
    phi = rng.uniform(0, 2 * np.pi, waves)
    z = 0.1 * np.sin(np.outer(P[:, 0], f) + np.outer(P[:, 1], gg) + phi).sum(1)
    return P, np.concatenate([P, z[:, None]], 1), tris.astype(np.int32)


def area_weights(uv, xyz, tris):
    """Per-vertex density weight, the area ratio of weighting.h:79: sum of
    incident surface face areas / sum of incident parameter-space face areas
    (ratios above 1e10 take the largest other ratio, weighting.h:80-92).
    numpy arithmetic; the library's gcvt_vertex_weights is the exact form."""
    e1 = xyz[tris[:, 1]] - xyz[tris[:, 0]]
    e2 = xyz[tris[:, 2]] - xyz[tris[:, 0]]
    a3 = 0.5 * np.linalg.norm(np.cross(e1, e2), axis=1)
    u1, u2 = e1[:, :2], e2[:, :2]
    a2 = 0.5 * np.abs(u1[:, 0] * u2[:, 1] - u2[:, 0] * u1[:, 1])
    s3 = np.zeros(len(uv))
    s2 = np.zeros(len(uv))
    for k in range(3):
        np.add.at(s3, tris[:, k], a3)
        np.add.at(s2, tris[:, k], a2)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = s3 / s2
    finite = np.isfinite(w) & (w <= 1e10)
    w[~finite] = w[finite].max()
    return w


def disk_mesh(nv=256, jitter=0.3, seed=2, waves=6, radius=0.48):
    """disk_surface with its per-vertex area-ratio weights.
    Returns (uv (V, 2) float64, weight (V,) float64, triangles (T, 3) int32)."""
    uv, xyz, tris = disk_surface(nv, jitter, seed, waves, radius)
    return uv, area_weights(uv, xyz, tris), tris


def raster_inputs(P, n):
    """The host marshalling of discretization (discretization.h:89-118):
    scale = longest bounding-box side / (n - 1), points shifted to the box's
    lower-left corner.  Returns (shifted points, scale, left, lower)."""
    l, b = P[:, 0].min(), P[:, 1].min()
    r, u = P[:, 0].max(), P[:, 1].max()
    scale = (u - b) / (n - 1) if (u - b) > (r - l) else (r - l) / (n - 1)
    Q = np.ascontiguousarray(np.stack([P[:, 0] - l, P[:, 1] - b], 1))
    return Q, scale, l, b


def mesh_constraints(uv, tris, scale, left, lower):
    """The CDT constraints of a disk mesh, as the reference's pipeline takes
    them: its boundary vertices are the constraint points and its boundary
    edges the constraint segments (detect_constrains, main.cpp:211-214), and
    each constraint point's pixel becomes a fixed site (generateMask,
    gcvt.h:141-158: x = int((p.x - left) / scale)).  Returns (bv: the
    boundary vertex ids, be: the boundary edges as vertex id pairs, px, py:
    the fixed pixels)."""
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]).astype(np.int64)
    key = np.sort(e, 1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    be = e[cnt[inv.ravel()] == 1]
    bv = np.unique(be)
    px = ((uv[bv, 0] - left) / scale).astype(np.int64)
    py = ((uv[bv, 1] - lower) / scale).astype(np.int64)
    return bv, be, px, py


def small_case(n, m, seed, k=6, a_max=4.0):
    """A small Gaussian-density case for parity tests."""
    rho = gaussian_density(n, k, a_max, 0.03, 0.2, seed)
    return disk_sites(n, m, seed, rho), rho, np.zeros((n, n), np.uint8)
