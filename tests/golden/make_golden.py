"""Records outputs of the reference's own kernels as golden fixtures.

Runs on a GPU machine: the reference's source/gcvt.cu and discretization.cu are
compiled from their sources into oracle/_ref/*.cubin by oracle/build_oracle.py
(where the reference checkout exists) and driven by oracle/ref_harness.c with
gcvt.cu's launch sequence.  Inputs are generated here from fixed seeds and
stored next to the outputs, so the CPU tests (tests/test_golden.py) need no
generator and no GPU.

    python tests/golden/make_golden.py OUTDIR
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "surface-remesher_gb300", "python")]

import oracle as orc  # noqa: E402
from workloads import MARKER, disk_mesh, raster_inputs, small_case  # noqa: E402


def pts_grid(n, xs, ys):
    g = np.full((n, n, 2), MARKER, np.int16)
    g[ys, xs, 0] = xs
    g[ys, xs, 1] = ys
    return g


def label_cases():
    rng = np.random.default_rng(20261203)
    out = []
    for t in range(12):
        n = [256, 512][t % 2]
        kind = t % 6
        if kind == 0:
            m = int(rng.integers(1, 40))
            p = rng.choice(n * n, m, replace=False)
        elif kind == 1:
            s = int(rng.integers(3, 30))
            ox, oy = rng.integers(0, s, 2)
            X, Y = np.meshgrid(np.arange(int(ox), n, s), np.arange(int(oy), n, s))
            p = (Y * n + X).ravel()
        elif kind == 2:
            pts = set()
            for _ in range(40):
                x = int(rng.integers(0, n))
                r = int(rng.integers(1, n // 64)) * 64 + int(rng.integers(-3, 3))
                k = int(rng.integers(1, 20))
                for yy in (r - k, r + k):
                    if 0 <= yy < n:
                        pts.add(yy * n + x)
            p = np.array(sorted(pts))
        elif kind == 3:
            c = int(rng.integers(0, n))
            p = np.unique(rng.integers(0, n, 25) * n + c)
        elif kind == 4:
            p = rng.choice(n * n, int(n * n * 0.05), replace=False)
        else:
            s = int(rng.integers(3, 20))
            p = np.array([y * n + x for y in range(0, n, s) for x in range((y // s) % 2 * (s // 2), n, s)])
        ys, xs = np.divmod(np.asarray(p, np.int64), n)
        out.append((n, xs.astype(np.int16), ys.astype(np.int16)))
    return out


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    # 1. labels (pba2DCompute)
    d = {}
    for i, (n, xs, ys) in enumerate(label_cases()):
        g = pts_grid(n, xs, ys)
        d["n%d" % i] = np.int32(n)
        d["xs%d" % i] = xs
        d["ys%d" % i] = ys
        d["labels%d" % i] = orc.ref_pba_label(g)
    np.savez_compressed(os.path.join(outdir, "ref_labels.npz"), **d)
    # 2. energy, one Lloyd step, and a whole gCVT run on Gaussian densities
    d = {}
    for i, (n, m, seed, omega) in enumerate(((256, 300, 101, 2.0), (512, 1500, 102, 1.5))):
        sites, rho, mask = small_case(n, m, seed)
        ys, xs = np.nonzero(sites[..., 0] != MARKER)
        lab, tot, new = orc.ref_lloyd_step(sites, rho, mask, omega)
        d["n%d" % i] = np.int32(n)
        d["omega%d" % i] = np.float32(omega)
        d["xs%d" % i] = xs.astype(np.int16)
        d["ys%d" % i] = ys.astype(np.int16)
        d["density%d" % i] = rho
        d["energy%d" % i] = np.float32(orc.ref_energy(lab, rho))
        d["totals%d" % i] = tot[:, ys, xs]
        nys, nxs = np.nonzero(new[..., 0] != MARKER)
        d["new_xs%d" % i] = nxs.astype(np.int16)
        d["new_ys%d" % i] = nys.astype(np.int16)
    n, m, seed = 256, 400, 103
    sites, rho, mask = small_case(n, m, seed)
    ys, xs = np.nonzero(sites[..., 0] != MARKER)
    out, info = orc.ref_gcvt(sites, rho, mask, 1, 300)
    d["run_n"] = np.int32(n)
    d["run_xs"] = xs.astype(np.int16)
    d["run_ys"] = ys.astype(np.int16)
    d["run_density"] = rho
    d["run_labels"] = out
    d["run_iterations"] = np.int32(info["iterations"])
    d["run_energies"] = np.array(info["energies"], np.float32)
    np.savez_compressed(os.path.join(outdir, "ref_lloyd.npz"), **d)
    # 3. rasteriser (discretization_d) on jittered disk meshes
    d = {}
    for i, (nv, n, seed, jit) in enumerate(((24, 256, 11, 0.3), (40, 256, 12, 0.45))):
        P, w, T = disk_mesh(nv, jitter=jit, seed=seed)
        Q, scale, _, _ = raster_inputs(P, n)
        dens, _ = orc.ref_rasterize(Q, w, T, scale, n)
        d["n%d" % i] = np.int32(n)
        d["points%d" % i] = Q
        d["weight%d" % i] = w
        d["tris%d" % i] = T
        d["scale%d" % i] = np.float64(scale)
        d["density%d" % i] = dens
    np.savez_compressed(os.path.join(outdir, "ref_raster.npz"), **d)
    print("wrote", sorted(os.listdir(outdir)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
