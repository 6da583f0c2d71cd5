"""Records outputs of the reference's own recover() and
weighting_vertices_with_area() as golden fixtures (ref_lift.npz).

Runs on a CPU where the reference checkout exists: oracle/build_oracle.py
compiles the reference's source/recover.h and source/weighting.h, unchanged,
behind oracle/ref_recover.cpp's stand-ins for CGAL and Boost into
oracle/_ref/librecover_ref.so.  Inputs come from fixed seeds and are stored
next to the outputs, so the tests need neither the generator nor the
reference.

    python tests/golden/make_golden_lift.py OUTDIR
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "surface-remesher_gb300", "python")]

import oracle as orc  # noqa: E402
from workloads import disk_surface  # noqa: E402


def delaunay(points):
    """Stand-in CDT over the points (scipy's unconstrained Delaunay)."""
    from scipy.spatial import Delaunay
    return Delaunay(points).simplices.astype(np.int32)


def query_points(rng, uv, tris, m):
    """An outside point first (its lift has no earlier location), then random
    points over [-0.05, 1.05]^2 (some outside the mesh), mesh vertices and
    edge midpoints (points on several faces)."""
    out = [np.array([[-0.25, -0.25]])]
    out.append(rng.uniform(-0.05, 1.05, (m, 2)))
    out.append(uv[rng.integers(0, len(uv), m // 8)])
    f = tris[rng.integers(0, len(tris), m // 8)]
    out.append((uv[f[:, 0]] + uv[f[:, 1]]) / 2)
    return np.concatenate(out)


def case_disk(seed, nv, m, nfixed):
    rng = np.random.default_rng(seed)
    uv, xyz, tris = disk_surface(nv, seed=seed)
    free = query_points(rng, uv, tris, m)
    fixed = rng.choice(len(uv), nfixed, replace=False).astype(np.int32)
    pts = np.concatenate([free, uv[fixed]])
    return uv, xyz, tris, pts, fixed, delaunay(pts)


def case_degenerate(seed):
    """Faces the binning must not lose: exactly or nearly collinear ones, a
    repeated vertex, a 1e-9 sliver, and a face whose uv area is 0 with a
    positive surface area (its vertices' weights exceed 1e10); plus a vertex
    on no face (weight 0/0)."""
    rng = np.random.default_rng(seed)
    uv, xyz, tris = disk_surface(10, seed=seed)
    extra_uv = np.array([[0.2, 0.3], [0.4, 0.3], [0.6, 0.3],          # collinear
                         [0.1, 0.1], [0.9, 0.1], [0.5, 0.1 + 1e-9],   # sliver
                         [0.3, 0.7], [0.3, 0.7], [0.45, 0.7],         # uv area 0
                         [0.05, 0.95]])                               # on no face
    extra_xyz = np.concatenate([extra_uv, rng.uniform(-0.1, 0.1, (len(extra_uv), 1))], 1)
    extra_xyz[7, 2] += 0.05
    V = len(uv)
    extra_tris = np.array([[V, V + 1, V + 2], [V + 3, V + 4, V + 5], [V + 6, V + 7, V + 8],
                           [tris[0, 0], tris[0, 0], tris[0, 1]]], np.int32)
    uv = np.concatenate([uv, extra_uv])
    xyz = np.concatenate([xyz, extra_xyz])
    tris = np.concatenate([extra_tris[:2], tris, extra_tris[2:]]).astype(np.int32)
    free = query_points(rng, uv[:V], tris[2:-2], 200)
    on_sliver = np.stack([rng.uniform(0.1, 0.9, 20), np.full(20, 0.1)], 1)
    on_line = np.stack([rng.uniform(0.2, 0.6, 20), np.full(20, 0.3)], 1)
    pts = np.concatenate([free, on_sliver, on_line])
    return uv, xyz, tris, pts, np.zeros(0, np.int32), delaunay(pts)


def case_nonfinite(seed):
    """A face with a NaN vertex (every later test of it passes) and one with
    an infinite vertex, points with NaN and infinite coordinates."""
    rng = np.random.default_rng(seed)
    uv, xyz, tris = disk_surface(8, seed=seed)
    V = len(uv)
    uv = np.concatenate([uv, [[np.nan, 0.5], [np.inf, 0.2], [0.3, 0.4]]])
    xyz = np.concatenate([xyz, [[0.0, 0.5, 0.0], [1.0, 0.2, 0.0], [0.3, 0.4, 0.1]]])
    tris = np.concatenate([tris[:5], [[V + 1, V + 2, 0]], tris[5:], [[V, V + 2, 1]]]).astype(
        np.int32)
    free = query_points(rng, uv[:V], tris[:5], 120)
    odd = np.array([[np.nan, 0.5], [0.5, np.nan], [np.inf, 0.5], [-np.inf, 0.3], [0.4, np.inf]])
    pts = np.concatenate([free[:60], odd, free[60:]])
    cdt = delaunay(free)
    return uv, xyz, tris, pts, np.zeros(0, np.int32), cdt


CASES = [("disk_small", lambda: case_disk(11, 20, 300, 12)),
         ("disk_mid", lambda: case_disk(12, 40, 2000, 40)),
         ("degenerate", lambda: case_degenerate(13)),
         ("nonfinite", lambda: case_nonfinite(14))]


def main(outdir):
    if not orc.recover_ref_available():
        raise SystemExit("oracle/_ref/librecover_ref.so missing: run oracle/build_oracle.py "
                         "with the reference checkout present")
    d = {}
    for i, (name, make) in enumerate(CASES):
        uv, xyz, tris, pts, fixed, cdt = make()
        lifted, keep = orc.ref_lift(uv, xyz, tris, pts, fixed, cdt)
        d.update({"name%d" % i: name, "uv%d" % i: uv, "xyz%d" % i: xyz, "tris%d" % i: tris,
                  "points%d" % i: pts, "fixed%d" % i: fixed, "cdt%d" % i: cdt,
                  "lifted%d" % i: lifted, "keep%d" % i: keep,
                  "weights%d" % i: orc.ref_vertex_weights(uv, xyz, tris)})
        print(name, len(uv), "vertices", len(tris), "faces", len(pts), "points", len(cdt),
              "triangles", int(keep.sum()), "kept", int(np.isnan(lifted[:, 0]).sum()), "NaN lifts")
    np.savez_compressed(os.path.join(outdir, "ref_lift.npz"), **d)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
