"""The constrained Delaunay stage's mesh operations (csrc/cdt_core.cuh),
compiled for the host and run one after the other (tests/cdt_core_host.cpp):
from a Delaunay triangulation of lattice sites, constraint points are located
and inserted (inside triangles, on edges, outside the hull), segments are
recovered by flips, and flips restore the constrained Delaunay property.  The
result must pass the restated DelaunayChecker with its constraint check
(oracle/delaunay_oracle.py check_cdt), exactly, under the symbolic
perturbation.  The GPU runs the same functions in parallel rounds
(tests/test_cdt_gpu.py).  No GPU needed."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
import delaunay_oracle as D

CSRC = os.path.join(ROOT, "surface-remesher_gb300", "csrc")
SHIFT = 15


@pytest.fixture(scope="module")
def host_bin(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    out = str(tmp_path_factory.mktemp("cdt") / "cdt_host")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, "-o", out,
                    os.path.join(ROOT, "tests", "cdt_core_host.cpp")], check=True)
    return out


def start_triangulation(pts):
    """Any triangulation of the sites to start from: Qhull's, made
    counter-clockwise (flips turn it into the perturbed Delaunay one)."""
    from scipy.spatial import Delaunay
    tri = Delaunay(pts.astype(np.float64)).simplices.astype(np.int64)
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    o = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    tri[o < 0] = tri[o < 0][:, [0, 2, 1]]
    return tri[o != 0]


def run(binary, X, Y, R, tris, inserts, segs, rounds=False, serial=None):
    """The harness's triangles; with rounds=True the segments go through the
    GPU's claim rounds (the harness checks every winner writes only what it
    claimed) and `serial`, when given, receives how many were left to the
    one-at-a-time pass."""
    lines = [str(len(X))] + ["%d %d %d" % (x, y, r) for x, y, r in zip(X, Y, R)]
    lines += [str(len(tris))] + ["%d %d %d" % tuple(t) for t in tris]
    lines += [str(len(inserts))] + [str(int(p)) for p in inserts]
    lines += [str(len(segs))] + ["%d %d" % tuple(s) for s in segs]
    r = subprocess.run([binary] + (["rounds"] if rounds else []), input="\n".join(lines) + "\n",
                       capture_output=True, text=True, check=True)
    head, *rest = r.stdout.strip().split("\n")
    assert head.startswith("ok"), head
    if serial is not None:
        serial.append(int(head.split()[2]))
    return np.array([list(map(int, l.split())) for l in rest], np.int64)


def disk_case(seed, n=64, sites=140, ring=36, inner=4, radius=22.0, ring_r=25.0):
    """Lattice sites in a disk, constraint points on a jittered ring around
    it (most outside the sites' hull) and a few inside, segments along the
    ring (a closed polygon, as a mesh boundary gives)."""
    rng = np.random.default_rng(seed)
    cx = cy = n / 2
    cand = [(x, y) for x in range(n) for y in range(n) if (x - cx) ** 2 + (y - cy) ** 2 < radius ** 2]
    pick = rng.choice(len(cand), sites, replace=False)
    sp = np.array([cand[i] for i in sorted(pick)], np.int64)
    sp = sp[np.lexsort((sp[:, 1], sp[:, 0]))]  # x-major, as the library lists sites
    th = np.sort(rng.uniform(0, 2 * np.pi, ring))
    rr = ring_r + rng.uniform(-2.5, 2.5, ring)
    cpts = np.stack([cx + rr * np.cos(th), cy + rr * np.sin(th)], 1)
    ins = rng.uniform(cx - 10, cx + 10, (inner, 2))
    cpts = np.concatenate([cpts, ins])
    F = len(sp)
    X = np.concatenate([sp[:, 0] << SHIFT, np.rint(cpts[:, 0] * 2 ** SHIFT).astype(np.int64)])
    Y = np.concatenate([sp[:, 1] << SHIFT, np.rint(cpts[:, 1] * 2 ** SHIFT).astype(np.int64)])
    R = np.concatenate([sp[:, 1] * n + sp[:, 0], n * n + np.arange(len(cpts))])
    segs = np.array([(F + k, F + (k + 1) % ring) for k in range(ring)], np.int64)
    return sp, X, Y, R, segs, F, len(cpts)


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_host_cdt_is_constrained_delaunay(host_bin, seed):
    sp, X, Y, R, segs, F, C = disk_case(seed)
    tris = run(host_bin, X, Y, R, start_triangulation(sp), np.arange(F, F + C), segs)
    pts = np.stack([X, Y], 1)
    info = D.check_cdt(pts, tris, segs, R.tolist())
    assert info["constraints"] == len(segs)
    assert info["vertices"] == F + C


def test_host_cdt_on_a_full_lattice_block(host_bin):
    # many co-circular sites: every predicate tie goes through the perturbation
    n = 32
    sp = np.array([(x, y) for x in range(8, 24) for y in range(8, 24)], np.int64)
    rng = np.random.default_rng(7)
    cpts = np.array([(7.3, 7.6), (24.4, 8.2), (23.9, 24.7), (7.8, 23.3), (15.37, 15.61),
                     (12.1, 19.43)]) + rng.uniform(-0.01, 0.01, (6, 2))
    F = len(sp)
    X = np.concatenate([sp[:, 0] << SHIFT, np.rint(cpts[:, 0] * 2 ** SHIFT).astype(np.int64)])
    Y = np.concatenate([sp[:, 1] << SHIFT, np.rint(cpts[:, 1] * 2 ** SHIFT).astype(np.int64)])
    R = np.concatenate([sp[:, 1] * n + sp[:, 0], n * n + np.arange(len(cpts))])
    segs = np.array([(F, F + 1), (F + 1, F + 2), (F + 2, F + 3), (F + 3, F), (F + 4, F + 5)])
    tris = run(host_bin, X, Y, R, start_triangulation(sp), np.arange(F, F + 6), segs)
    info = D.check_cdt(np.stack([X, Y], 1), tris, segs, R.tolist())
    assert info["constraints"] == 5 and info["vertices"] == F + 6


def test_checker_rejects_a_missing_constraint(host_bin):
    sp, X, Y, R, segs, F, C = disk_case(11)
    pts = np.stack([X, Y], 1)
    # the plain Delaunay triangulation of all points misses some ring segment
    tris = run(host_bin, X, Y, R, start_triangulation(sp), np.arange(F, F + C), segs[:0])
    D.check_cdt(pts, tris, segs[:0], R.tolist())
    edges = {tuple(sorted(e)) for t in tris.tolist() for e in ((t[0], t[1]), (t[1], t[2]),
                                                               (t[2], t[0]))}
    missing = [s for s in segs.tolist() if tuple(sorted(s)) not in edges]
    if missing:
        with pytest.raises(AssertionError):
            D.check_cdt(pts, tris, segs, R.tolist())


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_host_cdt_recovers_long_segments_across_the_sites(host_bin, seed):
    # a sparse ring (segments crossing several edges) and a zigzag polyline
    # through the middle of the sites: each segment crosses many Delaunay
    # edges that Sloan's flips must remove
    sp, X, Y, R, segs, F, C = disk_case(seed, sites=220, ring=9, inner=0, radius=22.0,
                                        ring_r=21.5)
    rng = np.random.default_rng(seed)
    n = 64
    zig = np.stack([np.linspace(20.3, 43.7, 6), 32 + rng.uniform(-6, 6, 6)], 1)
    X = np.concatenate([X, np.rint(zig[:, 0] * 2 ** SHIFT).astype(np.int64)])
    Y = np.concatenate([Y, np.rint(zig[:, 1] * 2 ** SHIFT).astype(np.int64)])
    R = np.concatenate([R, n * n + C + np.arange(6)])
    segs = np.concatenate([segs, [(F + C + k, F + C + k + 1) for k in range(5)]])
    tris = run(host_bin, X, Y, R, start_triangulation(sp), np.arange(F, F + C + 6), segs)
    pts = np.stack([X, Y], 1)
    # the plain Delaunay triangulation misses several of these segments
    dt = run(host_bin, X, Y, R, start_triangulation(sp), np.arange(F, F + C + 6), segs[:0])
    edges = {tuple(sorted(e)) for t in dt.tolist() for e in ((t[0], t[1]), (t[1], t[2]),
                                                             (t[2], t[0]))}
    assert sum(tuple(sorted(s)) not in edges for s in segs.tolist()) >= 3
    info = D.check_cdt(pts, tris, segs, R.tolist())
    assert info["constraints"] == len(segs)


def test_host_cdt_reports_crossing_segments(host_bin):
    # two constraint segments that cross each other: invalid input, reported
    sp, X, Y, R, segs, F, C = disk_case(31, ring=0, inner=0)
    n = 64
    extra = np.array([(20.5, 32.3), (44.5, 31.7), (32.4, 20.2), (31.6, 44.1)])
    X = np.concatenate([X, np.rint(extra[:, 0] * 2 ** SHIFT).astype(np.int64)])
    Y = np.concatenate([Y, np.rint(extra[:, 1] * 2 ** SHIFT).astype(np.int64)])
    R = np.concatenate([R, n * n + np.arange(4)])
    tris = start_triangulation(sp)
    lines = [str(len(X))] + ["%d %d %d" % (x, y, r) for x, y, r in zip(X, Y, R)]
    lines += [str(len(tris))] + ["%d %d %d" % tuple(t) for t in tris]
    lines += ["4"] + [str(F + k) for k in range(4)]
    lines += ["2", "%d %d" % (F, F + 1), "%d %d" % (F + 2, F + 3)]
    out = subprocess.run([host_bin], input="\n".join(lines) + "\n", capture_output=True,
                         text=True, check=True).stdout
    assert out.startswith("error segment 4"), out


def test_host_cdt_splits_a_segment_at_points_inside_it(host_bin):
    # lattice sites exactly on a constraint segment: the segment becomes the
    # chain of edges between them
    sp, X, Y, R, segs, F, C = disk_case(41, ring=0, inner=0)
    n = 64
    on = [k for k in range(F) if sp[k, 1] == 32 and 18 <= sp[k, 0] <= 46]
    extra = np.array([(17.5, 32.0), (46.5, 32.0)])
    X = np.concatenate([X, np.rint(extra[:, 0] * 2 ** SHIFT).astype(np.int64)])
    Y = np.concatenate([Y, np.rint(extra[:, 1] * 2 ** SHIFT).astype(np.int64)])
    R = np.concatenate([R, n * n + np.arange(2)])
    segs = np.array([(F, F + 1)])
    tris = run(host_bin, X, Y, R, start_triangulation(sp), [F, F + 1], segs)
    info = D.check_cdt(np.stack([X, Y], 1), tris, segs, R.tolist())
    assert len(on) >= 1 and info["constraints"] == len(on) + 1


@pytest.mark.parametrize("seed", [1, 2, 3, 21, 22])
def test_claim_rounds_give_the_sequential_result(host_bin, seed):
    # the GPU's parallel segment rounds, replayed: winners touch only what
    # they claimed, and the result is the unique constrained Delaunay
    # triangulation, the same as segment after segment
    if seed < 20:
        sp, X, Y, R, segs, F, C = disk_case(seed, ring=48, inner=0, ring_r=21.0)
    else:
        sp, X, Y, R, segs, F, C = disk_case(seed, sites=220, ring=12, inner=0, ring_r=21.5)
    start = start_triangulation(sp)
    ins = np.arange(F, F + C)
    seq = run(host_bin, X, Y, R, start, ins, segs)
    serial = []
    par = run(host_bin, X, Y, R, start, ins, segs, rounds=True, serial=serial)
    assert np.array_equal(seq, par)
    D.check_cdt(np.stack([X, Y], 1), par, segs, R.tolist())
    assert serial[0] < len(segs)  # most segments recovered in the rounds
