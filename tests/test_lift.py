"""Lift to the surface and per-vertex weights: recover() (recover.h:98-157) and
weighting_vertices_with_area() (weighting.h:38-97).

CPU: the oracle's restatement against the fixtures recorded from the
reference's own headers (tests/golden/ref_lift.npz) and, where the reference
build exists, against it on fresh inputs.  GPU: gcvt_lift /
gcvt_vertex_weights bit for bit against the fixtures and the oracle."""
import os
import sys

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLD)


def same_f64(a, b):
    """Bit-identical doubles, any NaN equal to any NaN."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if a.shape != b.shape:
        return False
    nan = np.isnan(a)
    return bool((nan == np.isnan(b)).all() and
                (a[~nan].view(np.uint64) == b[~nan].view(np.uint64)).all())


@pytest.fixture(scope="module")
def lift_npz():
    return np.load(os.path.join(GOLD, "ref_lift.npz"))


def golden_cases(z):
    i = 0
    while "uv%d" % i in z:
        yield (str(z["name%d" % i]), z["uv%d" % i], z["xyz%d" % i], z["tris%d" % i],
               z["points%d" % i], z["fixed%d" % i], z["cdt%d" % i], z["lifted%d" % i],
               z["keep%d" % i], z["weights%d" % i])
        i += 1


def test_golden_cases_cover_the_edge_cases(lift_npz):
    names = [c[0] for c in golden_cases(lift_npz)]
    assert names == ["disk_small", "disk_mid", "degenerate", "nonfinite"]
    for name, uv, xyz, tris, pts, fixed, cdt, lifted, keep, w in golden_cases(lift_npz):
        nfree = len(pts) - len(fixed)
        assert np.isnan(lifted[0]).all(), name           # first point unlocated
        assert 0 < keep.sum() <= len(keep), name
        if name == "degenerate":
            assert not keep.all()
            assert np.isnan(w).sum() == 1                # the vertex on no face
            assert (w == np.nanmax(w)).sum() >= 3       # ratios over 1e10 -> the maximum
        if name == "nonfinite":
            assert not np.isfinite(pts[:nfree]).all()


def test_oracle_lift_equals_reference(oracle, lift_npz):
    for name, uv, xyz, tris, pts, fixed, cdt, lifted, keep, w in golden_cases(lift_npz):
        got, face, k = oracle.lift(uv, xyz, tris, pts, fixed, cdt)
        assert same_f64(got, lifted), name
        assert np.array_equal(k, keep), name
        assert same_f64(oracle.vertex_weights(uv, xyz, tris), w), name


def test_oracle_against_reference_build_on_fresh_inputs(oracle):
    if not oracle.recover_ref_available():
        pytest.skip("reference recover.h build absent (needs the reference checkout)")
    import make_golden_lift as mk
    for seed in range(3):
        uv, xyz, tris, pts, fixed, cdt = mk.case_disk(100 + seed, 16 + 8 * seed, 400, 10)
        got, _, k = oracle.lift(uv, xyz, tris, pts, fixed, cdt)
        want, kw = oracle.ref_lift(uv, xyz, tris, pts, fixed, cdt)
        assert same_f64(got, want) and np.array_equal(k, kw), seed
        assert same_f64(oracle.vertex_weights(uv, xyz, tris),
                        oracle.ref_vertex_weights(uv, xyz, tris)), seed


def test_oracle_lift_properties(oracle):
    """Located points reproduce the mesh: a vertex lifts to its own surface
    point (weights exactly 1, 0, 0 on some face) and constraint points keep
    theirs."""
    from workloads import disk_surface
    uv, xyz, tris = disk_surface(12, seed=3)
    fixed = np.arange(0, len(uv), 7, dtype=np.int32)
    pts = np.concatenate([uv, uv[fixed]])
    got, face, _ = oracle.lift(uv, xyz, tris, pts, fixed)
    assert (face[:len(uv)] >= 0).all()
    assert np.allclose(got[:len(uv)], xyz, atol=1e-12)
    assert same_f64(got[len(uv):], xyz[fixed])


@pytest.mark.gpu
def test_gpu_lift_equals_reference_fixtures(gcvt_lib, lift_npz):
    for name, uv, xyz, tris, pts, fixed, cdt, lifted, keep, w in golden_cases(lift_npz):
        got, face, k = gcvt_lib.lift(uv, xyz, tris, pts, fixed, cdt)
        assert same_f64(got, lifted), name
        assert np.array_equal(k, keep), name
        assert same_f64(gcvt_lib.vertex_weights(uv, xyz, tris), w), name


@pytest.mark.gpu
def test_gpu_lift_equals_oracle_larger(gcvt_lib, oracle):
    """A 5,000-point query set on a 96 x 96-vertex disk mesh (17k faces),
    faces reported too."""
    from workloads import disk_surface
    rng = np.random.default_rng(7)
    uv, xyz, tris = disk_surface(96, seed=7)
    pts = np.concatenate([rng.uniform(-0.02, 1.02, (4000, 2)), uv[::17],
                          (uv[tris[::9, 0]] + uv[tris[::9, 2]]) / 2])
    fixed = np.arange(0, len(uv), 101, dtype=np.int32)
    pts = np.concatenate([pts, uv[fixed]])
    from scipy.spatial import Delaunay
    cdt = Delaunay(pts).simplices.astype(np.int32)
    want, wface, wkeep = oracle.lift(uv, xyz, tris, pts, fixed, cdt)
    got, face, keep = gcvt_lib.lift(uv, xyz, tris, pts, fixed, cdt)
    assert np.array_equal(face, wface)
    assert same_f64(got, want)
    assert np.array_equal(keep, wkeep)
    assert same_f64(gcvt_lib.vertex_weights(uv, xyz, tris), oracle.vertex_weights(uv, xyz, tris))


@pytest.mark.gpu
def test_gpu_lift_full_size_properties(gcvt_lib, oracle):
    """65,536 points on the 256 x 256-vertex disk mesh of the mesh-driven
    workload (93k faces): the located faces pass the reference's test and no
    lower-index face does (checked against every face for a sample)."""
    from workloads import disk_surface
    rng = np.random.default_rng(9)
    uv, xyz, tris = disk_surface(256, seed=2)
    pts = rng.uniform(0.0, 1.0, (65536, 2))
    got, face, _ = gcvt_lib.lift(uv, xyz, tris, pts)
    sample = rng.choice(len(pts), 300, replace=False)
    want, wface, _ = oracle.lift(uv, xyz, tris, pts[sample])
    located = wface >= 0
    assert np.array_equal(face[sample][located], wface[located])
    assert same_f64(got[sample][located], want[located])
    r = np.hypot(pts[:, 0] - 0.5, pts[:, 1] - 0.5)
    assert (face[r < 0.45] >= 0).all() and (face[r > 0.49] < 0).all()


@pytest.mark.gpu
def test_gpu_lift_device_memory_and_errors(gcvt_lib):
    import torch
    from workloads import disk_surface
    uv, xyz, tris = disk_surface(20, seed=4)
    rng = np.random.default_rng(4)
    pts = rng.uniform(0, 1, (500, 2))
    want, wface, _ = gcvt_lib.lift(uv, xyz, tris, pts)
    lib = gcvt_lib.load_library()
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda()
         for k, v in dict(uv=uv, xyz=xyz, tris=tris, pts=pts).items()}
    out = torch.empty((500, 3), dtype=torch.float64, device="cuda")
    face = torch.empty(500, dtype=torch.int32, device="cuda")
    rc = lib.gcvt_lift(d["uv"].data_ptr(), d["xyz"].data_ptr(), len(uv), d["tris"].data_ptr(),
                       len(tris), d["pts"].data_ptr(), 500, 0, None, None, 0, out.data_ptr(),
                       face.data_ptr(), None, gcvt_lib.MEM_DEVICE)
    assert rc == 0
    assert same_f64(out.cpu().numpy(), want) and np.array_equal(face.cpu().numpy(), wface)
    bad = tris.copy()
    bad[3, 1] = len(uv)
    with pytest.raises(RuntimeError):
        gcvt_lib.lift(uv, xyz, bad, pts)
    with pytest.raises(RuntimeError):
        gcvt_lib.lift(uv, xyz, tris, pts, cdt=np.array([[0, 1, 500]], np.int32))
    with pytest.raises(RuntimeError):
        gcvt_lib.vertex_weights(uv, xyz, bad)
    empty, eface, ekeep = gcvt_lib.lift(uv, xyz, tris, np.zeros((0, 2)))
    assert empty.shape == (0, 3) and ekeep.shape == (0,)


@pytest.mark.gpu
def test_gpu_lift_slivers_equal_oracle(gcvt_lib, oracle):
    """Flat triangles from conditioning 1e2 to 1e20 (binned with widened boxes,
    or tested by every point), queried on and around them."""
    rng = np.random.default_rng(21)
    uv, tris = [], []
    for k, h in enumerate(10.0 ** -np.arange(1, 11)):
        y0 = 0.05 + 0.09 * k
        base = len(uv)
        a, b = np.array([0.1, y0]), np.array([0.9, y0 + 1e-3 * k])
        c = a + (0.5 + 0.01 * k) * (b - a) + np.array([0.0, h])   # h above the long edge
        uv += [a.tolist(), b.tolist(), c.tolist()]
        tris.append([base, base + 1, base + 2])
        tris.append([base + 1, base, base + 2])   # the same sliver, other orientation
    uv = np.array(uv)
    xyz = np.concatenate([uv, rng.normal(0, 1, (len(uv), 1))], 1)
    tris = np.array(tris, np.int32)
    near = []
    for t in tris[::2]:
        a, b, c = uv[t]
        s = rng.random((300, 2))
        near.append(a + s[:, :1] * (b - a) + s[:, 1:] * (c - a) * rng.uniform(-2, 3, (300, 1)))
        near.append(a + rng.random((100, 1)) * (b - a))          # on the long edge
    pts = np.concatenate(near + [rng.uniform(0, 1, (500, 2))])
    want, wface, _ = oracle.lift(uv, xyz, tris, pts)
    got, face, _ = gcvt_lib.lift(uv, xyz, tris, pts)
    assert np.array_equal(face, wface)
    assert same_f64(got, want)
