"""The drop-in boundary from C++: a program that calls gCVT and
discretization_d with the reference's signatures (gcvt.h:29,
discretization.h:66) links against libgcvt_gb300.so (CPU check) and, on a
GPU, returns the same grids as the library's other entry points and the
oracle."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def dropin_exe(gcvt_lib, tmp_path_factory):
    libdir = os.path.dirname(gcvt_lib.LIB_PATH)
    if not os.path.exists(gcvt_lib.LIB_PATH):
        pytest.skip("library not built")
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_main")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "dropin_main.cpp"),
                        "-L" + libdir, "-lgcvt_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_signatures_link(dropin_exe):
    assert os.path.exists(dropin_exe)


@pytest.mark.gpu
def test_gcvt_symbol_equals_library(dropin_exe, gcvt_lib, oracle, tmp_path, cuda_device):
    from workloads import small_case
    n = 512
    sites, rho, mask = small_case(n, 1500, seed=44)
    mask = mask.copy()
    mask[100:103, 200] = 1            # three fixed sites (the pixels hold their coordinates)
    sites[100:103, 200, 0] = 200
    sites[100:103, 200, 1] = np.arange(100, 103)
    paths = [str(tmp_path / f) for f in ("s.bin", "d.bin", "m.bin", "out.bin")]
    sites.tofile(paths[0])
    rho.tofile(paths[1])
    mask.astype(np.uint8).tofile(paths[2])
    r = subprocess.run([dropin_exe, "gcvt", paths[0], paths[1], paths[2], str(n), "1", "200",
                        paths[3]], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(paths[3], np.int16).reshape(n, n, 2)
    want = gcvt_lib.gcvt(sites.copy(), rho, mask, depth=1, max_iter=200)
    assert np.array_equal(got, want)
    # the output is the exact labelling of the sites it ends with
    final = np.full_like(got, -32768)
    ys, xs = np.nonzero((got[..., 0] == np.arange(n)[None, :]) & (got[..., 1] == np.arange(n)[:, None]))
    final[ys, xs, 0], final[ys, xs, 1] = xs, ys
    assert np.array_equal(got, oracle.pba_label(final))


@pytest.mark.gpu
def test_discretization_symbol_equals_oracle(dropin_exe, oracle, tmp_path, cuda_device):
    from workloads import disk_mesh, raster_inputs
    P, w, T = disk_mesh(24, seed=3)
    Q, scale, _, _ = raster_inputs(P, 256)
    paths = [str(tmp_path / f) for f in ("p.bin", "w.bin", "t.bin", "out.bin")]
    np.ascontiguousarray(Q).tofile(paths[0])
    w.tofile(paths[1])
    T.astype(np.int32).tofile(paths[2])
    r = subprocess.run([dropin_exe, "raster", paths[0], paths[1], str(len(w)), paths[2],
                        str(len(T)), repr(float(scale)), "256", paths[3]],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(paths[3], np.float32).reshape(256, 256)
    want = oracle.rasterize(Q, w, T, scale, 256)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
