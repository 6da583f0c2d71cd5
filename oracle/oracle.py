"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/liboracle.so (the C restatement of gcvt.cu's algorithm)
and, where present, oracle/_build/librefh.so with the reference's kernels
from oracle/_ref/*.cubin.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference legs use this module.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
MARKER = -32768
P, I = ctypes.c_void_p, ctypes.c_int

FAITHFUL, EXACT = 0, 1


class OrcStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("levels", ctypes.c_int),
                ("last_energy", ctypes.c_double), ("omega", ctypes.c_float)]


_lib = None
_refh = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(BUILD, "liboracle.so")
        if not os.path.exists(path):
            from build_oracle import build_oracle  # noqa: local build on demand
            build_oracle()
        L = ctypes.CDLL(path)
        for f in ("orc_pba_label", "orc_spec_label", "orc_brute_label"):
            getattr(L, f).argtypes = [P, P, I]
            getattr(L, f).restype = I
        L.orc_gcvt.argtypes = [P, P, P, I, I, I, I, I, I, ctypes.POINTER(OrcStats)]
        L.orc_gcvt.restype = I
        L.orc_lloyd_step.argtypes = [P, P, P, I, ctypes.c_float, P, P, P, P]
        L.orc_lloyd_step.restype = I
        L.orc_faithful_step.argtypes = [P, P, P, I, ctypes.c_float, P, P, P]
        L.orc_faithful_step.restype = I
        L.orc_faithful_energy.argtypes = [P, P, I, I]
        L.orc_faithful_energy.restype = ctypes.c_float
        L.orc_rasterize.argtypes = [P, P, I, P, I, P, ctypes.c_double, I, I]
        L.orc_rasterize.restype = I
        L.orc_seed_sites.argtypes = [P, P, P, I, I, ctypes.c_longlong]
        L.orc_seed_sites.restype = I
        L.orc_lift.argtypes = [P, P, I, P, I, P, I, I, P, P, I, P, P, P, I]
        L.orc_lift.restype = I
        L.orc_vertex_weights.argtypes = [P, P, I, P, I, P]
        L.orc_vertex_weights.restype = I
        _lib = L
    return _lib


def _chk(rc, name):
    if rc < 0:
        raise RuntimeError("%s failed: %d" % (name, rc))
    return rc


def pba_label(sites):
    n = sites.shape[0]
    out = np.empty_like(sites)
    _chk(lib().orc_pba_label(sites.ctypes.data, out.ctypes.data, n), "orc_pba_label")
    return out


def spec_label(sites):
    n = sites.shape[0]
    out = np.empty_like(sites)
    _chk(lib().orc_spec_label(sites.ctypes.data, out.ctypes.data, n), "orc_spec_label")
    return out


def brute_label(sites):
    n = sites.shape[0]
    out = np.empty_like(sites)
    _chk(lib().orc_brute_label(sites.ctypes.data, out.ctypes.data, n), "orc_brute_label")
    return out


def gcvt(voronoi, density, mask, depth=1, max_iter=1000, mode=EXACT, fixed_iters=0, threads=0):
    """Restated gCVT; returns (labels, stats dict).  voronoi is not modified."""
    v = np.ascontiguousarray(voronoi).copy()
    n = v.shape[0]
    st = OrcStats()
    _chk(lib().orc_gcvt(v.ctypes.data, np.ascontiguousarray(density, np.float32).ctypes.data,
                        np.ascontiguousarray(mask, np.uint8).ctypes.data, n, depth, max_iter,
                        mode, fixed_iters, threads, ctypes.byref(st)), "orc_gcvt")
    return v, {k: getattr(st, k) for k, _ in st._fields_}


def lloyd_step(sites, density, mask, omega):
    """One exact-mode Lloyd step: (labels, moments[3,n,n], energy, new_sites)."""
    n = sites.shape[0]
    labels = np.empty_like(sites)
    mom = np.empty((3, n, n), np.float64)
    e = ctypes.c_double()
    out = np.empty_like(sites)
    _chk(lib().orc_lloyd_step(sites.ctypes.data, density.ctypes.data,
                              np.ascontiguousarray(mask, np.uint8).ctypes.data, n,
                              ctypes.c_float(omega), labels.ctypes.data, mom.ctypes.data,
                              ctypes.byref(e), out.ctypes.data), "orc_lloyd_step")
    return labels, mom, e.value, out


def faithful_step(sites, density, mask, omega):
    """One faithful Lloyd step: (labels, totals[3,n,n] float32, new_sites)."""
    n = sites.shape[0]
    labels = np.empty_like(sites)
    tot = np.empty((3, n, n), np.float32)
    out = np.empty_like(sites)
    _chk(lib().orc_faithful_step(sites.ctypes.data, density.ctypes.data,
                                 np.ascontiguousarray(mask, np.uint8).ctypes.data, n,
                                 ctypes.c_float(omega), labels.ctypes.data, tot.ctypes.data,
                                 out.ctypes.data), "orc_faithful_step")
    return labels, tot, out


def faithful_energy(labels, density, level=0):
    return float(lib().orc_faithful_energy(labels.ctypes.data, density.ctypes.data,
                                           labels.shape[0], level))


def rasterize(points, weight, triangles, scale, n, threads=0):
    out = np.empty((n, n), np.float32)
    _chk(lib().orc_rasterize(points.ctypes.data, weight.ctypes.data, len(weight),
                             triangles.ctypes.data, len(triangles), out.ctypes.data,
                             ctypes.c_double(scale), n, threads), "orc_rasterize")
    return out


def seed_sites(density, mask, num, seed=-1):
    n = density.shape[0]
    v = np.empty((n, n, 2), np.int16)
    _chk(lib().orc_seed_sites(v.ctypes.data, density.ctypes.data,
                              np.ascontiguousarray(mask, np.uint8).ctypes.data, num, n, seed),
         "orc_seed_sites")
    return v


def _lift_args(uv, xyz, triangles, points, fixed, cdt):
    uv = np.ascontiguousarray(uv, np.float64)
    xyz = np.ascontiguousarray(xyz, np.float64)
    tri = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    pts = np.ascontiguousarray(points, np.float64).reshape(-1, 2)
    fixed = np.ascontiguousarray(np.zeros(0) if fixed is None else fixed, np.int32).ravel()
    cdt = np.ascontiguousarray(np.zeros((0, 3)) if cdt is None else cdt, np.int32).reshape(-1, 3)
    return uv, xyz, tri, pts, fixed, cdt


def lift(uv, xyz, triangles, points, fixed=None, cdt=None, threads=0):
    """recover (recover.h:98-157) restated: (lifted xyz (P, 3), face (P,),
    keep (C,) bool); the last len(fixed) points are the constraint points."""
    uv, xyz, tri, pts, fixed, cdt = _lift_args(uv, xyz, triangles, points, fixed, cdt)
    out = np.empty((len(pts), 3), np.float64)
    face = np.empty(len(pts), np.int32)
    keep = np.empty(len(cdt), np.uint8)
    _chk(lib().orc_lift(uv.ctypes.data, xyz.ctypes.data, len(uv), tri.ctypes.data, len(tri),
                        pts.ctypes.data, len(pts), len(fixed), fixed.ctypes.data, cdt.ctypes.data,
                        len(cdt), out.ctypes.data, face.ctypes.data, keep.ctypes.data, threads),
         "orc_lift")
    return out, face, keep.astype(bool)


def vertex_weights(uv, xyz, triangles):
    """weighting_vertices_with_area (weighting.h:38-97) restated."""
    uv, xyz, tri, _, _, _ = _lift_args(uv, xyz, triangles, np.zeros((0, 2)), None, None)
    w = np.empty(len(uv), np.float64)
    _chk(lib().orc_vertex_weights(uv.ctypes.data, xyz.ctypes.data, len(uv), tri.ctypes.data,
                                  len(tri), w.ctypes.data), "orc_vertex_weights")
    return w


_recover_ref = None


def recover_ref_available():
    return os.path.exists(os.path.join(REF, "librecover_ref.so"))


def _rr():
    global _recover_ref
    if _recover_ref is None:
        R = ctypes.CDLL(os.path.join(REF, "librecover_ref.so"))
        R.refr_recover.argtypes = [P, P, I, P, I, P, I, P, I, P, I, P, P]
        R.refr_recover.restype = I
        R.refr_weights.argtypes = [P, P, I, P, I, P]
        R.refr_weights.restype = I
        _recover_ref = R
    return _recover_ref


def ref_lift(uv, xyz, triangles, points, fixed=None, cdt=None):
    """The reference's own recover() (recover.h, compiled by ref_recover.cpp):
    (lifted xyz (P, 3), keep (C,) bool)."""
    uv, xyz, tri, pts, fixed, cdt = _lift_args(uv, xyz, triangles, points, fixed, cdt)
    out = np.empty((len(pts), 3), np.float64)
    keep = np.empty(len(cdt), np.uint8)
    _chk(_rr().refr_recover(uv.ctypes.data, xyz.ctypes.data, len(uv), tri.ctypes.data, len(tri),
                            pts.ctypes.data, len(pts), fixed.ctypes.data, len(fixed),
                            cdt.ctypes.data, len(cdt), out.ctypes.data, keep.ctypes.data),
         "refr_recover")
    return out, keep.astype(bool)


def ref_vertex_weights(uv, xyz, triangles):
    """The reference's own weighting_vertices_with_area (weighting.h)."""
    uv, xyz, tri, _, _, _ = _lift_args(uv, xyz, triangles, np.zeros((0, 2)), None, None)
    w = np.empty(len(uv), np.float64)
    _chk(_rr().refr_weights(uv.ctypes.data, xyz.ctypes.data, len(uv), tri.ctypes.data, len(tri),
                            w.ctypes.data), "refr_weights")
    return w


# ---- the reference's own kernels -------------------------------------------

def seed_ref_available():
    return os.path.exists(os.path.join(REF, "libseed_ref.so"))


_seed = None


def _sr():
    global _seed
    if _seed is None:
        S = ctypes.CDLL(os.path.join(REF, "libseed_ref.so"))
        S.refseed_state.argtypes = [P, P]
        S.refseed_state.restype = None
        S.refseed_sites.argtypes = [P, P, P, I, I]
        S.refseed_sites.restype = None
        _seed = S
    return _seed


def ref_seed_sites(density, mask, num, state=None):
    """The reference's own putConstrains + randomPoints (gcvt.h:56-122,
    compiled from the checkout into oracle/_ref/libseed_ref.so).  state: the
    generator's (z, w, jsr, jcong) to start from (None: zeros, the unseeded
    globals); returns (site grid, state after)."""
    S = _sr()
    n = density.shape[0]
    st = np.zeros(4, np.uint64) if state is None else np.array(state, np.uint64)
    S.refseed_state(None, st.ctypes.data)
    v = np.empty((n, n, 2), np.int16)
    d = np.ascontiguousarray(density, np.float32).copy()
    S.refseed_sites(v.ctypes.data, d.ctypes.data,
                    np.ascontiguousarray(mask, np.uint8).ctypes.data, int(num), n)
    after = np.zeros(4, np.uint64)
    S.refseed_state(after.ctypes.data, None)
    return v, after


def ref_available():
    return (os.path.exists(os.path.join(REF, "gcvt_ref.cubin")) and
            os.path.exists(os.path.join(BUILD, "librefh.so")))


def refh():
    """The reference-kernel harness; needs a GPU and the cubins."""
    global _refh
    if _refh is None:
        path = os.path.join(BUILD, "librefh.so")
        if not os.path.exists(path):
            from build_oracle import build_harness
            build_harness()
        R = ctypes.CDLL(path)
        R.refh_init.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        R.refh_pba_label.argtypes = [P, P, I]
        R.refh_energy.argtypes = [P, P, I, ctypes.POINTER(ctypes.c_float)]
        R.refh_lloyd_step.argtypes = [P, P, P, I, ctypes.c_float, P, P, P]
        R.refh_gcvt.argtypes = [P, P, P, I, I, I, I, P, I, P, P]
        R.refh_rasterize.argtypes = [P, P, I, P, I, P, ctypes.c_double, I, P]
        raster = os.path.join(REF, "raster_ref.cubin")
        rc = R.refh_init(os.path.join(REF, "gcvt_ref.cubin").encode(),
                         raster.encode() if os.path.exists(raster) else None)
        if rc != 0:
            raise RuntimeError("refh_init failed: %d" % rc)
        _refh = R
    return _refh


def ref_pba_label(sites):
    n = sites.shape[0]
    out = np.empty_like(sites)
    _chk(refh().refh_pba_label(sites.ctypes.data, out.ctypes.data, n), "refh_pba_label")
    return out


def ref_energy(labels, density):
    e = ctypes.c_float()
    _chk(refh().refh_energy(labels.ctypes.data, density.ctypes.data, labels.shape[0],
                            ctypes.byref(e)), "refh_energy")
    return e.value


def ref_lloyd_step(sites, density, mask, omega):
    n = sites.shape[0]
    labels = np.empty_like(sites)
    tot = np.empty((3, n, n), np.float32)
    out = np.empty_like(sites)
    _chk(refh().refh_lloyd_step(sites.ctypes.data, density.ctypes.data,
                                np.ascontiguousarray(mask, np.uint8).ctypes.data, n,
                                ctypes.c_float(omega), labels.ctypes.data, tot.ctypes.data,
                                out.ctypes.data), "refh_lloyd_step")
    return labels, tot, out


def ref_gcvt(voronoi, density, mask, depth=1, max_iter=1000, fixed_iters=0):
    """The reference's kernels under gCVT's loop; returns (labels, info)."""
    v = np.ascontiguousarray(voronoi).copy()
    n = v.shape[0]
    energies = np.zeros(4096, np.float32)
    stats = np.zeros(3, np.int32)
    times = np.zeros(2, np.float32)
    _chk(refh().refh_gcvt(v.ctypes.data, np.ascontiguousarray(density, np.float32).ctypes.data,
                          np.ascontiguousarray(mask, np.uint8).ctypes.data, n, depth, max_iter,
                          fixed_iters, energies.ctypes.data, len(energies), stats.ctypes.data,
                          times.ctypes.data), "refh_gcvt")
    ne = int(stats[1])
    return v, {"iterations": int(stats[0]), "omega": float(stats[2:3].view(np.float32)[0]),
               "energies": energies[:min(ne, 4096)].tolist(),
               "total_ms": float(times[0]), "loop_ms": float(times[1])}


def ref_rasterize(points, weight, triangles, scale, n):
    out = np.empty((n, n), np.float32)
    t = ctypes.c_float()
    _chk(refh().refh_rasterize(points.ctypes.data, weight.ctypes.data, len(weight),
                               triangles.ctypes.data, len(triangles), out.ctypes.data,
                               ctypes.c_double(scale), n, ctypes.byref(t)), "refh_rasterize")
    return out, t.value
