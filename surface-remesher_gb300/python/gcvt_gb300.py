"""ctypes binding of libgcvt_gb300.so (include/gcvt_gb300.h).

The Python mirror of the reference's CVT interface (source/gcvt.h):
  * ``gcvt(voronoi, density, mask, depth, max_iter)`` -- gCVT (gcvt.h:29):
    site grid in, label grid out, in place on ``voronoi``;
  * ``label_grid(sites)`` -- one exact labelling pass (pba2DCompute);
  * ``Context`` -- the context API: load once, label / iterate / run / read
    back, with host (numpy) or device (objects exposing ``data_ptr()``, e.g.
    torch CUDA tensors) buffers.

Grids follow the reference: a site/label grid is an int16 array of shape
(n, n, 2) holding (x, y) per pixel, MARKER = -32768 where there is no site.
There is no fallback: every call runs the CUDA library, and loading fails
loudly when the library is missing.
"""
import ctypes
import os

import numpy as np

MARKER = -32768
MEM_HOST, MEM_DEVICE = 0, 1

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.normpath(os.path.join(_HERE, "..", "lib", "libgcvt_gb300.so"))

STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported grid size", 3: "CUDA runtime error",
          4: "invalid input data (a site pixel not holding its own coordinates, a Delaunay "
             "star over 64 neighbours)", 5: "no problem loaded",
          6: "allocation failed"}


class GcvtError(RuntimeError):
    def __init__(self, code, where):
        super().__init__("%s: %s (status %d)" % (where, STATUS.get(code, "unknown"), code))
        self.code = code


class Tuning(ctypes.Structure):
    _fields_ = [("cell_blocks_per_sm", ctypes.c_int), ("hint_slack", ctypes.c_int),
                ("jfa_tail_halo", ctypes.c_int), ("lloyd_ms", ctypes.c_float),
                ("jfa_ms", ctypes.c_float), ("cell_mode", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RunInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("levels", ctypes.c_int),
                ("omega", ctypes.c_float), ("energy", ctypes.c_double),
                ("sampled_energy", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol the header declares, with its ctypes signature.
P, I = ctypes.c_void_p, ctypes.c_int
SIGNATURES = {
    "gcvt_status_string": ([I], ctypes.c_char_p),
    "gcvt_version": ([], I),
    "gcvt_ctx_create": ([I, ctypes.POINTER(P)], I),
    "gcvt_ctx_destroy": ([P], I),
    "gcvt_ctx_set_stream": ([P, P], I),
    "gcvt_ctx_load": ([P, I, P, P, P, I], I),
    "gcvt_ctx_label": ([P, P, I], I),
    "gcvt_ctx_iterate": ([P, I], I),
    "gcvt_ctx_run": ([P, I, I, ctypes.POINTER(RunInfo)], I),
    "gcvt_ctx_sites": ([P, P, I], I),
    "gcvt_ctx_moments": ([P, P, I], I),
    "gcvt_ctx_info": ([P, ctypes.POINTER(RunInfo)], I),
    "gcvt_ctx_time_kernels": ([P, I, P], I),
    "gcvt_compute": ([P, P, P, I, I, I], I),
    "gcvt_label_grid": ([P, P, I, I], I),
    "gcvt_label_grid_static": ([P, P, I, P], I),
    "gcvt_rasterize": ([P, P, I, P, I, P, ctypes.c_double, I, I], I),
    "gcvt_ctx_extract_points": ([P, ctypes.c_double, ctypes.c_double, ctypes.c_double, P, I,
                                 ctypes.POINTER(I), I], I),
    "gcvt_ctx_delaunay": ([P, P, I, ctypes.POINTER(I), I], I),
    "gcvt_ctx_cdt": ([P, ctypes.c_double, ctypes.c_double, ctypes.c_double, P, I, P, I, P, I,
                      ctypes.POINTER(I), ctypes.POINTER(I), I], I),
    "gcvt_seed_sites": ([P, P, P, I, I, P], I),
    "gcvt_ctx_jfa_label": ([P, P, P, I], I),
    "gcvt_ctx_autotune": ([P, ctypes.POINTER(Tuning)], I),
    "gcvt_mlp_param_count": ([], I),
    "gcvt_ctx_learning": ([P, I, I], I),
    "gcvt_ctx_set_mlp": ([P, P, I], I),
    "gcvt_ctx_features": ([P, P, P, P, I, ctypes.POINTER(I)], I),
    "gcvt_ctx_iterate_learned": ([P, I, I, ctypes.POINTER(I), ctypes.POINTER(I)], I),
    "gcvt_ctx_set_target_energy": ([P, ctypes.c_double], I),
    "gcvt_batch_set_mlp": ([P, P, I], I),
    "gcvt_batch_iterate_learned": ([P, I, I, ctypes.POINTER(I), ctypes.POINTER(I)], I),
    "gcvt_mlp_forward": ([P, P, I, P, I], I),
    "gcvt_mlp_train": ([P, ctypes.c_longlong, P, I, I, ctypes.c_float, ctypes.c_ulonglong, P], I),
    "gcvt_mlp_gradient": ([P, ctypes.c_longlong, P, I, ctypes.c_ulonglong, I, P, P], I),
    "gcvt_ctx_set_tuning": ([P, ctypes.POINTER(Tuning)], I),
    "gcvt_batch_create": ([I, P, ctypes.POINTER(P)], I),
    "gcvt_batch_destroy": ([P], I),
    "gcvt_batch_set_stream": ([P, P], I),
    "gcvt_batch_iterate": ([P, I], I),
    "gcvt_batch_run": ([P, I, P], I),
    "gcvt_centroidal_voronoi": ([P, P, P, I, I, I, I], I),
    "gcvt_lift": ([P, P, I, P, I, P, I, I, P, P, I, P, P, P, I], I),
    "gcvt_vertex_weights": ([P, P, I, P, I, P, I], I),
}
CPP_SYMBOLS = {"gCVT": "_Z4gCVTPsPfPbiii",
               "discretization_d": "_Z16discretization_dPdS_iPiiPfdi"}

_lib = None


def load_library(path=None):
    """Load libgcvt_gb300.so (raises OSError when it is not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    lib = ctypes.CDLL(path or LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if path is None:
        _lib = lib
    return lib


def _check(code, where):
    if code != 0:
        raise GcvtError(code, where)


def _host_ptr(a, dtype, shape=None):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous %s numpy array" % np.dtype(dtype))
    if shape is not None and a.shape != shape:
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return a.ctypes.data


def _ptr_mem(a, dtype, shape):
    """(address, GCVT_MEM_*) of a numpy array or a torch tensor (CUDA tensors
    are device memory, CPU tensors -- e.g. pinned ones -- host memory)."""
    if hasattr(a, "data_ptr"):
        return a.data_ptr(), (MEM_DEVICE if getattr(a, "is_cuda", False) else MEM_HOST)
    return _host_ptr(a, dtype, shape), MEM_HOST


class Context:
    """A device context for grids up to n_max (gcvt_ctx_*)."""

    def __init__(self, n_max):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _check(self.lib.gcvt_ctx_create(int(n_max), ctypes.byref(h)), "gcvt_ctx_create")
        self.h = h
        self.n_max = int(n_max)
        self.n = None

    def close(self):
        if self.h:
            self.lib.gcvt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_handle):
        _check(self.lib.gcvt_ctx_set_stream(self.h, stream_handle), "gcvt_ctx_set_stream")

    def load(self, sites, density, mask=None):
        if hasattr(sites, "data_ptr"):
            n = int(sites.shape[0])
            mp = mask.data_ptr() if mask is not None else None
            mem = MEM_DEVICE if getattr(sites, "is_cuda", False) else MEM_HOST
            _check(self.lib.gcvt_ctx_load(self.h, n, sites.data_ptr(), density.data_ptr(), mp,
                                          mem), "gcvt_ctx_load")
        else:
            n = int(sites.shape[0])
            sp = _host_ptr(sites, np.int16, (n, n, 2))
            dp = _host_ptr(density, np.float32, (n, n))
            mp = _host_ptr(mask, np.uint8, (n, n)) if mask is not None else None
            _check(self.lib.gcvt_ctx_load(self.h, n, sp, dp, mp, MEM_HOST), "gcvt_ctx_load")
        self.n = n

    def label(self, out=None):
        n = self.n
        if out is None:
            out = np.empty((n, n, 2), np.int16)
        p, mem = _ptr_mem(out, np.int16, (n, n, 2))
        _check(self.lib.gcvt_ctx_label(self.h, p, mem), "gcvt_ctx_label")
        return out

    def iterate(self, iterations):
        _check(self.lib.gcvt_ctx_iterate(self.h, int(iterations)), "gcvt_ctx_iterate")

    def run(self, depth=1, max_iter=1000):
        info = RunInfo()
        _check(self.lib.gcvt_ctx_run(self.h, int(depth), int(max_iter), ctypes.byref(info)),
               "gcvt_ctx_run")
        return info.as_dict()

    def sites(self, out=None):
        n = self.n
        if out is None:
            out = np.empty((n, n, 2), np.int16)
        p, mem = _ptr_mem(out, np.int16, (n, n, 2))
        _check(self.lib.gcvt_ctx_sites(self.h, p, mem), "gcvt_ctx_sites")
        return out

    def moments(self):
        """(W, X, Y, E) planes of shape (n, n) at the current site pixels."""
        n = self.n
        out = np.empty((4, n, n), np.float64)
        _check(self.lib.gcvt_ctx_moments(self.h, out.ctypes.data, MEM_HOST), "gcvt_ctx_moments")
        return out

    def time_kernels(self, iterations):
        """Mean device ms of (one Lloyd iteration, one exact labelling pass,
        one jump-flooding labelling) over `iterations` repetitions; the sites
        move as in iterate()."""
        ms = (ctypes.c_float * 3)()
        _check(self.lib.gcvt_ctx_time_kernels(self.h, int(iterations), ms), "gcvt_ctx_time_kernels")
        return list(ms)

    def extract_points(self, scale=1.0, left=0.0, lower=0.0, capacity=None):
        """CDT input points (count, 2) float64 of the current free sites, in
        delaunayInput's order (delaunay.h:46-57)."""
        cnt = I(0)
        if capacity is None:
            _check(self.lib.gcvt_ctx_extract_points(self.h, float(scale), float(left),
                                                    float(lower), None, 0, ctypes.byref(cnt),
                                                    MEM_HOST), "gcvt_ctx_extract_points")
            capacity = cnt.value
        out = np.empty((max(capacity, 1), 2), np.float64)
        _check(self.lib.gcvt_ctx_extract_points(self.h, float(scale), float(left), float(lower),
                                                out.ctypes.data, int(capacity), ctypes.byref(cnt),
                                                MEM_HOST), "gcvt_ctx_extract_points")
        return out[:min(cnt.value, capacity)]

    def delaunay(self, capacity=None):
        """Delaunay triangles (T, 3) int32 of the current free sites, as
        indices into extract_points' list, counter-clockwise."""
        cnt = I(0)
        if capacity is None:  # a triangulation of V points has at most 2V - 5 triangles
            _check(self.lib.gcvt_ctx_extract_points(self.h, 1.0, 0.0, 0.0, None, 0,
                                                    ctypes.byref(cnt), MEM_HOST),
                   "gcvt_ctx_extract_points")
            capacity = max(2 * cnt.value - 5, 0)
        out = np.empty((max(capacity, 1), 3), np.int32)
        _check(self.lib.gcvt_ctx_delaunay(self.h, out.ctypes.data, int(capacity),
                                          ctypes.byref(cnt), MEM_HOST), "gcvt_ctx_delaunay")
        return out[:min(cnt.value, capacity)]

    def cdt(self, scale, left, lower, cpoints, segments, capacity=None):
        """Constrained Delaunay triangles (T, 3) int32 of the current free
        sites (extract_points' order) and the constraint points cpoints
        (C, 2) float64 (indices after the sites), with the segments (S, 2)
        index pairs as edges; returns (triangles, detail mask)."""
        c = np.ascontiguousarray(cpoints, np.float64).reshape(-1, 2)
        sg = np.ascontiguousarray(segments, np.int32).reshape(-1, 2)
        cnt, det = I(0), I(0)
        if capacity is None:
            _check(self.lib.gcvt_ctx_extract_points(self.h, 1.0, 0.0, 0.0, None, 0,
                                                    ctypes.byref(cnt), MEM_HOST),
                   "gcvt_ctx_extract_points")
            capacity = 2 * (cnt.value + len(c)) + 16
        out = np.empty((max(capacity, 1), 3), np.int32)
        code = self.lib.gcvt_ctx_cdt(self.h, float(scale), float(left), float(lower),
                                     c.ctypes.data, len(c), sg.ctypes.data, len(sg),
                                     out.ctypes.data, int(capacity), ctypes.byref(cnt),
                                     ctypes.byref(det), MEM_HOST)
        if code:
            raise GcvtError(code, "gcvt_ctx_cdt (detail %d)" % det.value)
        return out[:min(cnt.value, capacity)], det.value

    def autotune(self):
        """Pick the fastest launch choices for the loaded problem (results
        unchanged); returns them as a dict."""
        t = Tuning()
        _check(self.lib.gcvt_ctx_autotune(self.h, ctypes.byref(t)), "gcvt_ctx_autotune")
        return t.as_dict()

    def set_tuning(self, cell_blocks_per_sm=0, hint_slack=2, jfa_tail_halo=0, cell_mode=0):
        t = Tuning(int(cell_blocks_per_sm), int(hint_slack), int(jfa_tail_halo), 0.0, 0.0,
                   int(cell_mode))
        _check(self.lib.gcvt_ctx_set_tuning(self.h, ctypes.byref(t)), "gcvt_ctx_set_tuning")

    def learning(self, enable=True, track_ids=False):
        _check(self.lib.gcvt_ctx_learning(self.h, int(bool(enable)), int(bool(track_ids))),
               "gcvt_ctx_learning")

    def set_mlp(self, params):
        p = np.ascontiguousarray(params, np.float32)
        _check(self.lib.gcvt_ctx_set_mlp(self.h, p.ctypes.data, int(p.size)), "gcvt_ctx_set_mlp")

    def features(self, with_ids=False):
        """(features (m, 10), ids (m,) or None, xy (m, 2)) of the current sites."""
        cnt = I(0)
        _check(self.lib.gcvt_ctx_features(self.h, None, None, None, 0, ctypes.byref(cnt)),
               "gcvt_ctx_features")
        m = cnt.value
        f = np.empty((max(m, 1), 10), np.float32)
        ids = np.empty(max(m, 1), np.int32) if with_ids else None
        xy = np.empty((max(m, 1), 2), np.int32)
        _check(self.lib.gcvt_ctx_features(self.h, f.ctypes.data,
                                          None if ids is None else ids.ctypes.data,
                                          xy.ctypes.data, m, ctypes.byref(cnt)),
               "gcvt_ctx_features")
        return f[:m], (None if ids is None else ids[:m]), xy[:m]

    def iterate_learned(self, iterations, jump_every=10):
        """Lloyd iterations with a learned step every jump_every; returns
        (jumps tried, jumps kept)."""
        tried, kept = I(0), I(0)
        _check(self.lib.gcvt_ctx_iterate_learned(self.h, int(iterations), int(jump_every),
                                                 ctypes.byref(tried), ctypes.byref(kept)),
               "gcvt_ctx_iterate_learned")
        return tried.value, kept.value

    def set_target_energy(self, target):
        """Later runs also stop at the first iteration with energy <= target
        (0: off)."""
        _check(self.lib.gcvt_ctx_set_target_energy(self.h, float(target)),
               "gcvt_ctx_set_target_energy")

    def jfa_label(self, labels=True):
        """(labels or None, (differing, farther, pixels)) of jump flooding."""
        n = self.n
        out = np.empty((n, n, 2), np.int16) if labels else None
        st = (ctypes.c_ulonglong * 3)()
        _check(self.lib.gcvt_ctx_jfa_label(self.h, None if out is None else out.ctypes.data, st,
                                           MEM_HOST), "gcvt_ctx_jfa_label")
        return out, tuple(int(v) for v in st)

    def info(self):
        info = RunInfo()
        _check(self.lib.gcvt_ctx_info(self.h, ctypes.byref(info)), "gcvt_ctx_info")
        return info.as_dict()


def gcvt(voronoi, density, mask, depth=1, max_iter=1000):
    """gCVT: runs the Lloyd loop from the site grid ``voronoi`` and overwrites
    it with the final label grid (gcvt.cu:1087-1156)."""
    lib = load_library()
    n = int(voronoi.shape[0])
    _check(lib.gcvt_compute(_host_ptr(voronoi, np.int16, (n, n, 2)),
                            _host_ptr(density, np.float32, (n, n)),
                            _host_ptr(mask, np.uint8, (n, n)), n, int(depth), int(max_iter)),
           "gcvt_compute")
    return voronoi


class Batch:
    """Several loaded Contexts iterated together (gcvt_batch_*): one launch
    pair per iteration for all of them; results are read through the
    Contexts."""

    def __init__(self, contexts):
        self.lib = load_library()
        self.contexts = list(contexts)
        arr = (P * len(self.contexts))(*[c.h for c in self.contexts])
        self.h = P()
        _check(self.lib.gcvt_batch_create(len(self.contexts), arr, ctypes.byref(self.h)),
               "gcvt_batch_create")

    def set_stream(self, stream):
        _check(self.lib.gcvt_batch_set_stream(self.h, stream), "gcvt_batch_set_stream")

    def iterate(self, iterations):
        _check(self.lib.gcvt_batch_iterate(self.h, int(iterations)), "gcvt_batch_iterate")

    def run(self, max_iter=1000):
        infos = (RunInfo * len(self.contexts))()
        _check(self.lib.gcvt_batch_run(self.h, int(max_iter), infos), "gcvt_batch_run")
        return [i.as_dict() for i in infos]

    def set_mlp(self, params):
        p = np.ascontiguousarray(params, np.float32)
        _check(self.lib.gcvt_batch_set_mlp(self.h, p.ctypes.data, len(p)), "gcvt_batch_set_mlp")

    def iterate_learned(self, iterations, jump_every=4):
        """Every member's learned run at once; returns (jumps tried, kept)
        summed over the charts."""
        tried, kept = I(0), I(0)
        _check(self.lib.gcvt_batch_iterate_learned(self.h, int(iterations), int(jump_every),
                                                   ctypes.byref(tried), ctypes.byref(kept)),
               "gcvt_batch_iterate_learned")
        return tried.value, kept.value

    def close(self):
        if self.h:
            self.lib.gcvt_batch_destroy(self.h)
            self.h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp_param_count():
    return int(load_library().gcvt_mlp_param_count())


def mlp_init(seed=0):
    """He-initialised FP32 parameters of the step MLP."""
    rng = np.random.default_rng(seed)
    p = np.zeros(mlp_param_count(), np.float32)
    o = 0
    for fan_in, fan_out in ((10, 64), (64, 64), (64, 2)):
        p[o:o + fan_in * fan_out] = rng.normal(0, np.sqrt(2.0 / fan_in), fan_in * fan_out)
        o += fan_in * fan_out + fan_out
    return p


def mlp_forward(params, feat, tensor_cores=True):
    lib = load_library()
    f = np.ascontiguousarray(feat, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    out = np.empty((len(f), 2), np.float32)
    _check(lib.gcvt_mlp_forward(p.ctypes.data, f.ctypes.data, len(f), out.ctypes.data,
                                int(bool(tensor_cores))), "gcvt_mlp_forward")
    return out


def mlp_train(samples, params, steps=2000, batch=4096, lr=1e-3, seed=0):
    """Train on samples (m, 12) float32; returns (params, per-step losses)."""
    lib = load_library()
    s = np.ascontiguousarray(samples, np.float32)
    p = np.array(params, np.float32, copy=True)
    loss = np.empty(steps, np.float32)
    _check(lib.gcvt_mlp_train(s.ctypes.data, len(s), p.ctypes.data, int(steps), int(batch),
                              float(lr), int(seed), loss.ctypes.data), "gcvt_mlp_train")
    return p, loss


def mlp_gradient(samples, params, batch, seed=0, step=0):
    """Gradient (FP32, gcvt_mlp_param_count()) and mean loss of the batch the
    trainer draws at `step` with `seed`, at the FP32 parameters `params`."""
    lib = load_library()
    s = np.ascontiguousarray(samples, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    g = np.empty(mlp_param_count(), np.float32)
    loss = np.empty(1, np.float32)
    _check(lib.gcvt_mlp_gradient(s.ctypes.data, len(s), p.ctypes.data, int(batch), int(seed),
                                 int(step), g.ctypes.data, loss.ctypes.data), "gcvt_mlp_gradient")
    return g, float(loss[0])


def seed_sites(density, mask, num, state=None):
    """Initial site grid (n, n, 2) int16 as centroidalVoronoi makes it
    (gcvt.h:76-122).  state: None for the library's own generator, or a
    numpy uint64 array of 4 words (z, w, jsr, jcong), updated in place."""
    lib = load_library()
    n = int(density.shape[0])
    v = np.empty((n, n, 2), np.int16)
    sp = None
    if state is not None:
        if not (isinstance(state, np.ndarray) and state.dtype == np.uint64 and state.size == 4):
            raise TypeError("state must be a numpy uint64 array of 4 words")
        sp = state.ctypes.data
    mp = None if mask is None else _host_ptr(mask, np.uint8, (n, n))
    _check(lib.gcvt_seed_sites(v.ctypes.data, _host_ptr(density, np.float32, (n, n)), mp,
                               int(num), n, sp), "gcvt_seed_sites")
    return v


def centroidal_voronoi(density, mask, vertices, depth=1, max_iter=1000):
    """centroidalVoronoi (gcvt.h:124-139): seed, then gCVT; returns the label grid."""
    lib = load_library()
    n = int(density.shape[0])
    v = np.empty((n, n, 2), np.int16)
    _check(lib.gcvt_centroidal_voronoi(v.ctypes.data, _host_ptr(density, np.float32, (n, n)),
                                       _host_ptr(mask, np.uint8, (n, n)), int(vertices), n,
                                       int(depth), int(max_iter)), "gcvt_centroidal_voronoi")
    return v


def label_grid(sites):
    """Labels of a site grid (one exact pass, bit-identical to pba2DCompute)."""
    lib = load_library()
    n = int(sites.shape[0])
    if hasattr(sites, "data_ptr"):
        import torch  # device path: output on the same device
        out = torch.empty_like(sites)
        _check(lib.gcvt_label_grid(sites.data_ptr(), out.data_ptr(), n, MEM_DEVICE),
               "gcvt_label_grid")
        return out
    out = np.empty_like(sites)
    _check(lib.gcvt_label_grid(_host_ptr(sites, np.int16, (n, n, 2)), out.ctypes.data, n,
                               MEM_HOST), "gcvt_label_grid")
    return out


def rasterize(points, weight, triangles, scale, n):
    """Density grid (n, n) float32 of a mesh: points (V, 2) float64, weight (V,)
    float64, triangles (T, 3) int32 (discretization_d's arguments)."""
    lib = load_library()
    out = np.empty((n, n), np.float32)
    _check(lib.gcvt_rasterize(_host_ptr(points, np.float64), _host_ptr(weight, np.float64),
                              len(weight), _host_ptr(triangles, np.int32), len(triangles),
                              out.ctypes.data, float(scale), int(n), MEM_HOST), "gcvt_rasterize")
    return out


def lift(uv, xyz, triangles, points, fixed=None, cdt=None):
    """recover() (recover.h:98-157) on the GPU.  uv (V, 2) and xyz (V, 3)
    float64 per mesh vertex, triangles (T, 3) int32, points (P, 2) float64 --
    the free points, then len(fixed) constraint points whose mesh vertices
    are `fixed` -- and cdt (C, 3) int32 triangles over the points.  Returns
    (lifted xyz (P, 3) float64, face (P,) int32, keep (C,) bool)."""
    lib = load_library()
    uv = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    tri = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    pts = np.ascontiguousarray(points, np.float64).reshape(-1, 2)
    fixed = np.ascontiguousarray(np.zeros(0) if fixed is None else fixed, np.int32).ravel()
    cdt = np.ascontiguousarray(np.zeros((0, 3)) if cdt is None else cdt, np.int32).reshape(-1, 3)
    out = np.empty((len(pts), 3), np.float64)
    face = np.empty(len(pts), np.int32)
    keep = np.empty(len(cdt), np.uint8)
    _check(lib.gcvt_lift(uv.ctypes.data, xyz.ctypes.data, len(uv), tri.ctypes.data, len(tri),
                         pts.ctypes.data, len(pts), len(fixed), fixed.ctypes.data,
                         cdt.ctypes.data, len(cdt), out.ctypes.data, face.ctypes.data,
                         keep.ctypes.data, MEM_HOST), "gcvt_lift")
    return out, face, keep.astype(bool)


def vertex_weights(uv, xyz, triangles):
    """weighting_vertices_with_area (weighting.h:38-97) on the GPU: (V,)
    float64 area-ratio weights."""
    lib = load_library()
    uv = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    tri = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    w = np.empty(len(uv), np.float64)
    _check(lib.gcvt_vertex_weights(uv.ctypes.data, xyz.ctypes.data, len(uv), tri.ctypes.data,
                                   len(tri), w.ctypes.data, MEM_HOST), "gcvt_vertex_weights")
    return w


def sites_from_points(n, xs, ys):
    """Site grid with a site at each (x, y)."""
    g = np.full((n, n, 2), MARKER, np.int16)
    g[ys, xs, 0] = xs
    g[ys, xs, 1] = ys
    return g
