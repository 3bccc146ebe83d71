"""ctypes binding of libgcurval_gb300.so (include/gcurval_gb300.h).

The library is the only compute path: if it is missing or a GPU is absent the
calls fail with GcvError; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgcurval_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "gcurval_gb300.h")

GCV_OK = 0
GCV_ERR_INVALID = 1
GCV_ERR_CUDA = 2
GCV_ERR_OUT_OF_MEMORY = 3
GCV_ERR_STATE = 4
GCV_ERR_OVERFLOW = 5
GCV_ERR_TIMEOUT = 6
GCV_ERR_NO_DEVICE = 7

GCV_DEVICE = 0
GCV_HOST = 1
GCV_RETURN_US = 2
GCV_RETURN_POINTS = 3

GCV_PLAIN_FP64 = 0
GCV_MIXED = 1
# gcv_mapping: the float-float length walk's threads per knot interval
GCV_MAP_LANE = 0
GCV_MAP_HALF_WARP = 1

STATUS_NAMES = {0: "GCV_OK", 1: "GCV_ERR_INVALID", 2: "GCV_ERR_CUDA", 3: "GCV_ERR_OUT_OF_MEMORY",
                4: "GCV_ERR_STATE", 5: "GCV_ERR_OVERFLOW", 6: "GCV_ERR_TIMEOUT", 7: "GCV_ERR_NO_DEVICE"}

_P = ctypes.c_void_p


class GcvError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Options(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("max_depth", ctypes.c_int), ("precision", ctypes.c_int),
                ("stream", _P), ("collect_stats", ctypes.c_int), ("learned", ctypes.c_int),
                ("mapping", ctypes.c_int), ("host_in_place", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int64), ("store_where", ctypes.c_int), ("store_what", ctypes.c_int),
                ("point_dim", ctypes.c_int), ("data", _P)]


class ResultF32(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int64), ("store_where", ctypes.c_int), ("store_what", ctypes.c_int),
                ("point_dim", ctypes.c_int), ("data", _P)]


class Stats(ctypes.Structure):
    _fields_ = [("n_curves", ctypes.c_int64), ("n_segments", ctypes.c_int64), ("n_leaves", ctypes.c_int64),
                ("n_panels", ctypes.c_int64), ("n_deep_segments", ctypes.c_int64), ("n_capped", ctypes.c_int64),
                ("n_samples", ctypes.c_int64), ("n_newton", ctypes.c_int64), ("ms_setup", ctypes.c_double),
                ("ms_length", ctypes.c_double), ("ms_scan", ctypes.c_double), ("ms_sample", ctypes.c_double),
                ("n_launches", ctypes.c_int64), ("ms_learned", ctypes.c_double),
                ("length_blocks_per_sm", ctypes.c_int), ("sample_threads", ctypes.c_int),
                ("sample_blocks_per_sm", ctypes.c_int), ("tuned", ctypes.c_int),
                ("length_blocks_per_sm_code", ctypes.c_int * 11)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["length_blocks_per_sm_code"] = list(d["length_blocks_per_sm_code"])
        return d


_SIGS = {
    "gcv_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "gcv_last_error": (ctypes.c_char_p, []),
    "gcv_version": (ctypes.c_int, []),
    "gcv_default_options": (ctypes.c_int, [ctypes.POINTER(Options), ctypes.c_int]),
    "gcv_create_ellipses": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_int,
                                           ctypes.POINTER(Options)]),
    "gcv_create_bsplines": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                           ctypes.c_int, ctypes.POINTER(Options)]),
    "gcv_create_batch": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, ctypes.c_int,
                                        ctypes.POINTER(Options)]),
    "gcv_destroy": (ctypes.c_int, [_P]),
    "gcv_set_options": (ctypes.c_int, [_P, ctypes.POINTER(Options)]),
    "gcv_create_arclength_table": (ctypes.c_int, [_P]),
    "gcv_get_all_curve_arclengths": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "gcv_get_arclength": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "gcv_arclength_reverse": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(Result)]),
    "gcv_arclength_reverse_into": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P,
                                                  ctypes.c_int]),
    "gcv_free_result": (ctypes.c_int, [ctypes.POINTER(Result)]),
    "gcv_clear_arclength": (ctypes.c_int, [_P]),
    "gcv_synchronize": (ctypes.c_int, [_P]),
    "gcv_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "gcv_get_shape": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_int)]),
    "gcv_measure_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "gcv_release_cached_memory": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    "gcv_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_P)]),
    "gcv_host_free": (ctypes.c_int, [_P]),
    "gcv_step_graph": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, _P]),
    "gcv_step_graph_reset": (ctypes.c_int, [_P]),
    # FP32 data
    "gcv_create_ellipses_f32": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_int,
                                               ctypes.POINTER(Options)]),
    "gcv_create_bsplines_f32": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P,
                                               _P, ctypes.c_int, ctypes.POINTER(Options)]),
    "gcv_get_all_curve_arclengths_f32": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "gcv_get_arclength_f32": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "gcv_arclength_reverse_into_f32": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P,
                                                      ctypes.c_int]),
    "gcv_arclength_reverse_f32": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(ResultF32)]),
    "gcv_free_result_f32": (ctypes.c_int, [ctypes.POINTER(ResultF32)]),
    "gcv_bspline_lengths_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                                   ctypes.c_double, ctypes.c_int, _P, _P,
                                                   ctypes.POINTER(ctypes.c_int64)]),
    # learned form (include/gcurval_gb300_learned.h)
    "gcv_mlp_param_count": (ctypes.c_int, []),
    "gcv_mlp_last_error": (ctypes.c_char_p, []),
    "gcv_learned_features": (ctypes.c_int, [_P, _P]),
    "gcv_learned_labels": (ctypes.c_int, [_P, _P, _P, _P]),
    "gcv_mlp_trainer_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_ulonglong]),
    "gcv_mlp_trainer_destroy": (ctypes.c_int, [_P]),
    "gcv_mlp_trainer_set_weights": (ctypes.c_int, [_P, _P]),
    "gcv_mlp_trainer_get_weights": (ctypes.c_int, [_P, _P]),
    "gcv_mlp_trainer_forward": (ctypes.c_int, [_P, _P, ctypes.c_int, _P]),
    "gcv_mlp_trainer_gradients": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int, _P, _P]),
    "gcv_mlp_trainer_step": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_float, _P]),
    "gcv_mlp_infer": (ctypes.c_int, [_P, _P, ctypes.c_int, _P]),
    "gcv_set_learned_model": (ctypes.c_int, [_P, _P]),
    # Bundle reader (include/gcurval_gb300_bundle.h)
    "gcv_bundle_parse": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                        ctypes.c_int64, ctypes.c_int, ctypes.c_int, _P, ctypes.POINTER(_P)]),
    "gcv_bundle_sizes": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int64)]),
    "gcv_bundle_fill": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P]),
    "gcv_bundle_destroy": (None, [_P]),
}

LEARNED_HEADER = os.path.join(os.path.dirname(HEADER), "gcurval_gb300_learned.h")
BUNDLE_HEADER = os.path.join(os.path.dirname(HEADER), "gcurval_gb300_bundle.h")

_lib = None


def declared_symbols(header: str = HEADER):
    """Names of the functions a header of include/ declares (default gcurval_gb300.h)."""
    import re
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gcv_[a-z0-9_]+)\s*\(", txt)))


def load(path: str = LIB_PATH):
    """Loads the library (building it first when only the sources exist)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise GcvError(GCV_ERR_NO_DEVICE, f"{path} is missing; build it with python -m gcurval_gb300.build")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != GCV_OK:
        msg = _lib.gcv_last_error().decode() if _lib is not None else ""
        raise GcvError(status, msg)


def release_cached_memory() -> int:
    """Frees the device buffers destroyed contexts left in the library's
    memory cache; returns the bytes freed."""
    lib = load()
    n = ctypes.c_int64()
    check(lib.gcv_release_cached_memory(ctypes.byref(n)))
    return n.value


class _PinnedBlock:
    """Page-locked host memory from gcv_host_alloc, exposed to NumPy through
    the array interface; freed when the last array viewing it goes."""

    def __init__(self, n: int, dtype):
        self._lib = load()
        self.dtype = np.dtype(dtype)
        self.addr = _P()
        check(self._lib.gcv_host_alloc(ctypes.c_size_t(max(n, 1) * self.dtype.itemsize), ctypes.byref(self.addr)))
        self.__array_interface__ = {"data": (self.addr.value, False), "shape": (n,), "typestr": self.dtype.str,
                                    "version": 3}

    def __del__(self):
        if getattr(self, "addr", None) is not None and self.addr.value:
            self._lib.gcv_host_free(self.addr)
            self.addr = None


def pinned_empty(n: int, dtype=np.float64) -> np.ndarray:
    """A 1-D NumPy array of n elements in page-locked host memory: host inputs
    and outputs in such arrays are copied by the copy engines directly."""
    return np.asarray(_PinnedBlock(int(n), dtype))


def pinned_copy(a) -> np.ndarray:
    """A page-locked copy of a 1-D array."""
    a = np.ascontiguousarray(a)
    out = pinned_empty(a.shape[0], a.dtype)
    out[...] = a
    return out


def measure_fma_peak(which: int) -> float:
    """FMA throughput of the current GPU in TFLOP/s (0: FP64, 1: FP32)."""
    lib = load()
    v = ctypes.c_double()
    check(lib.gcv_measure_fma_peak(int(which), ctypes.byref(v)))
    return v.value


def default_options(precision: int = GCV_PLAIN_FP64) -> Options:
    lib = load()
    o = Options()
    check(lib.gcv_default_options(ctypes.byref(o), precision))
    return o
