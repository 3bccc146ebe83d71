"""gcurval_gb300: adaptive arc length and arc-length sampling of parametric
curves on one GB300 GPU.

Python mirror of the reference's driver class
``gcurval::ArclengthCalculateGpu`` (gcurval/arclength_calculate.h:10-18,
gcurval/detail/cuda/arclength_calculate.h:93-507) over the C ABI in
include/gcurval_gb300.h.  Method names, argument meaning and the
where / what enums follow the reference:

    calc = ArclengthCalculateGpu.ellipses(a, b)          # ellipse.h:121-129
    calc.createArclengthTable()                          # :185
    lengths = calc.getAllCurveArclengths()               # :212
    L0 = calc.getArclength(0)                            # :218
    res = calc.arclengthReverse(n_per_curve, positions, True,
                                GCV_HOST, GCV_RETURN_US) # :224
    calc.clearArclength()                                # :233

All compute runs in libgcurval_gb300.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import (GCV_DEVICE, GCV_HOST, GCV_MAP_HALF_WARP, GCV_MAP_LANE, GCV_MIXED, GCV_PLAIN_FP64,
                   GCV_RETURN_POINTS, GCV_RETURN_US,
                   GcvError, Options, Result, ResultF32, Stats, check, default_options, load, pinned_copy,
                   pinned_empty, release_cached_memory)

__all__ = ["ArclengthCalculateGpu", "ArclengthReverseResult", "GcvError", "GCV_DEVICE", "GCV_HOST",
           "GCV_RETURN_US", "GCV_RETURN_POINTS", "GCV_PLAIN_FP64", "GCV_MIXED", "GCV_MAP_LANE", "GCV_MAP_HALF_WARP",
           "default_options", "load", "pinned_copy", "pinned_empty",
           "release_cached_memory"]

_P = ctypes.c_void_p


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):  # torch tensor
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(_P)


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _is_f32(a) -> bool:
    """A float32 numpy array or torch tensor."""
    dt = getattr(a, "dtype", None)
    return dt is not None and str(dt) in ("float32", "torch.float32")


_cudart_lib = None


def _cudart():
    """The CUDA runtime's shared library (for reading device results back)."""
    global _cudart_lib
    if _cudart_lib is None:
        import glob
        import os
        cands = []
        for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
            if d:
                cands += sorted(glob.glob(os.path.join(d, "lib64", "libcudart.so*")))
                cands += sorted(glob.glob(os.path.join(d, "targets", "*", "lib", "libcudart.so*")))
        for c in cands + ["libcudart.so"]:
            try:
                _cudart_lib = ctypes.CDLL(c)
                break
            except OSError:
                continue
        if _cudart_lib is None:
            raise GcvError(2, "libcudart.so not found")
        _cudart_lib.cudaMemcpy.restype = ctypes.c_int
        _cudart_lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return _cudart_lib


class ArclengthReverseResult:
    """Result of arclengthReverse (gcurval/base/structs.inl.h:66-77): n_points
    parameters ``us`` or ``points`` (n_points x dim), in host memory (numpy)
    or device memory (owned by this object, freed with it)."""

    def __init__(self, res, lib, dtype=np.float64):
        self._res = res
        self._lib = lib
        self.dtype = np.dtype(dtype)
        self.n_points = int(res.n_points)
        self.store_where = int(res.store_where)
        self.store_what = int(res.store_what)
        self.point_dim = int(res.point_dim)

    @property
    def device_ptr(self) -> int:
        return int(self._res.data or 0)

    def numpy(self) -> np.ndarray:
        width = 1 if self.store_what == GCV_RETURN_US else self.point_dim
        n = self.n_points * width
        out = np.empty(n, self.dtype)
        nb = n * self.dtype.itemsize
        if n:
            if self.store_where == GCV_HOST:
                ctypes.memmove(out.ctypes.data, self._res.data, nb)
            else:
                rc = _cudart().cudaMemcpy(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(self._res.data),
                                          ctypes.c_size_t(nb), 2)  # cudaMemcpyDeviceToHost
                if rc != 0:
                    raise GcvError(2, f"cudaMemcpy of the device result failed ({rc})")
        return out if width == 1 else out.reshape(-1, width)

    @property
    def us(self) -> np.ndarray:
        return self.numpy()

    @property
    def points(self) -> np.ndarray:
        return self.numpy()

    def free(self):
        if self._res is not None and self._res.data:
            if self.dtype == np.float32:
                self._lib.gcv_free_result_f32(ctypes.byref(self._res))
            else:
                self._lib.gcv_free_result(ctypes.byref(self._res))
        self._res = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ArclengthCalculateGpu:
    """One batch of curves on the GPU (a gcv_ctx)."""

    def __init__(self, handle, keep=(), f32=False):
        self._lib = load()
        self._h = handle
        self._keep = keep  # host/device arrays the context borrows
        # FP32 data (the reference's ArclengthCalculateGpu<float>): float
        # lengths, positions, parameters and points
        self.f32 = bool(f32)
        self.dtype = np.float32 if f32 else np.float64
        n = ctypes.c_int64()
        s = ctypes.c_int64()
        d = ctypes.c_int()
        check(self._lib.gcv_get_shape(self._h, ctypes.byref(n), ctypes.byref(s), ctypes.byref(d)))
        self.n_curve = int(n.value)
        self.n_segments = int(s.value)
        self.point_dim = int(d.value)

    # ---------------------------------------------------------------- makers
    @staticmethod
    def _opts(precision=GCV_PLAIN_FP64, rtol=None, max_depth=None, stream=None, collect_stats=False,
              learned=False, mapping=None, host_in_place=False) -> Options:
        o = default_options(precision)
        o.learned = int(bool(learned))
        o.host_in_place = int(bool(host_in_place))
        if mapping is not None:
            o.mapping = {"lane": GCV_MAP_LANE, "half_warp": GCV_MAP_HALF_WARP}.get(mapping, mapping)
        if rtol is not None:
            o.rtol = float(rtol)
        if max_depth is not None:
            o.max_depth = int(max_depth)
        if stream is not None:
            o.stream = ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))
        o.collect_stats = int(bool(collect_stats))
        return o

    @classmethod
    def ellipses(cls, a, b, rot=None, cx=None, cy=None, **kw):
        """samples/sample1_ellipse/ellipse.h:121-129 (plus rotation and centre).
        float32 arrays select the FP32 entry points (Dt = float)."""
        lib = load()
        f32 = _is_f32(a)
        dt = np.float32 if f32 else np.float64
        arrs = [None if x is None else (x if _is_device(x) else np.ascontiguousarray(x, dt))
                for x in (a, b, rot, cx, cy)]
        where = GCV_DEVICE if _is_device(arrs[0]) else GCV_HOST
        h = _P()
        o = cls._opts(**kw)
        create = lib.gcv_create_ellipses_f32 if f32 else lib.gcv_create_ellipses
        check(create(ctypes.byref(h), len(arrs[0]), *[_ptr(x) for x in arrs], where, ctypes.byref(o)))
        return cls(h, keep=tuple(arrs), f32=f32)

    @classmethod
    def bsplines(cls, degree, dim, knots_offset, knot_vector, ctrl_pts, **kw):
        """samples/sample2_bspline/arclength_calculate.h:505-518 layout.
        float32 knots and control points select the FP32 entry points."""
        lib = load()
        dev = _is_device(knot_vector)
        f32 = _is_f32(knot_vector)
        dt = np.float32 if f32 else np.float64
        ko = knots_offset if dev else np.ascontiguousarray(knots_offset, np.int32)
        kv = knot_vector if dev else np.ascontiguousarray(knot_vector, dt)
        cp = ctrl_pts if dev else np.ascontiguousarray(ctrl_pts, dt)
        h = _P()
        o = cls._opts(**kw)
        create = lib.gcv_create_bsplines_f32 if f32 else lib.gcv_create_bsplines
        check(create(ctypes.byref(h), len(ko) - 1, int(degree), int(dim), _ptr(ko), _ptr(kv), _ptr(cp),
                     GCV_DEVICE if dev else GCV_HOST, ctypes.byref(o)))
        return cls(h, keep=(ko, kv, cp), f32=f32)

    @classmethod
    def from_batch(cls, batch, **kw):
        """Any CurveBatch (gcurval_gb300.datasets) through gcv_create_batch.
        host_in_place=True: page-locked knot and control arrays (pinned_copy)
        are read in place by every table build instead of being copied; the
        context keeps references to them."""
        lib = load()
        arrs = (np.ascontiguousarray(batch.kind, np.uint8), np.ascontiguousarray(batch.degree, np.uint8),
                np.ascontiguousarray(batch.dim, np.uint8), np.ascontiguousarray(batch.knot_off, np.int64),
                np.ascontiguousarray(batch.knots, np.float64), np.ascontiguousarray(batch.ctrl_off, np.int64),
                np.ascontiguousarray(batch.ctrl, np.float64))
        h = _P()
        o = cls._opts(**kw)
        check(lib.gcv_create_batch(ctypes.byref(h), batch.n_curve, *[_ptr(x) for x in arrs], GCV_HOST, ctypes.byref(o)))
        return cls(h, keep=arrs if o.host_in_place else ())

    @classmethod
    def from_device_batch(cls, kind, degree, dim, knot_off, knots, ctrl_off, ctrl, **kw):
        """A batch whose arrays already live on the GPU (torch CUDA tensors of
        dtypes uint8, uint8, uint8, int64, float64, int64, float64); the
        context borrows them, so they must outlive it."""
        lib = load()
        arrs = (kind, degree, dim, knot_off, knots, ctrl_off, ctrl)
        for a in arrs:
            if not _is_device(a):
                raise ValueError("from_device_batch takes CUDA tensors")
        h = _P()
        o = cls._opts(**kw)
        check(lib.gcv_create_batch(ctypes.byref(h), int(kind.shape[0]), *[_ptr(x) for x in arrs], GCV_DEVICE,
                                   ctypes.byref(o)))
        return cls(h, keep=arrs)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gcv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------ reference API
    def set_options(self, precision=GCV_PLAIN_FP64, rtol=None, max_depth=None, stream=None, collect_stats=False,
                    learned=False, mapping=None):
        o = self._opts(precision, rtol, max_depth, stream, collect_stats, learned, mapping)
        check(self._lib.gcv_set_options(self._h, ctypes.byref(o)))

    def createArclengthTable(self):
        check(self._lib.gcv_create_arclength_table(self._h))

    def getAllCurveArclengths(self, out=None) -> np.ndarray:
        get = self._lib.gcv_get_all_curve_arclengths_f32 if self.f32 else self._lib.gcv_get_all_curve_arclengths
        if out is not None and _is_device(out):
            check(get(self._h, _ptr(out), GCV_DEVICE))
            return out
        res = np.empty(self.n_curve, self.dtype)
        check(get(self._h, _ptr(res), GCV_HOST))
        return res

    def getArclength(self, cid: int) -> float:
        if self.f32:
            v = ctypes.c_float()
            check(self._lib.gcv_get_arclength_f32(self._h, int(cid), ctypes.byref(v)))
            return np.float32(v.value)
        v = ctypes.c_double()
        check(self._lib.gcv_get_arclength(self._h, int(cid), ctypes.byref(v)))
        return v.value

    def arclengthReverse(self, n_ptrs_for_curves, sample_position, is_relative=True, where=GCV_DEVICE,
                         what=GCV_RETURN_US) -> ArclengthReverseResult:
        n = np.ascontiguousarray(n_ptrs_for_curves, np.int32)
        pos = np.ascontiguousarray(sample_position, self.dtype)
        self._check_counts(n, pos.shape[0])
        r = ResultF32() if self.f32 else Result()
        rev = self._lib.gcv_arclength_reverse_f32 if self.f32 else self._lib.gcv_arclength_reverse
        check(rev(self._h, _ptr(n), _ptr(pos), int(bool(is_relative)), int(where), int(what), ctypes.byref(r)))
        return ArclengthReverseResult(r, self._lib, self.dtype)

    def arclengthReverseInto(self, n_ptrs_for_curves, sample_position, out, is_relative=True, what=GCV_RETURN_US):
        """Sampling into a caller buffer (numpy or torch, host or device)."""
        in_dev = _is_device(sample_position)
        n = n_ptrs_for_curves if _is_device(n_ptrs_for_curves) else np.ascontiguousarray(n_ptrs_for_curves, np.int32)
        if _is_device(n) != in_dev:
            raise ValueError("counts and positions must live in the same memory")
        pos = sample_position if in_dev else np.ascontiguousarray(sample_position, self.dtype)
        if _is_f32(pos) != self.f32 or _is_f32(out) != self.f32:
            raise ValueError(f"positions and output must be {np.dtype(self.dtype).name} for this context")
        total = self._check_counts(n, int(pos.shape[0]))
        width = 1 if what == GCV_RETURN_US else self.point_dim
        n_out = int(out.numel()) if hasattr(out, "numel") else int(out.size)
        if n_out < total * width:
            raise ValueError(f"output holds {n_out} values, {total * width} needed")
        into = self._lib.gcv_arclength_reverse_into_f32 if self.f32 else self._lib.gcv_arclength_reverse_into
        check(into(self._h, _ptr(n), _ptr(pos), int(bool(is_relative)), GCV_DEVICE if in_dev else GCV_HOST,
                   int(what), _ptr(out), GCV_DEVICE if _is_device(out) else GCV_HOST))
        return out

    def clearArclength(self):
        check(self._lib.gcv_clear_arclength(self._h))

    def _check_counts(self, n, n_positions: int) -> int:
        """The C ABI reads n_curve counts and their sum of positions through raw
        pointers, as the reference does; check the sizes before handing them over."""
        if tuple(n.shape) != (self.n_curve,):
            raise ValueError(f"{n.shape[0] if len(n.shape) else 0} sample counts for {self.n_curve} curves")
        total = int(n.sum())
        if total != n_positions:
            raise ValueError(f"sample counts add up to {total}, {n_positions} positions given")
        return total

    # ------------------------------------------------------------ graph
    def stepGraph(self, n_ptrs_for_curves, sample_position, out, is_relative=True, what=GCV_RETURN_US):
        """createArclengthTable + arclengthReverseInto on CUDA tensors as one
        captured CUDA graph (gcv_step_graph): captured on the first call,
        replayed on later calls with the same tensors."""
        for a in (n_ptrs_for_curves, sample_position, out):
            if not _is_device(a):
                raise ValueError("stepGraph takes CUDA tensors")
        total = self._check_counts(n_ptrs_for_curves, int(sample_position.shape[0]))
        width = 1 if what == GCV_RETURN_US else self.point_dim
        if int(out.numel()) < total * width:
            raise ValueError(f"output holds {int(out.numel())} values, {total * width} needed")
        check(self._lib.gcv_step_graph(self._h, _ptr(n_ptrs_for_curves), _ptr(sample_position), int(bool(is_relative)),
                                       int(what), _ptr(out)))
        return out

    def resetGraph(self):
        check(self._lib.gcv_step_graph_reset(self._h))

    # ------------------------------------------------------- learned form
    def set_learned_model(self, weights):
        """Installs the learned form's network (packed FP32 weights, see
        gcurval_gb300.learned); None removes it.  Takes effect for contexts
        created with learned=True."""
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        if w is not None and w.size != self._lib.gcv_mlp_param_count():
            raise ValueError(f"{w.size} weights, {self._lib.gcv_mlp_param_count()} expected")
        check(self._lib.gcv_set_learned_model(self._h, _ptr(w)))

    def learned_features(self, out):
        """The 16 features of every knot interval into `out` (CUDA float32, n_segments x 16)."""
        check(self._lib.gcv_learned_features(self._h, _ptr(out)))
        return out

    def learned_labels(self, depth, share, tguess):
        """Labels from the current (plain) table into CUDA tensors: depth
        (int32, n_segments), share (float32, n_segments x 4), tguess (float32,
        n_segments x 8)."""
        check(self._lib.gcv_learned_labels(self._h, _ptr(depth), _ptr(share), _ptr(tguess)))

    # ------------------------------------------------------------- extras
    def synchronize(self):
        check(self._lib.gcv_synchronize(self._h))

    def stats(self) -> dict:
        s = Stats()
        check(self._lib.gcv_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()
