"""ctypes front-end of the two CPU oracles (test infrastructure only).

* ``Oracle``     the plain-C restatement (``_build/libgcv_oracle.so``), built by
                 ``oracle/Makefile`` on any host, including the GPU host.
* ``Reference``  the reference's own CPU driver (``_ref/libgcv_ref.so``), built
                 only where the reference source tree exists.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module, as the checker.  The product path never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libgcv_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgcv_ref.so")
# The reference source tree, read only to compile its CPU driver; it exists
# on the development host only.  GCV_REFERENCE_TREE overrides the location.
REF_TREE = os.environ.get("GCV_REFERENCE_TREE") or "/root/reference"

# the reference's defaults for double: MAX_ERROR_DOUBLE (gcurval/config.h:32)
# and MaxRecursiveDepth<double> (gcurval/config.h:42)
REF_MAX_ERROR = 1e-14
REF_MAX_DEPTH = 23

_P = ctypes.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def build(ref: bool = True) -> None:
    """Compile the restatement (and the reference driver when its tree is present)."""
    targets = ["port"]
    if ref and os.path.exists(os.path.join(REF_TREE, "gcurval", "gcurval.h")):
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, f"REF={REF_TREE}"] + targets, check=True)


class _Batch(ctypes.Structure):
    _fields_ = [("n_curve", ctypes.c_int), ("kind", _P), ("degree", _P), ("dim", _P),
                ("knot_off", _P), ("knots", _P), ("ctrl_off", _P), ("ctrl", _P)]


_port = None


def _load_port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        lib = ctypes.CDLL(PORT_SO)
        lib.gcvo_build.restype = _P
        lib.gcvo_build.argtypes = [ctypes.POINTER(_Batch), ctypes.c_double, ctypes.c_int, ctypes.c_int]
        lib.gcvo_free.argtypes = [_P]
        lib.gcvo_lengths.argtypes = [_P, _P]
        lib.gcvo_reverse.argtypes = [_P, _P, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int]
        lib.gcvo_s_at.restype = ctypes.c_double
        lib.gcvo_s_at.argtypes = [_P, ctypes.c_int, ctypes.c_double]
        lib.gcvo_s_at_many.argtypes = [_P, _P, _P, _P, ctypes.c_int]
        lib.gcvo_speed.restype = ctypes.c_double
        lib.gcvo_speed.argtypes = [ctypes.POINTER(_Batch), ctypes.c_int, ctypes.c_double]
        lib.gcvo_point.argtypes = [ctypes.POINTER(_Batch), ctypes.c_int, ctypes.c_double, _P]
        lib.gcvo_point_seg.argtypes = [ctypes.POINTER(_Batch), ctypes.c_int, ctypes.c_int, ctypes.c_double, _P]
        lib.gcvo_table_entries.restype = ctypes.c_int64
        lib.gcvo_table_entries.argtypes = [_P]
        lib.gcvo_evals.restype = ctypes.c_int64
        lib.gcvo_evals.argtypes = [_P]
        lib.gcvo_curve_table.restype = ctypes.c_int64
        lib.gcvo_curve_table.argtypes = [_P, ctypes.c_int, _P, _P, _P]
        _port = lib
    return _port


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


class Oracle:
    """Adaptive GL3 tables of a CurveBatch, built by the C restatement of
    ArclengthCalculateCpu (gcurval/detail/cpu/arclength_calculate.h)."""

    def __init__(self, batch, max_error: float = REF_MAX_ERROR, max_depth: int = REF_MAX_DEPTH,
                 nthreads: int | None = None):
        self.lib = _load_port()
        self.batch = batch
        self.nthreads = nthreads or default_threads()
        # keep the arrays alive (the C side keeps pointers)
        self._arrs = [np.ascontiguousarray(batch.kind, np.uint8), np.ascontiguousarray(batch.degree, np.uint8),
                      np.ascontiguousarray(batch.dim, np.uint8), np.ascontiguousarray(batch.knot_off, np.int64),
                      np.ascontiguousarray(batch.knots, np.float64), np.ascontiguousarray(batch.ctrl_off, np.int64),
                      np.ascontiguousarray(batch.ctrl, np.float64)]
        k, dg, dm, ko, kv, co, cp = self._arrs
        self._b = _Batch(batch.n_curve, _ptr(k), _ptr(dg), _ptr(dm), _ptr(ko), _ptr(kv), _ptr(co), _ptr(cp))
        self.h = self.lib.gcvo_build(ctypes.byref(self._b), max_error, max_depth, self.nthreads)
        if not self.h:
            raise ValueError("oracle rejected the batch")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.gcvo_free(h)
            self.h = None

    def lengths(self) -> np.ndarray:
        out = np.zeros(self.batch.n_curve)
        self.lib.gcvo_lengths(self.h, _ptr(out))
        return out

    def point_dim(self) -> int:
        d = np.where(self.batch.kind == 0, 2, self.batch.dim)
        return int(d[0]) if d.size and np.all(d == d[0]) else 3

    def _counts(self, n_per_curve, values) -> np.ndarray:
        """Sample counts checked against the table's curve count and the value array
        (the C side trusts both sizes)."""
        n = np.ascontiguousarray(n_per_curve, np.int32)
        if n.shape != (self.batch.n_curve,):
            raise ValueError(f"{n.shape[0] if n.ndim else 0} sample counts for {self.batch.n_curve} curves")
        if np.any(n < 0) or int(n.astype(np.int64).sum()) != values.shape[0]:
            raise ValueError("sample counts do not match the number of values")
        return n

    def reverse(self, n_per_curve, positions, is_relative=True, what=0) -> np.ndarray:
        pos = np.ascontiguousarray(positions, np.float64)
        n = self._counts(n_per_curve, pos)
        width = 1 if what == 0 else self.point_dim()
        out = np.zeros(int(n.astype(np.int64).sum()) * width)
        self.lib.gcvo_reverse(self.h, _ptr(n), _ptr(pos), int(bool(is_relative)), int(what), _ptr(out),
                              self.nthreads)
        return out if what == 0 else out.reshape(-1, width)

    def s_at(self, n_per_curve, u) -> np.ndarray:
        u = np.ascontiguousarray(u, np.float64)
        n = self._counts(n_per_curve, u)
        out = np.zeros(u.shape[0])
        self.lib.gcvo_s_at_many(self.h, _ptr(n), _ptr(u), _ptr(out), self.nthreads)
        return out

    def speed(self, cid: int, u: float) -> float:
        if not 0 <= cid < self.batch.n_curve:
            raise IndexError(cid)
        return self.lib.gcvo_speed(ctypes.byref(self._b), cid, u)

    def point(self, cid: int, u: float) -> np.ndarray:
        if not 0 <= cid < self.batch.n_curve:
            raise IndexError(cid)
        out = np.zeros(3)
        self.lib.gcvo_point(ctypes.byref(self._b), cid, u, _ptr(out))
        return out

    def point_on_segment(self, cid: int, segid: int, u: float) -> np.ndarray:
        """C(u) from the polynomial piece of knot interval segid (u may be
        either end of it)."""
        if not 0 <= cid < self.batch.n_curve:
            raise IndexError(cid)
        out = np.zeros(3)
        if self.lib.gcvo_point_seg(ctypes.byref(self._b), cid, segid, u, _ptr(out)) != 0:
            raise IndexError(segid)
        return out

    def table_entries(self) -> int:
        return int(self.lib.gcvo_table_entries(self.h))

    def evals(self) -> int:
        return int(self.lib.gcvo_evals(self.h))

    def curve_table(self, cid: int):
        if not 0 <= cid < self.batch.n_curve:
            raise IndexError(cid)
        u = ctypes.POINTER(ctypes.c_double)()
        al = ctypes.POINTER(ctypes.c_double)()
        sg = ctypes.POINTER(ctypes.c_int)()
        n = self.lib.gcvo_curve_table(self.h, cid, ctypes.byref(u), ctypes.byref(al), ctypes.byref(sg))
        return (np.ctypeslib.as_array(u, (n,)).copy(), np.ctypeslib.as_array(al, (n,)).copy(),
                np.ctypeslib.as_array(sg, (n,)).copy())


class ScaledOracle:
    """The oracle with its absolute tolerance scaled per curve: max_error =
    rel x the curve's control-polygon length (a bound of its length), rounded
    down to a power of two; curves of one tolerance share one Oracle.  The
    reference's fixed absolute tolerance (1e-14) makes curves thousands of
    units long refine to its depth limit at great cost without need; at
    rel = 1e-16 every length is good to ~1e-14 relative, far below the 1e-8
    the GPU forms are checked against.  Same algorithm, only MAX_ERROR differs
    per group (a compile-time constant of the reference)."""

    def __init__(self, batch, rel: float = 1e-16, nthreads: int | None = None):
        from gcurval_gb300 import datasets as ds
        self.batch = batch
        pl = ds.control_polygon_length(batch)
        tol = np.exp2(np.floor(np.log2(np.maximum(rel * pl, 1e-300))))
        self.groups = []
        for t in np.unique(tol):
            idx = np.nonzero(tol == t)[0]
            sub = batch.subset(idx)
            self.groups.append((idx, sub, Oracle(sub, max_error=float(max(t, 1e-300)), nthreads=nthreads)))

    def lengths(self) -> np.ndarray:
        out = np.zeros(self.batch.n_curve)
        for idx, _, o in self.groups:
            out[idx] = o.lengths()
        return out

    def s_at(self, n_per_curve, u) -> np.ndarray:
        """Arc length from each curve's start to each u (curve-major, as the
        batch orders its samples)."""
        n = np.ascontiguousarray(n_per_curve, np.int64)
        u = np.ascontiguousarray(u, np.float64)
        off = np.concatenate([[0], np.cumsum(n)])
        if off[-1] != u.size:
            raise ValueError("sample counts do not match the number of values")
        out = np.zeros(u.size)
        for idx, _, o in self.groups:
            sel = np.concatenate([np.arange(off[i], off[i + 1]) for i in idx]) if idx.size else np.zeros(0, np.int64)
            out[sel] = o.s_at(n[idx].astype(np.int32), u[sel])
        return out


_ref = None


def reference_available() -> bool:
    if os.path.exists(REF_SO):
        return True
    if os.path.exists(os.path.join(REF_TREE, "gcurval", "gcurval.h")):
        try:
            build(ref=True)
        except Exception:
            return False
        return os.path.exists(REF_SO)
    return False


def _load_ref():
    global _ref
    if _ref is None:
        if not reference_available():
            raise RuntimeError("the reference CPU driver is not built (no reference tree on this host)")
        lib = ctypes.CDLL(REF_SO)
        lib.gcvref_ellipse_run.argtypes = [ctypes.c_int, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, _P,
                                           ctypes.c_int]
        lib.gcvref_bspline_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P,
                                           ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int]
        lib.gcvref_max_error.restype = ctypes.c_double
        lib.gcvref_load_bundle.argtypes = [ctypes.c_char_p, ctypes.c_int, _P, _P, ctypes.c_int, _P, ctypes.c_int]
        lib.gcvref_ellipse_rule.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _P, _P, _P]
        lib.gcvref_bspline_rule.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, ctypes.c_int, _P, _P,
                                            _P]
        _ref = lib
    return _ref


class Reference:
    """The reference's own ArclengthCalculateCpu on a batch of one curve kind
    (ellipses, or B-splines of one degree and dimension)."""

    def __init__(self, batch, nthreads: int = 1):
        self.lib = _load_ref()
        self.batch = batch
        self.nthreads = nthreads
        kinds = np.unique(batch.kind)
        if kinds.size != 1:
            raise ValueError("the reference driver takes one curve kind per batch")
        self.is_ellipse = int(kinds[0]) == 0
        if self.is_ellipse:
            prm = batch.ctrl.reshape(-1, 5)
            self.a = np.ascontiguousarray(prm[:, 0])
            self.b = np.ascontiguousarray(prm[:, 1])
        else:
            self.p = int(batch.degree[0])
            self.d = int(batch.dim[0])
            if not (np.all(batch.degree == self.p) and np.all(batch.dim == self.d)):
                raise ValueError("the reference driver takes one degree and dimension per batch")
            self.ko = np.ascontiguousarray(batch.knot_off, np.int32)
            self.kv = np.ascontiguousarray(batch.knots)
            self.cp = np.ascontiguousarray(batch.ctrl)

    def run(self, n_per_curve=None, positions=None, is_relative=True, what=0):
        """(lengths, samples-or-None): createArclengthTable + getAllCurveArclengths
        (+ arclengthReverse with host results)."""
        n = self.batch.n_curve
        lengths = np.zeros(n)
        out = None
        npc = pos = None
        if n_per_curve is not None:
            npc = np.ascontiguousarray(n_per_curve, np.int32)
            pos = np.ascontiguousarray(positions, np.float64)
            width = 1 if what == 0 else (2 if self.is_ellipse else self.d)
            out = np.zeros(int(npc.astype(np.int64).sum()) * width)
        if self.is_ellipse:
            rc = self.lib.gcvref_ellipse_run(n, _ptr(self.a), _ptr(self.b), _ptr(npc), _ptr(pos),
                                             int(bool(is_relative)), int(what), _ptr(out), _ptr(lengths),
                                             self.nthreads)
        else:
            rc = self.lib.gcvref_bspline_run(n, self.p, self.d, _ptr(self.ko), _ptr(self.kv), _ptr(self.cp),
                                             _ptr(npc), _ptr(pos), int(bool(is_relative)), int(what), _ptr(out),
                                             _ptr(lengths), self.nthreads)
        if rc != 0:
            raise RuntimeError(f"reference driver returned {rc}")
        if out is not None and what:
            out = out.reshape(-1, 2 if self.is_ellipse else self.d)
        return lengths, out


def reference_load_bundle(path: str, n_curve: int):
    """(knots_offset int32[n+1], knots, ctrl (n_points, 2)) of the first
    n_curve curves of a Bundle file, read and normalised by the reference's
    own loader (samples/sample2_bspline/dataset_loader.h:40-126)."""
    lib = _load_ref()
    cap = 64 * n_curve + 64
    ko = np.zeros(n_curve + 1, np.int32)
    kv = np.zeros(cap)
    cp = np.zeros(2 * cap)
    nk = lib.gcvref_load_bundle(path.encode(), n_curve, _ptr(ko), _ptr(kv), cap, _ptr(cp), cap)
    if nk < 0:
        raise RuntimeError("the reference loader's output does not fit (or n_curve is outside 1..1000)")
    n_pts = nk - 4 * n_curve
    return ko, kv[:nk].copy(), cp[:2 * n_pts].reshape(-1, 2).copy()


RULE_IDS = {"polyline": 0, "simpson": 1, "vincent_forsey": 2}


def reference_rule_values(rule: str, begin, end, ellipse=None, bspline=None) -> np.ndarray:
    """The reference's own point-based rule functors (gcurval/base/functors.inl.h:
    145-238) on [begin[i], end[i]]: of the ellipse (a, b) (x = a cos t,
    y = b sin t), or of one cubic 2D B-spline (knots, ctrl (n, 2), segid) on
    its knot interval segid."""
    lib = _load_ref()
    b = np.ascontiguousarray(begin, np.float64)
    e = np.ascontiguousarray(end, np.float64)
    out = np.zeros(b.size)
    if ellipse is not None:
        rc = lib.gcvref_ellipse_rule(RULE_IDS[rule], float(ellipse[0]), float(ellipse[1]), b.size, _ptr(b), _ptr(e),
                                     _ptr(out))
    else:
        kv, cp, segid = bspline
        kv = np.ascontiguousarray(kv, np.float64)
        cp = np.ascontiguousarray(cp, np.float64)
        rc = lib.gcvref_bspline_rule(RULE_IDS[rule], cp.shape[0], _ptr(kv), _ptr(cp), int(segid), b.size, _ptr(b),
                                     _ptr(e), _ptr(out))
    if rc != 0:
        raise ValueError("bad rule or knot interval")
    return out
