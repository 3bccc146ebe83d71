"""The reference's on-disk B-spline format ("Bundle" text files, the only input
format it ships; samples/sample2_bspline/dataset_loader.h:40-126).

Per curve, whitespace separated: ``degree n_ctrl n_knots``, then the n_ctrl x
coordinates, the n_ctrl y coordinates and the n_knots knots.  The reference
loader centres every curve's control points on their mean and divides them by
the largest absolute coordinate (dataset_loader.h:77-103); ``normalize`` does
the same.  Parsing is one vectorised pass over all numbers of a file.

``load_device`` does the parsing and the normalisation on the GPU
(include/gcurval_gb300_bundle.h) and returns the device arrays that
``ArclengthCalculateGpu.from_device_batch`` takes; the host only reads the
files' bytes.
"""
from __future__ import annotations

import numpy as np

import ctypes

from .datasets import KIND_BSPLINE, CurveBatch


def parse(text: str):
    """(degrees, ctrl list of (n, 2) arrays, knot list) of every curve in one
    Bundle text."""
    vals = np.array(text.split(), dtype=np.float64)
    degrees, ctrls, knots = [], [], []
    i, n = 0, vals.size
    while i + 3 <= n:
        p, nc, nk = int(vals[i]), int(vals[i + 1]), int(vals[i + 2])
        i += 3
        if nc < p + 1 or nk != nc + p + 1 or i + 2 * nc + nk > n:
            raise ValueError(f"malformed curve record at number {i - 3}: degree {p}, {nc} points, {nk} knots")
        x = vals[i:i + nc]
        y = vals[i + nc:i + 2 * nc]
        i += 2 * nc
        knots.append(vals[i:i + nk].copy())
        i += nk
        degrees.append(p)
        ctrls.append(np.stack([x, y], axis=1))
    if i != n:
        raise ValueError("trailing numbers after the last curve record")
    return degrees, ctrls, knots


def normalize(ctrl: np.ndarray) -> np.ndarray:
    """Centre on the mean control point, scale by the largest |coordinate|
    (dataset_loader.h:77-103)."""
    c = ctrl - ctrl.mean(axis=0)
    m = np.abs(c).max()
    return c / m if m > 0 else c


def load(paths, n_curve: int | None = None, dim: int = 2, samples_per_curve: int = 1024,
         rtol: float = 1e-10) -> CurveBatch:
    """A CurveBatch of the first n_curve curves of the Bundle files (all when
    None), normalised like the reference loader; dim 3 adds z = 0."""
    degrees, ctrls, knots = [], [], []
    for p in ([paths] if isinstance(paths, str) else paths):
        with open(p) as f:
            d, c, k = parse(f.read())
        degrees += d
        ctrls += c
        knots += k
        if n_curve is not None and len(degrees) >= n_curve:
            break
    if n_curve is not None:
        degrees, ctrls, knots = degrees[:n_curve], ctrls[:n_curve], knots[:n_curve]
    n = len(degrees)
    pts = [normalize(c) for c in ctrls]
    if dim == 3:
        pts = [np.concatenate([q, np.zeros((q.shape[0], 1))], axis=1) for q in pts]
    knot_off = np.concatenate([[0], np.cumsum([k.size for k in knots])]).astype(np.int64)
    ctrl_off = np.concatenate([[0], np.cumsum([q.size for q in pts])]).astype(np.int64)
    return CurveBatch(np.full(n, KIND_BSPLINE, np.uint8), np.asarray(degrees, np.uint8), np.full(n, dim, np.uint8),
                      knot_off, np.concatenate(knots) if n else np.zeros(0),
                      ctrl_off, np.concatenate([q.reshape(-1) for q in pts]) if n else np.zeros(0),
                      np.full(n, samples_per_curve, np.int32), None, "bundle", rtol)


def load_device(paths, n_curve: int | None = None, dim: int = 2, normalize: bool = True, stream=None):
    """(kind, degree, dim, knot_off, knots, ctrl_off, ctrl) CUDA tensors of the
    first n_curve curves (all when None) of the Bundle files (a path, a list
    of paths, or bytes objects holding file contents), parsed and normalised
    on the GPU (gcv_bundle_parse / gcv_bundle_fill).  Same numbers as
    ``load``; the files are joined with a newline between them."""
    import torch

    from . import _lib
    lib = _lib.load()
    items = [paths] if isinstance(paths, (str, bytes)) else list(paths)
    blobs = []
    for it in items:
        if isinstance(it, bytes):
            blobs.append(it)
        else:
            with open(it, "rb") as f:
                blobs.append(f.read())
    off = [0]
    for bl in blobs:
        off.append(off[-1] + len(bl) + 1)
    text = b"\n".join(blobs) + b"\n"
    host = torch.frombuffer(bytearray(text), dtype=torch.uint8)
    dev = host.to("cuda")
    file_off = (ctypes.c_int64 * len(off))(*off)
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    h = ctypes.c_void_p()
    _lib.check(lib.gcv_bundle_parse(ctypes.c_void_p(dev.data_ptr()), len(text), file_off, len(blobs),
                                    -1 if n_curve is None else int(n_curve), int(dim), _lib.GCV_DEVICE,
                                    ctypes.c_void_p(st), ctypes.byref(h)))
    try:
        nc, nk, nv = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(lib.gcv_bundle_sizes(h, ctypes.byref(nc), ctypes.byref(nk), ctypes.byref(nv)))
        n = nc.value
        u8 = dict(dtype=torch.uint8, device="cuda")
        arrs = (torch.empty(n, **u8), torch.empty(n, **u8), torch.empty(n, **u8),
                torch.empty(n + 1, dtype=torch.int64, device="cuda"),
                torch.empty(nk.value, dtype=torch.float64, device="cuda"),
                torch.empty(n + 1, dtype=torch.int64, device="cuda"),
                torch.empty(nv.value, dtype=torch.float64, device="cuda"))
        _lib.check(lib.gcv_bundle_fill(h, int(bool(normalize)), *[ctypes.c_void_p(a.data_ptr()) for a in arrs]))
    finally:
        lib.gcv_bundle_destroy(h)
    return arrs
