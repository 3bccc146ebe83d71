"""gcv_bspline_lengths_noalloc: the allocation-free entry point for callers that
cannot call cudaMalloc (fixed device-memory budgets, code inside another
library's allocator hooks).  Its results must equal the allocating path's
(gcv_create_bsplines + gcv_create_arclength_table + gcv_get_all_curve_arclengths)
within the length tolerance the parity tests use, on consecutive calls that
share the entry point's static scratch array.

The file name sorts last so that a run stopping at the first failure has run
every other test first.
"""
import ctypes

import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import _lib
from gcurval_gb300 import datasets as ds

pytestmark = pytest.mark.gpu

LEN_RTOL = 1e-10
_P = ctypes.c_void_p


def _noalloc_fn():
    lib = g.load()
    fn = lib.gcv_bspline_lengths_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_double, ctypes.c_int, _P, _P,
                   ctypes.POINTER(ctypes.c_int64)]
    return lib, fn


def _allocating_lengths(batch, rtol=1e-10, max_depth=30, with_capped=False):
    p, d, ko, kv, cp = ds.reference_layout(batch)
    calc = g.ArclengthCalculateGpu.bsplines(p, d, ko, kv, cp, rtol=rtol, max_depth=max_depth)
    calc.createArclengthTable()
    out = calc.getAllCurveArclengths()
    capped = calc.stats()["n_capped"]
    calc.close()
    return (out, capped) if with_capped else out


def _call(n_curve, p, d, ko, kv, cp, rtol=1e-10, max_depth=30):
    """(status, lengths, capped) of one call on device copies of the arrays."""
    torch = pytest.importorskip("torch")
    lib, fn = _noalloc_fn()
    dev = torch.device("cuda", 0)
    t_ko = torch.from_numpy(np.ascontiguousarray(ko, np.int32)).to(dev)
    t_kv = torch.from_numpy(np.ascontiguousarray(kv, np.float64)).to(dev)
    t_cp = torch.from_numpy(np.ascontiguousarray(cp, np.float64)).to(dev)
    out = torch.full((max(n_curve, 1),), float("nan"), dtype=torch.float64, device=dev)
    capped = ctypes.c_int64(-1)
    torch.cuda.synchronize()
    st = fn(n_curve, p, d, _P(t_ko.data_ptr()), _P(t_kv.data_ptr()), _P(t_cp.data_ptr()), rtol, max_depth,
            _P(out.data_ptr()), None, ctypes.byref(capped))
    return st, out.cpu().numpy()[:n_curve], capped.value, lib


def _noalloc_lengths(batch, rtol=1e-10, max_depth=30, with_capped=False):
    p, d, ko, kv, cp = ds.reference_layout(batch)
    st, out, capped, lib = _call(batch.n_curve, p, d, ko, kv, cp, rtol, max_depth)
    assert st == _lib.GCV_OK, lib.gcv_last_error()
    return (out, capped) if with_capped else out


@pytest.mark.parametrize("degree,dim", [(3, 2), (5, 3), (2, 2)])
def test_noalloc_matches_allocating_path_twice(degree, dim):
    a = ds.uniform_bsplines(400, n_ctrl=40, degree=degree, dim=dim, seed=11 + degree)
    b = ds.uniform_bsplines(250, n_ctrl=23, degree=degree, dim=dim, seed=31 + degree)
    ref_a = _allocating_lengths(a)
    ref_b = _allocating_lengths(b)
    # two calls in a row on different batches share the scratch array
    got_a = _noalloc_lengths(a)
    got_b = _noalloc_lengths(b)
    assert np.max(np.abs(got_a - ref_a) / ref_a) <= LEN_RTOL
    assert np.max(np.abs(got_b - ref_b) / ref_b) <= LEN_RTOL
    # and the same batch again gives the same numbers
    np.testing.assert_array_equal(_noalloc_lengths(a), got_a)


def test_noalloc_rejects_batches_above_its_limit():
    torch = pytest.importorskip("torch")
    lib, fn = _noalloc_fn()
    # knots_offset[n] implies more intervals than the static scratch holds;
    # the call must refuse before launching anything
    n = 20000
    p = 3
    per = 64 + p + 1
    ko = torch.arange(0, (n + 1) * per, per, dtype=torch.int32, device="cuda")
    assert (n * (per - 2 * p - 1)) > 1048576
    kv = torch.zeros(8, dtype=torch.float64, device="cuda")
    cp = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    st = fn(n, p, 2, _P(ko.data_ptr()), _P(kv.data_ptr()), _P(cp.data_ptr()), 1e-10, 30, _P(out.data_ptr()), None,
            None)
    assert st == _lib.GCV_ERR_INVALID
    assert b"allocation-free limit" in lib.gcv_last_error()


def test_noalloc_reports_capped_panels_like_the_allocating_path():
    # a depth limit of 3 cannot meet rtol 1e-12 on random-walk cubics: both
    # paths accept the same panels at the cap and count them
    a = ds.uniform_bsplines(60, n_ctrl=12, degree=3, dim=2, seed=5)
    ref, ref_capped = _allocating_lengths(a, rtol=1e-12, max_depth=3, with_capped=True)
    got, capped = _noalloc_lengths(a, rtol=1e-12, max_depth=3, with_capped=True)
    assert ref_capped > 0
    assert capped == ref_capped
    assert np.max(np.abs(got - ref) / ref) <= LEN_RTOL
    # and a batch that meets its tolerance reports none
    assert _noalloc_lengths(a, with_capped=True)[1] == 0


@pytest.mark.parametrize("case", ["nonzero_start", "too_short", "decreasing"])
def test_noalloc_rejects_malformed_offsets_before_reading_through_them(case):
    # The offsets are checked by the entry point's first kernel; the kernels
    # that read knots and control points through them return at once, so the
    # arrays below (sized for the well-formed batch) are never over-read.
    a = ds.uniform_bsplines(8, n_ctrl=10, degree=3, dim=2, seed=2)
    p, d, ko, kv, cp = ds.reference_layout(a)
    ko = ko.astype(np.int64).copy()
    if case == "nonzero_start":
        ko[0] = 3  # knots_offset[n] unchanged: n_seg stays in range
        want = b"offsets must start at 0"
    elif case == "too_short":
        ko[4] = ko[3] + 5  # curve 3 gets 5 < 2 * 3 + 1 knots
        want = b"curve 3: fewer than 2 * degree + 1 knots"
    else:
        ko[5], ko[6] = ko[6], ko[5]  # curve 5's offsets decrease
        want = b"curve 5: fewer than 2 * degree + 1 knots"
    st, out, capped, lib = _call(a.n_curve, p, d, ko, kv, cp)
    assert st == _lib.GCV_ERR_INVALID
    assert want in lib.gcv_last_error()
    # nothing was written to the output
    assert np.all(np.isnan(out))
    # and the entry point still works afterwards
    np.testing.assert_allclose(_noalloc_lengths(a), _allocating_lengths(a), rtol=LEN_RTOL)
