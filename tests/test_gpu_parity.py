"""GPU parity: the CUDA path through the C ABI against the reference's golden
vectors and the oracle (C restatement of the reference CPU driver).

Tolerances (FP64 plain path, rtol 1e-10):
  * total length:     |L_gpu - L_ref| / L_ref <= 1e-10
  * sample position:  |s_oracle(u_gpu) - target| / L <= 1e-10, where s_oracle
                      is the oracle's adaptive arc length from the curve start
  * against the reference's own sample parameters: |u_gpu - u_ref| within the
    reference's bisection resolution (its table interval / 2^22)
"""
import dataclasses
import math

import numpy as np
import pytest

import gcurval_gb300 as g
from conftest import golden_names, load_golden
from gcurval_gb300 import datasets as ds
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

LEN_RTOL = 1e-10
POS_RTOL = 1e-10


def build(batch, **kw):
    calc = g.ArclengthCalculateGpu.from_batch(batch, **kw)
    calc.createArclengthTable()
    return calc


def sample_errors(oracle, batch, u, pos, lengths):
    s = oracle.s_at(batch.n_samples, u)
    L = np.repeat(lengths, batch.n_samples)
    target = np.clip(pos, 0.0, 1.0) * L
    return np.abs(s - target) / np.where(L > 0, L, 1.0)


def ref_resolution(oracle, batch, u_ref):
    """Per-sample bisection resolution of the reference: its table interval / 2^22."""
    res = np.empty_like(u_ref)
    off = np.concatenate([[0], np.cumsum(batch.n_samples)])
    for c in range(batch.n_curve):
        tu, _, _ = oracle.curve_table(c)
        start = batch.knots[batch.knot_off[c] + (0 if batch.kind[c] == 0 else batch.degree[c])]
        edges = np.concatenate([[start], tu])
        uu = u_ref[off[c]:off[c + 1]]
        i = np.clip(np.searchsorted(edges, uu), 1, edges.size - 1)
        res[off[c]:off[c + 1]] = (edges[i] - edges[i - 1]) * 2.0 ** -22
    return res


@pytest.mark.parametrize("name", golden_names())
def test_golden_lengths(name, gpu_lib):
    b, z = load_golden(name)
    L = build(b).getAllCurveArclengths()
    ref = z["ref_lengths"]
    assert np.max(np.abs(L - ref) / ref) <= LEN_RTOL


@pytest.mark.parametrize("name", golden_names())
def test_golden_samples(name, gpu_lib):
    b, z = load_golden(name)
    calc = build(b)
    pos = z["positions"]
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST, g.GCV_RETURN_US).us
    o = Oracle(b)
    err = sample_errors(o, b, u, pos, o.lengths())
    assert np.max(err) <= POS_RTOL
    tol = ref_resolution(o, b, z["ref_us"]) + 1e-13
    assert np.all(np.abs(u - z["ref_us"]) <= tol)
    # absolute positions: L/3 and 1.5 L (beyond the end: the curve's last parameter)
    ua = calc.arclengthReverse(np.full(b.n_curve, 2), z["abs_positions"], False, g.GCV_HOST).us
    ends = np.array([b.knots[b.knot_off[c + 1] - 1 - (0 if b.kind[c] == 0 else b.degree[c])]
                     for c in range(b.n_curve)])
    np.testing.assert_allclose(ua[1::2], ends, rtol=0, atol=1e-12)
    s = o.s_at(np.full(b.n_curve, 1), ua[0::2])
    L = o.lengths()
    assert np.max(np.abs(s - L / 3) / L) <= POS_RTOL


@pytest.mark.parametrize("name", golden_names())
def test_golden_points(name, gpu_lib):
    b, z = load_golden(name)
    calc = build(b)
    pos = z["positions"]
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST, g.GCV_RETURN_US).us
    pts = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST, g.GCV_RETURN_POINTS).points
    o = Oracle(b)
    off = np.concatenate([[0], np.cumsum(b.n_samples)])
    for c in range(b.n_curve):
        for i in range(off[c], off[c + 1]):
            p = o.point(c, u[i])[: pts.shape[1]]
            scale = 1.0 + np.max(np.abs(p))
            assert np.max(np.abs(pts[i] - p)) <= 1e-11 * scale
    # the reference's points at its own parameters agree within its resolution
    dp = np.max(np.abs(pts - z["ref_points"]), axis=1)
    assert np.all(dp <= 1e-5 * (1.0 + np.max(np.abs(z["ref_points"]))))


def test_ellipses_rotated_centred_points(gpu_lib):
    b = ds.ellipses(64, n_samples=25, seed=3)
    calc = build(b)
    pos = b.sample_positions()
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us
    pts = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST, g.GCV_RETURN_POINTS).points
    o = Oracle(b)
    ref = np.array([o.point(i // 25, u[i])[:2] for i in range(u.size)])
    np.testing.assert_allclose(pts, ref, rtol=0, atol=1e-9)
    # rotation and centre do not change lengths
    b0 = ds.ellipses_from_axes(b.ctrl[0::5], b.ctrl[1::5])
    np.testing.assert_allclose(calc.getAllCurveArclengths(), build(b0).getAllCurveArclengths(), rtol=1e-14)


def test_ellipse_known_answers(gpu_lib):
    sp = pytest.importorskip("scipy.special")
    a = np.array([1.0, 3.0, 2.0, 10.0, 0.1, 7.5, 9.99])
    bb = np.array([1.0, 3.0, 1.0, 0.1, 10.0, 0.25, 0.1])
    L = build(ds.ellipses_from_axes(a, bb)).getAllCurveArclengths()
    assert L[0] == pytest.approx(2 * math.pi, rel=1e-14)
    assert L[1] == pytest.approx(6 * math.pi, rel=1e-14)
    for ai, bi, li in zip(a, bb, L):
        big, small = max(ai, bi), min(ai, bi)
        assert li == pytest.approx(4 * big * sp.ellipe(1 - (small / big) ** 2), rel=1e-12)


def test_straight_line_bspline(gpu_lib):
    pts = np.array([[0.0, 0.0], [1.0, 2.0], [2.5, 5.0], [3.0, 6.0], [4.0, 8.0]])
    kv = ds.clamped_uniform_knots(5, 3)
    b = ds._pack([1], [3], [2], [kv.size], kv, [pts.size], pts.reshape(-1), [11], "line", 1e-10)
    calc = build(b)
    L = calc.getAllCurveArclengths()[0]
    assert L == pytest.approx(math.hypot(4.0, 8.0), rel=1e-14)
    P = calc.arclengthReverse([11], np.linspace(0, 1, 11), True, g.GCV_HOST, g.GCV_RETURN_POINTS).points
    np.testing.assert_allclose(P, np.linspace(0, 1, 11)[:, None] * np.array([4.0, 8.0]), atol=1e-12)


@pytest.mark.parametrize("p,d", [(1, 2), (2, 2), (3, 2), (4, 2), (5, 2), (1, 3), (2, 3), (3, 3), (4, 3), (5, 3)])
def test_every_degree_and_dim(p, d, gpu_lib):
    rng = np.random.default_rng(100 * p + d)
    n = 24
    n_ctrl = rng.integers(p + 1, p + 40, n)
    nk, knots, clen, ctrl = ds._random_knot_bsplines(rng, np.full(n, p), np.full(n, d), n_ctrl, 1.0)
    b = ds._pack(np.ones(n), np.full(n, p), np.full(n, d), nk, knots, clen, ctrl, np.full(n, 31), "deg", 1e-10)
    calc = build(b)
    o = Oracle(b)
    Lo = o.lengths()
    assert np.max(np.abs(calc.getAllCurveArclengths() - Lo) / Lo) <= LEN_RTOL
    pos = b.sample_positions()
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us
    assert np.max(sample_errors(o, b, u, pos, Lo)) <= POS_RTOL


def test_mixed_kinds_in_one_batch(gpu_lib):
    b = ds.uneven_batch(600, seed=5, max_ctrl=300, max_samples=64)
    calc = build(b, rtol=1e-10)
    o = Oracle(b)
    Lo = o.lengths()
    L = calc.getAllCurveArclengths()
    assert np.max(np.abs(L - Lo) / Lo) <= LEN_RTOL
    pos = b.sample_positions()
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us
    assert np.max(sample_errors(o, b, u, pos, Lo)) <= POS_RTOL
    pts = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST, g.GCV_RETURN_POINTS).points
    assert pts.shape == (b.total_samples, 3)
    off = np.concatenate([[0], np.cumsum(b.n_samples)])
    for c in np.random.default_rng(1).choice(b.n_curve, 40, replace=False):
        for i in range(off[c], off[c + 1], 7):
            np.testing.assert_allclose(pts[i], o.point(int(c), u[i]), atol=1e-9 * (1 + np.abs(pts[i]).max()))


def test_repeated_knots_and_degenerate_curves(gpu_lib):
    # interior knot of multiplicity 3 (zero-width intervals) and a curve whose
    # control points coincide (length 0)
    kv = np.array([0, 0, 0, 0, 0.3, 0.3, 0.3, 0.7, 1, 1, 1, 1.0])
    c1 = np.random.default_rng(0).normal(size=(8, 2)).cumsum(0)
    c2 = np.ones((8, 2)) * 3.0
    b = ds._pack([1, 1], [3, 3], [2, 2], [12, 12], np.r_[kv, kv], [16, 16], np.r_[c1.ravel(), c2.ravel()], [9, 9],
                 "rep", 1e-10)
    calc = build(b)
    o = Oracle(b)
    L = calc.getAllCurveArclengths()
    assert L[0] == pytest.approx(o.lengths()[0], rel=LEN_RTOL)
    assert L[1] == 0.0
    pos = np.r_[np.linspace(0, 1, 9), np.linspace(0, 1, 9)]
    u = calc.arclengthReverse([9, 9], pos, True, g.GCV_HOST).us
    assert np.all(np.isfinite(u))
    np.testing.assert_array_equal(u[9:], 0.0)  # a zero-length curve samples at its start
    sub = b.subset([0])
    o0 = Oracle(sub)
    assert np.max(sample_errors(o0, sub, u[:9], pos[:9], o0.lengths())) <= POS_RTOL
    assert np.all(np.diff(u[:9]) >= 0)


def test_positions_outside_unit_interval_clamp(gpu_lib):
    b = ds.uniform_bsplines(3, n_ctrl=9, n_samples=4, seed=2)
    calc = build(b)
    u = calc.arclengthReverse([4, 4, 4], np.tile([-0.5, 0.0, 1.0, 2.0], 3), True, g.GCV_HOST).us
    np.testing.assert_array_equal(u.reshape(3, 4)[:, :2], 0.0)
    np.testing.assert_array_equal(u.reshape(3, 4)[:, 2:], 1.0)


def test_zero_sample_counts_and_empty_batch(gpu_lib):
    b = ds.uniform_bsplines(4, n_ctrl=9, n_samples=3, seed=2)
    calc = build(b)
    u = calc.arclengthReverse([0, 3, 0, 2], [0.0, 0.5, 1.0, 0.25, 0.75], True, g.GCV_HOST).us
    assert u.shape == (5,)
    o = Oracle(b)
    s = o.s_at(np.array([0, 3, 0, 2], np.int32), u)
    L = o.lengths()
    np.testing.assert_allclose(s, [0, 0.5 * L[1], L[1], 0.25 * L[3], 0.75 * L[3]], rtol=0, atol=1e-10 * L.max())
    e = ds.ellipses(0)
    ce = build(e)
    assert ce.getAllCurveArclengths().shape == (0,)
    r = ce.arclengthReverse([], [], True, g.GCV_HOST)
    assert r.n_points == 0


def test_nonfinite_control_points_do_not_hang(gpu_lib):
    b = ds.uniform_bsplines(3, n_ctrl=9, n_samples=5, seed=2)
    b.ctrl[b.ctrl_off[1] + 3] = np.nan
    calc = build(b)
    L = calc.getAllCurveArclengths()
    assert np.isfinite(L[0]) and np.isnan(L[1]) and np.isfinite(L[2])
    u = calc.arclengthReverse(b.n_samples, b.sample_positions(), True, g.GCV_HOST).us
    assert u.shape == (15,)


def test_decreasing_knots_rejected(gpu_lib):
    b = ds.uniform_bsplines(2, n_ctrl=9, seed=2)
    b.knots[b.knot_off[1] + 5] = 0.9
    b.knots[b.knot_off[1] + 6] = 0.1
    calc = g.ArclengthCalculateGpu.from_batch(b)
    with pytest.raises(g.GcvError) as ei:
        calc.createArclengthTable()
    assert ei.value.status == 1


def test_deep_segments_and_pool_growth(gpu_lib):
    sp = pytest.importorskip("scipy.special")
    # very eccentric ellipses at a tight tolerance need many leaves in their
    # single interval: the deep (global-memory) pass and the pool regrowth run
    a = np.full(300, 100.0)
    bb = np.geomspace(1e-3, 1e-1, 300)
    calc = build(ds.ellipses_from_axes(a, bb), rtol=1e-13, collect_stats=True)
    L = calc.getAllCurveArclengths()
    st = calc.stats()
    assert st["n_deep_segments"] > 0
    exact = 4 * a * sp.ellipe(1 - (bb / a) ** 2)
    assert np.max(np.abs(L - exact) / exact) <= 1e-12
    u = calc.arclengthReverse(np.full(300, 9), np.tile(np.linspace(0, 1, 9), 300), True, g.GCV_HOST).us
    assert np.all(np.diff(u.reshape(300, 9), axis=1) > 0)


def test_depth_cap_is_reported(gpu_lib):
    b = ds.uniform_bsplines(20, n_ctrl=30, seed=4)
    calc = build(b, rtol=1e-15, max_depth=2, collect_stats=True)
    st = calc.stats()
    assert st["n_capped"] > 0
    Lo = Oracle(b).lengths()
    # capped panels miss rtol; the result is still a coarse approximation
    assert np.max(np.abs(calc.getAllCurveArclengths() - Lo) / Lo) < 1e-3


def test_results_are_deterministic(gpu_lib):
    b = ds.uneven_batch(300, seed=9, max_ctrl=200, max_samples=40)
    c1 = build(b)
    c2 = build(b)
    np.testing.assert_array_equal(c1.getAllCurveArclengths(), c2.getAllCurveArclengths())
    pos = b.sample_positions()
    np.testing.assert_array_equal(c1.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us,
                                  c2.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us)


# ---------------------------------------------------- full workload sizes
def _full_size_checks(b, n_check=300, seed=0):
    calc = build(b, collect_stats=True)
    L = calc.getAllCurveArclengths()
    pos = b.sample_positions()
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us
    off = np.concatenate([[0], np.cumsum(b.n_samples)])
    # size-independent properties: every curve's parameters are sorted and
    # start / end at the curve's ends
    seg = np.repeat(np.arange(b.n_curve), b.n_samples)
    du = np.diff(u)
    same = seg[1:] == seg[:-1]
    assert np.all(du[same] >= -1e-15)
    starts = np.where(b.kind == 0, 0.0, b.knots[b.knot_off[:-1] + b.degree.astype(np.int64)])
    np.testing.assert_array_equal(u[off[:-1]], starts)
    # a random subset against the oracle
    idx = np.sort(np.random.default_rng(seed).choice(b.n_curve, n_check, replace=False))
    sub = b.subset(idx)
    o = Oracle(sub)
    Lo = o.lengths()
    assert np.max(np.abs(L[idx] - Lo) / Lo) <= LEN_RTOL
    usub = np.concatenate([u[off[i]:off[i + 1]] for i in idx])
    err = sample_errors(o, sub, usub, sub.sample_positions(), Lo)
    assert np.max(err) <= POS_RTOL
    return calc


def test_full_size_ellipses_4096x1000(gpu_lib):
    calc = _full_size_checks(ds.ellipses(4096, n_samples=1000, seed=0))
    assert calc.stats()["n_samples"] == 4096 * 1000


def test_full_size_uniform_bsplines_10000x1024(gpu_lib):
    calc = _full_size_checks(ds.uniform_bsplines(10000, n_samples=1024, seed=0), n_check=200)
    assert calc.stats()["n_segments"] == 10000 * 61


def test_host_buffers_stream_in_chunks_like_device_buffers(gpu_lib):
    # more than one 256 MB chunk of positions, curves of every code: the
    # chunked host pipeline must give the device path's results bit for bit
    torch = pytest.importorskip("torch")
    b = ds.uneven_batch(40000, seed=11)
    pos = b.sample_positions()
    assert b.total_samples * 8 > (256 << 20)
    calc = g.ArclengthCalculateGpu.from_batch(b, precision=g.GCV_MIXED)
    calc.createArclengthTable()
    h_out = np.zeros(b.total_samples)
    calc.arclengthReverseInto(b.n_samples, pos, h_out, True, g.GCV_RETURN_US)
    d_cnt = torch.from_numpy(b.n_samples.astype(np.int32)).cuda()
    d_pos = torch.from_numpy(pos).cuda()
    d_out = torch.empty(b.total_samples, dtype=torch.float64, device="cuda")
    calc.arclengthReverseInto(d_cnt, d_pos, d_out, True, g.GCV_RETURN_US)
    np.testing.assert_array_equal(h_out, d_out.cpu().numpy())
    # page-locked caller buffers are copied directly, without staging: the
    # same results, also with only one side page-locked
    p_pos, p_out = g.pinned_copy(pos), g.pinned_empty(b.total_samples)
    calc.arclengthReverseInto(b.n_samples, p_pos, p_out, True, g.GCV_RETURN_US)
    np.testing.assert_array_equal(h_out, p_out)
    h2 = np.zeros(b.total_samples)
    calc.arclengthReverseInto(b.n_samples, p_pos, h2, True, g.GCV_RETURN_US)
    np.testing.assert_array_equal(h_out, h2)
    p_out[:] = 0.0
    calc.arclengthReverseInto(b.n_samples, pos, p_out, True, g.GCV_RETURN_US)
    np.testing.assert_array_equal(h_out, p_out)
    calc.close()


def test_create_from_page_locked_arrays(gpu_lib):
    # a batch whose host arrays are page-locked: the same table and samples
    b = ds.uneven_batch(3000, seed=12)
    pb = dataclasses.replace(b, **{f: g.pinned_copy(getattr(b, f)) for f in
                                   ("kind", "degree", "dim", "knot_off", "knots", "ctrl_off", "ctrl", "n_samples")})
    pos = b.sample_positions()
    out = []
    # copied from pageable arrays, copied from page-locked ones, read in place
    for bb, pp, in_place in ((b, pos, False), (pb, g.pinned_copy(pos), False), (pb, g.pinned_copy(pos), True)):
        with g.ArclengthCalculateGpu.from_batch(bb, precision=g.GCV_MIXED, host_in_place=in_place) as calc:
            for _ in range(2):  # a second table build reads the arrays again
                calc.createArclengthTable()
            u = np.zeros(b.total_samples)
            calc.arclengthReverseInto(bb.n_samples, pp, u, True, g.GCV_RETURN_US)
            out.append((calc.getAllCurveArclengths(), u))
    for k in (1, 2):
        np.testing.assert_array_equal(out[0][0], out[k][0])
        np.testing.assert_array_equal(out[0][1], out[k][1])
