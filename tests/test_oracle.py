"""The oracle (C restatement of the reference CPU driver) against the golden
vectors produced by the reference's own driver, known answers, and (where the
reference tree is present) the live reference."""
import math

import numpy as np
import pytest

from conftest import golden_names, load_golden
from gcurval_gb300 import datasets as ds
from oracle.oracle import Oracle, Reference, reference_available


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_golden(name):
    b, z = load_golden(name)
    o = Oracle(b, max_error=float(z["max_error"]), max_depth=int(z["max_depth"]), nthreads=2)
    # same algorithm, same operation order: bit-identical
    np.testing.assert_array_equal(o.lengths(), z["ref_lengths"])
    np.testing.assert_array_equal(o.reverse(b.n_samples, z["positions"], True, 0), z["ref_us"])
    np.testing.assert_array_equal(o.reverse(b.n_samples, z["positions"], True, 1), z["ref_points"])
    np.testing.assert_array_equal(o.reverse(np.full(b.n_curve, 2), z["abs_positions"], False, 0), z["ref_us_abs"])


def test_circle_and_ellipse_known_answers():
    a = np.array([1.0, 2.5, 2.0, 10.0, 0.1, 5.969])
    bb = np.array([1.0, 2.5, 1.0, 0.1, 10.0, 8.458])
    o = Oracle(ds.ellipses_from_axes(a, bb), nthreads=1)
    L = o.lengths()
    assert L[0] == pytest.approx(2 * math.pi, rel=1e-15)
    assert L[1] == pytest.approx(5 * math.pi, rel=1e-15)
    scipy_special = pytest.importorskip("scipy.special")
    for ai, bi, li in zip(a, bb, L):
        big, small = max(ai, bi), min(ai, bi)
        exact = 4 * big * scipy_special.ellipe(1 - (small / big) ** 2)
        assert li == pytest.approx(exact, rel=1e-13)


def test_straight_bspline_is_polygon_length():
    # collinear, monotone control points: the curve is the segment between the ends
    pts = np.array([[0.0, 0.0], [1.0, 2.0], [2.5, 5.0], [3.0, 6.0], [4.0, 8.0]])
    kv = ds.clamped_uniform_knots(5, 3)
    b = ds._pack([1], [3], [2], [kv.size], kv, [pts.size], pts.reshape(-1), [0], "line", 1e-10)
    o = Oracle(b)
    assert o.lengths()[0] == pytest.approx(math.hypot(4.0, 8.0), rel=1e-14)


def test_s_at_inverts_reverse():
    b = ds.uniform_bsplines(6, n_ctrl=10, n_samples=21, seed=4)
    o = Oracle(b)
    pos = b.sample_positions()
    u = o.reverse(b.n_samples, pos)
    s = o.s_at(b.n_samples, u)
    L = np.repeat(o.lengths(), b.n_samples)
    # the reference's bisection resolution: well under 1e-9 of the length here
    assert np.max(np.abs(s - pos * L) / L) < 1e-9


def test_mixed_batch_lengths_equal_per_kind_runs():
    e = ds.ellipses(5, seed=3)
    s = ds.uniform_bsplines(4, n_ctrl=8, seed=3)
    both = ds._pack(np.r_[e.kind, s.kind], np.r_[e.degree, s.degree], np.r_[e.dim, s.dim],
                    np.r_[np.diff(e.knot_off), np.diff(s.knot_off)], np.r_[e.knots, s.knots],
                    np.r_[np.diff(e.ctrl_off), np.diff(s.ctrl_off)], np.r_[e.ctrl, s.ctrl],
                    np.r_[e.n_samples, s.n_samples], "both", 1e-10)
    L = Oracle(both).lengths()
    np.testing.assert_array_equal(L[:5], Oracle(e).lengths())
    np.testing.assert_array_equal(L[5:], Oracle(s).lengths())


def test_oracle_rejects_mismatched_counts():
    b = ds.uniform_bsplines(3, n_ctrl=8, n_samples=4, seed=1)
    o = Oracle(b)
    with pytest.raises(ValueError):
        o.s_at([4], np.zeros(4))  # 1 count for 3 curves
    with pytest.raises(ValueError):
        o.reverse([4, 4, 4], np.zeros(11))
    with pytest.raises(IndexError):
        o.point(3, 0.5)


def _repeated_knot_curve():
    kv = np.array([0, 0, 0, 0, 0.3, 0.3, 0.3, 0.7, 1, 1, 1, 1.0])
    pts = np.random.default_rng(0).normal(size=(8, 2)).cumsum(0)
    return ds._pack([1], [3], [2], [12], kv, [16], pts.ravel(), [5], "rep", 1e-10), kv, pts


def test_zero_width_spans_add_nothing():
    # the length with a triple interior knot equals the sum over the non-degenerate spans,
    # measured by splitting the curve at the knot into two clamped pieces
    b, kv, pts = _repeated_knot_curve()
    L = Oracle(b).lengths()[0]
    assert np.isfinite(L)
    # the curve interpolates its control point 3 at t = 0.3 (C0 joint): it is the union of
    # the cubic pieces on [0, 0.3] and [0.3, 1]
    left = ds._pack([1], [3], [2], [8], np.array([0, 0, 0, 0, 1, 1, 1, 1.0]), [8], pts[:4].ravel(), [0], "l", 1e-10)
    kr = np.array([0.3, 0.3, 0.3, 0.3, 0.7, 1, 1, 1, 1.0])
    right = ds._pack([1], [3], [2], [9], kr, [10], pts[3:].ravel(), [0], "r", 1e-10)
    assert L == pytest.approx(Oracle(left).lengths()[0] + Oracle(right).lengths()[0], rel=1e-13)


@pytest.mark.skipif(not reference_available(), reason="reference tree not present on this host")
def test_reference_returns_nan_on_repeated_knots():
    # documents the reference behaviour the oracle deliberately departs from:
    # its de Boor divides 0 by 0 on a zero-width span
    b, _, _ = _repeated_knot_curve()
    Lr, _ = Reference(b).run()
    assert np.isnan(Lr[0])


@pytest.mark.skipif(not reference_available(), reason="reference tree not present on this host")
def test_port_matches_live_reference_random():
    rng = np.random.default_rng(99)
    for p, d in ((3, 2), (2, 2), (5, 3)):
        b = ds.uniform_bsplines(5, n_ctrl=int(rng.integers(p + 2, 20)), degree=p, dim=d, n_samples=7,
                                seed=int(rng.integers(1 << 30)))
        pos = rng.uniform(-0.1, 1.1, b.total_samples)
        Lr, ur = Reference(b).run(b.n_samples, pos, True, 0)
        o = Oracle(b)
        np.testing.assert_array_equal(o.lengths(), Lr)
        np.testing.assert_array_equal(o.reverse(b.n_samples, pos, True, 0), ur)
