"""The oracle's restatement of the reference's point-based length rules
(oracle/point_rules.py): exact on straight lines, convergent at their orders
on circular arcs, and the reference's adaptive bisection with them reaches
the circle's length."""
import numpy as np
import pytest

from oracle import point_rules as pr

RULES = [pr.POLYLINE, pr.SIMPSON, pr.VINCENT_FORSEY]


def circle(r):
    return lambda t: np.array([r * np.cos(t), r * np.sin(t)])


@pytest.mark.parametrize("kind", RULES)
def test_rules_are_exact_on_lines(kind):
    line = lambda t: np.array([1.0 + 3.0 * t, -2.0 + 4.0 * t, 0.5 * t])
    assert pr.rule_on(kind, line, 0.2, 1.7) == pytest.approx(np.linalg.norm([4.5, 6.0, 0.75]), rel=1e-14)


@pytest.mark.parametrize("kind, order", [(pr.POLYLINE, 3), (pr.SIMPSON, 5), (pr.VINCENT_FORSEY, 5)])
def test_local_error_order_on_arcs(kind, order):
    c = circle(2.0)
    errs = []
    for h in (0.2, 0.1, 0.05):
        errs.append(abs(pr.rule_on(kind, c, 0.3, 0.3 + h) - 2.0 * h))
    # halving the arc divides the error by about 2^order
    for e0, e1 in zip(errs, errs[1:]):
        assert e0 / e1 == pytest.approx(2.0 ** order, rel=0.1)


@pytest.mark.parametrize("kind", RULES)
def test_adaptive_bisection_reaches_the_circle_length(kind):
    L = pr.adaptive_length(kind, circle(1.5), 0.0, 2 * np.pi, eps0=1e-9, max_depth=30)
    assert abs(L - 3.0 * np.pi) <= 3e-9


def test_rule_values_equal_the_reference_functors():
    """The restated rules give the reference's own functors' values bit for
    bit (tests/golden/point_rules.npz, written by make_golden.py from
    PolylineMethod / SimpsonMethod / VincentForseyRule compiled from the
    reference), on ellipse points from libm's cos / sin and on cubic
    B-spline points from the oracle's de Boor (itself bit-identical to the
    reference's)."""
    import math
    import os

    from gcurval_gb300 import datasets as ds
    from oracle.oracle import Oracle

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "point_rules.npz"))
    for i, (a, b) in enumerate(zip(z["ell_a"], z["ell_b"])):
        pt = lambda t, a=float(a), b=float(b): np.array([a * math.cos(t), b * math.sin(t)])
        for kind in RULES:
            got = [pr.rule_on(kind, pt, float(t0), float(t1)) for t0, t1 in zip(z["ell_begin"][i], z["ell_end"][i])]
            np.testing.assert_array_equal(got, z[f"ell_{kind}"][i])
    n = z["bs_knot_off"].size - 1
    bs = ds.CurveBatch(np.ones(n, np.uint8), np.full(n, 3, np.uint8), np.full(n, 2, np.uint8), z["bs_knot_off"],
                       z["bs_knots"], z["bs_ctrl_off"], z["bs_ctrl"], np.ones(n, np.int32))
    o = Oracle(bs)
    for c in range(n):
        for kind in RULES:
            got = []
            for sid, t0, t1 in zip(z["bs_seg"][c], z["bs_begin"][c], z["bs_end"][c]):
                pt = lambda t, c=c, sid=int(sid): o.point_on_segment(c, sid, t)[:2]
                got.append(pr.rule_on(kind, pt, float(t0), float(t1)))
            np.testing.assert_array_equal(got, z[f"bs_{kind}"][c])
