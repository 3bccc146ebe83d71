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
