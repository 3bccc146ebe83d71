"""CPU oracle of the reference's point-based length rules and of its adaptive
bisection with them, in FP64 numpy / Python.

Test infrastructure only: the plugin header's Polyline, Simpson and
Vincent-Forsey choices (include/gcurval_gb300/gcurval.cuh) are checked
against these restatements.

Rules (gcurval/base/functors.inl.h:145-238), for the points a = C(begin),
m = C((begin + end) / 2), b = C(end):
  Polyline        |b - a|                                          (:145-165)
  Simpson         (|-3a + 4m - b| + 4 |b - a| + |a - 4m + 3b|) / 6   (:167-206)
  VincentForsey   4/3 (|a - m| + |b - m|) - 1/3 |b - a|            (:208-238)
Adaptive driver (gcurval/detail/cpu/arclength_calculate.h:242-279,
arclengthRecursive): split [begin, end] at its midpoint while
|L + R - parent| exceeds the level's tolerance and the depth is below the
limit; the result is L + R.
"""
from __future__ import annotations

import math

import numpy as np

POLYLINE, SIMPSON, VINCENT_FORSEY = "polyline", "simpson", "vincent_forsey"


def _norm(v) -> float:
    """sqrt(x0^2 + x1^2 (+ x2^2)), summed left to right like a fixed-size
    vector's norm()."""
    s = 0.0
    for x in v:
        s += float(x) * float(x)
    return math.sqrt(s)


def rule(kind: str, a, m, b) -> float:
    """The rule from the points a = C(begin), m = C(mid), b = C(end), with the
    reference's operations in its order (so equal points give equal bits)."""
    a, m, b = (np.asarray(x, np.float64) for x in (a, m, b))
    if kind == POLYLINE:
        return _norm(b - a)
    if kind == SIMPSON:
        return 1.0 / 6.0 * (_norm(-3.0 * a + 4.0 * m - b) + 4.0 * _norm(b - a) + _norm(a - 4.0 * m + 3.0 * b))
    if kind == VINCENT_FORSEY:
        return 4.0 / 3.0 * (_norm(a - m) + _norm(b - m)) - 1.0 / 3.0 * _norm(b - a)
    raise ValueError(kind)


def rule_on(kind: str, point, t0: float, t1: float) -> float:
    """The rule on [t0, t1] of the curve point(t); the midpoint is
    (t0 + t1) / 2 as in the reference."""
    return rule(kind, point(t0), point((t0 + t1) / 2.0), point(t1))


def adaptive_length(kind: str, point, t0: float, t1: float, eps0: float, max_depth: int = 23) -> float:
    """The reference's recursive bisection with the rule; the tolerance of
    level k is eps0 * 2^-k (gcurval/base/constants.inl.h:8-30)."""

    def rec(b, e, parent, level):
        mid = 0.5 * (b + e)
        left = rule_on(kind, point, b, mid)
        right = rule_on(kind, point, mid, e)
        if level < max_depth and abs(left + right - parent) > eps0 * 2.0 ** -level:
            left = rec(b, mid, left, level + 1)
            right = rec(mid, e, right, level + 1)
        return left + right

    return rec(t0, t1, rule_on(kind, point, t0, t1), 0)
