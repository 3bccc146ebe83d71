"""GPU parity of the mixed-precision path (GCV_MIXED: float-float integrand and
panels on the FP32 pipes; FP64 prefix sum, near-tolerance error test and final
Newton update) against the FP64 oracle.

Tolerance (the path's rtol, 1e-8):
  * total length:    |L - L_oracle| / L_oracle <= 1e-8
  * sample position: |s_oracle(u) - target| / L <= 1e-8
"""
import math

import numpy as np
import pytest

import gcurval_gb300 as g
from conftest import golden_names, load_golden
from gcurval_gb300 import datasets as ds
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def build(batch, **kw):
    kw.setdefault("precision", g.GCV_MIXED)
    calc = g.ArclengthCalculateGpu.from_batch(batch, **kw)
    calc.createArclengthTable()
    return calc


def check(batch, oracle=None, calc=None):
    calc = calc or build(batch)
    o = oracle or Oracle(batch)
    Lo = o.lengths()
    L = calc.getAllCurveArclengths()
    len_err = np.max(np.abs(L - Lo) / Lo) if Lo.size else 0.0
    pos = batch.sample_positions()
    u = calc.arclengthReverse(batch.n_samples, pos, True, g.GCV_HOST).us
    s = o.s_at(batch.n_samples, u)
    Lr = np.repeat(Lo, batch.n_samples)
    pos_err = np.max(np.abs(s - np.clip(pos, 0, 1) * Lr) / Lr) if u.size else 0.0
    return len_err, pos_err, calc


@pytest.mark.parametrize("name", golden_names())
def test_mixed_golden(name, gpu_lib):
    b, z = load_golden(name)
    calc = build(b)
    L = calc.getAllCurveArclengths()
    assert np.max(np.abs(L - z["ref_lengths"]) / z["ref_lengths"]) <= RTOL
    le, pe, _ = check(b, calc=calc)
    assert le <= RTOL and pe <= RTOL


def test_mixed_ellipse_known_answers(gpu_lib):
    sp = pytest.importorskip("scipy.special")
    a = np.array([1.0, 3.0, 2.0, 10.0, 0.1, 7.5, 9.99, 0.37])
    bb = np.array([1.0, 3.0, 1.0, 0.1, 10.0, 0.25, 0.1, 5.2])
    L = build(ds.ellipses_from_axes(a, bb)).getAllCurveArclengths()
    assert L[0] == pytest.approx(2 * math.pi, rel=1e-12)
    for ai, bi, li in zip(a, bb, L):
        big, small = max(ai, bi), min(ai, bi)
        assert li == pytest.approx(4 * big * sp.ellipe(1 - (small / big) ** 2), rel=RTOL)


@pytest.mark.parametrize("p,d", [(1, 2), (2, 2), (3, 2), (4, 2), (5, 2), (1, 3), (2, 3), (3, 3), (4, 3), (5, 3)])
def test_mixed_every_degree_and_dim(p, d, gpu_lib):
    rng = np.random.default_rng(500 + 10 * p + d)
    n = 24
    n_ctrl = rng.integers(p + 1, p + 40, n)
    nk, knots, clen, ctrl = ds._random_knot_bsplines(rng, np.full(n, p), np.full(n, d), n_ctrl, 1.0)
    b = ds._pack(np.ones(n), np.full(n, p), np.full(n, d), nk, knots, clen, ctrl, np.full(n, 29), "deg", RTOL)
    le, pe, _ = check(b)
    assert le <= RTOL and pe <= RTOL


def test_mixed_uneven_batch(gpu_lib):
    b = ds.uneven_batch(800, seed=21, max_ctrl=400, max_samples=64)
    le, pe, calc = check(b)
    assert le <= RTOL and pe <= RTOL
    pts = calc.arclengthReverse(b.n_samples, b.sample_positions(), True, g.GCV_HOST, g.GCV_RETURN_POINTS).points
    assert np.all(np.isfinite(pts))


def test_mixed_matches_fp64_path_closely(gpu_lib):
    b = ds.uniform_bsplines(200, n_ctrl=40, seed=8)
    Lm = build(b).getAllCurveArclengths()
    Lp = build(b, precision=g.GCV_PLAIN_FP64, rtol=1e-12).getAllCurveArclengths()
    # float-float panels are far more accurate than the 1e-8 the path promises
    assert np.max(np.abs(Lm - Lp) / Lp) <= 1e-9


def test_mixed_full_size_3d_workload(gpu_lib):
    # 100,000 3D B-splines, degree 3|5, 32-256 control points, 2,048 samples each
    b = ds.mixed3d_bsplines(100_000, n_samples=2048, seed=0)
    calc = build(b, collect_stats=True)
    L = calc.getAllCurveArclengths()
    assert np.all(np.isfinite(L)) and np.all(L > 0)
    pos = b.sample_positions()
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us
    off = np.concatenate([[0], np.cumsum(b.n_samples)])
    cur = np.repeat(np.arange(b.n_curve), b.n_samples)
    du = np.diff(u)
    assert np.all(du[cur[1:] == cur[:-1]] >= -1e-15)
    idx = np.sort(np.random.default_rng(3).choice(b.n_curve, 120, replace=False))
    sub = b.subset(idx)
    o = Oracle(sub)
    Lo = o.lengths()
    assert np.max(np.abs(L[idx] - Lo) / Lo) <= RTOL
    usub = np.concatenate([u[off[i]:off[i + 1]] for i in idx])
    s = o.s_at(sub.n_samples, usub)
    Lr = np.repeat(Lo, sub.n_samples)
    assert np.max(np.abs(s - sub.sample_positions() * Lr) / Lr) <= RTOL


@pytest.mark.parametrize("learned", [False, True])
def test_half_warp_mapping_builds_the_same_table(learned, gpu_lib):
    # one half-warp per knot interval (GCV_MAP_HALF_WARP) against one lane per
    # interval: the same panels and leaves; the nodes of each panel are summed
    # in another order, so values agree to float-float rounding
    b = ds.uneven_batch(1500, seed=33, max_ctrl=300, max_samples=64)
    pos = b.sample_positions()
    out = {}
    for mapping in ("lane", "half_warp"):
        calc = g.ArclengthCalculateGpu.from_batch(b, precision=g.GCV_MIXED, rtol=b.rtol, learned=learned,
                                                  mapping=mapping, collect_stats=True)
        if learned:
            from gcurval_gb300 import learned as lm
            calc.set_learned_model(lm.load_model())
        calc.createArclengthTable()
        L = calc.getAllCurveArclengths()
        u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST).us
        st = calc.stats()
        calc.close()
        out[mapping] = (L, u, st["n_panels"], st["n_leaves"])
    (L0, u0, p0, l0), (L1, u1, p1, l1) = out["lane"], out["half_warp"]
    assert abs(p1 - p0) <= 1e-3 * p0 and abs(l1 - l0) <= 1e-3 * l0
    assert np.max(np.abs(L1 - L0) / L0) <= 1e-12
    assert np.max(np.abs(u1 - u0)) <= 1e-11
