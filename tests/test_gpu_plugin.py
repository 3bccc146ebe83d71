"""The header-only plugin path (include/gcurval_gb300/gcurval.cuh): user-defined
curve families through the reference's ArclengthCalculateGpu<Curve, CurveTraits>
API, built by nvcc from tests/plugin/plugin_driver.cu and checked against the
oracle (lengths, sample positions, points), with the default Gauss-Kronrod
rule and with the reference's point-based rules (Polyline, Simpson,
Vincent-Forsey) selected through CurveTraits::CalculateFunction."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from gcurval_gb300 import datasets as ds
from oracle import oracle as orc
from oracle import point_rules as pr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="session")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path_factory.mktemp("plugin") / "plugin_driver")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           "-o", exe, os.path.join(ROOT, "tests", "plugin", "plugin_driver.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(driver, tmp_path, family, payload, n, total, what, rtol=None):
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        f.write(np.array([n, what], np.int32).tobytes())
        for a in payload:
            f.write(np.ascontiguousarray(a).tobytes())
    args = [driver, family, fin, fout] + ([repr(rtol)] if rtol is not None else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(fout, np.float64)
    L = out[:n]
    rest = out[n:]
    return L, (rest if what == 0 else rest.reshape(total, 2))


def sample_err(o, batch, u, L):
    s = o.s_at(batch.n_samples, u)
    tgt = batch.positions * np.repeat(L, batch.n_samples)
    return np.max(np.abs(s - tgt) / np.repeat(L, batch.n_samples))


def ellipse_payload(b):
    prm = b.ctrl.reshape(-1, 5)
    return [prm[:, 0].copy(), prm[:, 1].copy(), b.n_samples.astype(np.int32), b.positions]


def test_plugin_ellipses_lengths_and_samples(driver, tmp_path):
    b = ds.ellipses(300, n_samples=33, seed=5)
    b.sample_positions()
    L, u = run(driver, tmp_path, "ellipse", ellipse_payload(b), b.n_curve, b.total_samples, 0)
    o = orc.Oracle(b)
    Lo = o.lengths()
    assert np.max(np.abs(L - Lo) / Lo) <= 1e-10
    assert sample_err(o, b, u, Lo) <= 1e-10
    assert np.all((u >= 0) & (u <= 2 * np.pi))


def test_plugin_ellipse_points(driver, tmp_path):
    b = ds.ellipses(40, n_samples=9, seed=6)
    b.sample_positions()
    _, u = run(driver, tmp_path, "ellipse", ellipse_payload(b), b.n_curve, b.total_samples, 0)
    _, pts = run(driver, tmp_path, "ellipse", ellipse_payload(b), b.n_curve, b.total_samples, 1)
    prm = np.repeat(b.ctrl.reshape(-1, 5), b.n_samples, axis=0)
    exp = np.stack([prm[:, 0] * np.cos(u), prm[:, 1] * np.sin(u)], axis=1)
    np.testing.assert_allclose(pts, exp, rtol=0, atol=1e-12 * np.max(np.abs(exp)))


def bspline_payload(b):
    return [b.knot_off.astype(np.int32), b.knots, b.ctrl, b.n_samples.astype(np.int32), b.positions]


def ragged_cubic_2d(n, seed):
    """Cubic planar B-splines with 4-40 control points and clamped knots whose
    interior values are sorted uniform draws (ragged interval counts)."""
    rng = np.random.default_rng(seed)
    knots, ctrl, klen, clen = [], [], [], []
    for _ in range(n):
        m = int(rng.integers(4, 41))
        inner = np.sort(rng.random(m - 4))
        kv = np.concatenate([np.zeros(4), inner, np.ones(4)])
        pts = np.cumsum(rng.normal(size=(m, 2)) ** 2, axis=0)
        knots.append(kv)
        ctrl.append(pts.reshape(-1))
        klen.append(kv.size)
        clen.append(pts.size)
    ko = np.concatenate([[0], np.cumsum(klen)]).astype(np.int64)
    co = np.concatenate([[0], np.cumsum(clen)]).astype(np.int64)
    ns = rng.integers(0, 50, n).astype(np.int32)
    return ds.CurveBatch(np.ones(n, np.uint8), np.full(n, 3, np.uint8), np.full(n, 2, np.uint8), ko,
                         np.concatenate(knots), co, np.concatenate(ctrl), ns, None, "ragged", 1e-10)


@pytest.mark.parametrize("maker", ["uniform", "ragged"])
def test_plugin_bsplines_through_shared_memory_hook(driver, tmp_path, maker):
    b = ds.uniform_bsplines(200, n_ctrl=24, n_samples=17, seed=7) if maker == "uniform" else ragged_cubic_2d(150, 8)
    b.sample_positions()
    L, u = run(driver, tmp_path, "bspline", bspline_payload(b), b.n_curve, b.total_samples, 0)
    o = orc.Oracle(b)
    Lo = o.lengths()
    assert np.max(np.abs(L - Lo) / Lo) <= 1e-10
    assert sample_err(o, b, u, Lo) <= 1e-10
    _, pts = run(driver, tmp_path, "bspline", bspline_payload(b), b.n_curve, b.total_samples, 1)
    cid = np.repeat(np.arange(b.n_curve), b.n_samples)
    for i in range(0, b.total_samples, max(1, b.total_samples // 60)):
        np.testing.assert_allclose(pts[i], o.point(int(cid[i]), float(u[i]))[:2], rtol=1e-12, atol=1e-12)


# ---------------------------------------------------------- point-based rules
RULES = {"polyline": pr.POLYLINE, "simpson": pr.SIMPSON, "vf": pr.VINCENT_FORSEY}
# the polyline converges at third order only: a looser tolerance keeps its tables small
RULE_RTOL = {"polyline": 1e-6, "simpson": 1e-9, "vf": 1e-10}


@pytest.mark.parametrize("rule", sorted(RULES))
def test_plugin_point_rules_ellipses(driver, tmp_path, rule):
    b = ds.ellipses(60, n_samples=17, seed=9)
    b.sample_positions()
    rtol = RULE_RTOL[rule]
    L, u = run(driver, tmp_path, "ellipse_" + rule, ellipse_payload(b), b.n_curve, b.total_samples, 0, rtol)
    o = orc.Oracle(b)
    Lo = o.lengths()
    assert np.max(np.abs(L - Lo) / Lo) <= 2 * rtol
    assert sample_err(o, b, u, Lo) <= 3 * rtol


@pytest.mark.parametrize("rule", sorted(RULES))
def test_plugin_point_rules_bsplines_through_shared_memory_hook(driver, tmp_path, rule):
    b = ragged_cubic_2d(80, 12)
    b.sample_positions()
    rtol = RULE_RTOL[rule]
    L, u = run(driver, tmp_path, "bspline_" + rule, bspline_payload(b), b.n_curve, b.total_samples, 0, rtol)
    o = orc.Oracle(b)
    Lo = o.lengths()
    assert np.max(np.abs(L - Lo) / Lo) <= 2 * rtol
    assert sample_err(o, b, u, Lo) <= 3 * rtol
    _, pts = run(driver, tmp_path, "bspline_" + rule, bspline_payload(b), b.n_curve, b.total_samples, 1, rtol)
    cid = np.repeat(np.arange(b.n_curve), b.n_samples)
    for i in range(0, b.total_samples, max(1, b.total_samples // 40)):
        np.testing.assert_allclose(pts[i], o.point(int(cid[i]), float(u[i]))[:2], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("rule", sorted(RULES))
def test_plugin_point_rule_values_match_the_oracle(driver, tmp_path, rule):
    """With an unbounded tolerance the walk accepts its 64 starting pieces
    per interval at once, so a curve's length is the sum over each interval's
    128 equal sub-panels of the rule: the rule formulas themselves, against
    the oracle."""
    kind = RULES[rule]

    def pieces(pt, t0, t1):
        t = t0 + (t1 - t0) * np.arange(129) / 128.0
        return sum(pr.rule_on(kind, pt, a, b) for a, b in zip(t[:-1], t[1:]))

    e = ds.ellipses(12, n_samples=2, seed=4)
    e.sample_positions()
    L, _ = run(driver, tmp_path, "ellipse_" + rule, ellipse_payload(e), e.n_curve, e.total_samples, 0, 1e300)
    prm = e.ctrl.reshape(-1, 5)
    for c in range(e.n_curve):
        pt = lambda t, a=prm[c, 0], bb=prm[c, 1]: np.array([a * np.cos(t), bb * np.sin(t)])
        assert L[c] == pytest.approx(pieces(pt, 0.0, 2 * np.pi), rel=1e-12)
    b = ragged_cubic_2d(10, 13)
    b.sample_positions()
    L, _ = run(driver, tmp_path, "bspline_" + rule, bspline_payload(b), b.n_curve, b.total_samples, 0, 1e300)
    o = orc.Oracle(b)
    for c in range(b.n_curve):
        kv = b.knots[b.knot_off[c]:b.knot_off[c + 1]]
        pt = lambda t, c=c: np.asarray(o.point(c, float(t)))[:2]
        exp = sum(pieces(pt, t0, t1) for t0, t1 in zip(kv[3:-4], kv[4:-3]) if t1 > t0)
        assert L[c] == pytest.approx(exp, rel=1e-12)
