"""The seeded workload generators: shapes, invariants and determinism."""
import numpy as np
import pytest

from gcurval_gb300 import datasets as ds


def _curve_knots(b, c):
    return b.knots[b.knot_off[c]:b.knot_off[c + 1]]


def test_uniform_bsplines_shape():
    b = ds.uniform_bsplines(50, n_ctrl=64, degree=3, dim=2, n_samples=1024, seed=0)
    assert b.n_curve == 50 and np.all(b.n_segments == 61)
    assert b.ctrl.size == 50 * 64 * 2 and b.total_samples == 50 * 1024
    kv = _curve_knots(b, 0)
    assert kv.size == 68 and np.all(kv[:4] == 0) and np.all(kv[-4:] == 1) and np.all(np.diff(kv) > -1e-300)
    assert np.all(b.ctrl[:2] == 0.0)  # the walk starts at the origin


def test_ellipses_shape_and_ranges():
    b = ds.ellipses(100, seed=0)
    prm = b.ctrl.reshape(-1, 5)
    assert np.all((prm[:, :2] >= 0.1) & (prm[:, :2] <= 10))
    assert np.all((prm[:, 2] >= 0) & (prm[:, 2] < 2 * np.pi))
    assert np.all(np.abs(prm[:, 3:]) <= 100)
    assert np.all(b.n_segments == 1)


def test_mixed3d_ranges():
    b = ds.mixed3d_bsplines(2000, n_samples=8, seed=1)
    assert set(np.unique(b.degree)) == {3, 5}
    n_ctrl = (np.diff(b.knot_off) - b.degree - 1)
    assert n_ctrl.min() >= 32 and n_ctrl.max() <= 256 and np.all(b.dim == 3)
    for c in range(0, 2000, 37):
        kv = _curve_knots(b, c)
        assert np.all(np.diff(kv) >= 0) and kv[0] == 0 and kv[-1] == 1


def test_uneven_batch_mix_and_near_duplicates():
    b = ds.uneven_batch(5000, seed=2)
    ell = b.kind == 0
    assert 0.15 < ell.mean() < 0.25
    bs = ~ell
    assert set(np.unique(b.degree[bs])) == {2, 3, 4, 5} and set(np.unique(b.dim[bs])) == {2, 3}
    n_ctrl = np.diff(b.knot_off)[bs] - b.degree[bs] - 1
    assert n_ctrl.min() >= 3 and n_ctrl.max() <= 4096
    assert b.n_samples.min() >= 16 and b.n_samples.max() <= 8192
    gaps = []
    for c in np.nonzero(bs)[0][:400]:
        kv = _curve_knots(b, c)
        d = np.diff(kv)
        assert np.all(d >= 0)
        gaps.append(np.sum(np.isclose(d, 1e-6, rtol=1e-3, atol=0)))
    assert sum(gaps) > 0  # near-duplicate knots (gap 1e-6) are present


def test_generators_are_deterministic():
    a = ds.uneven_batch(300, seed=9)
    b = ds.uneven_batch(300, seed=9)
    np.testing.assert_array_equal(a.knots, b.knots)
    np.testing.assert_array_equal(a.ctrl, b.ctrl)


@pytest.mark.parametrize("counts", [[1, 2, 5, 0, 3], [0, 0], [7]])
def test_uniform_positions(counts):
    pos = ds.uniform_positions(np.array(counts))
    off = np.concatenate([[0], np.cumsum(counts)])
    for i, n in enumerate(counts):
        seg = pos[off[i]:off[i + 1]]
        if n == 1:
            assert seg[0] == 0.0
        elif n > 1:
            np.testing.assert_allclose(seg, np.linspace(0, 1, n), atol=1e-15)


def test_subset_roundtrip():
    b = ds.uneven_batch(200, seed=4)
    b.sample_positions()
    s = b.subset([5, 0, 17])
    assert s.n_curve == 3
    np.testing.assert_array_equal(_curve_knots(s, 0), _curve_knots(b, 5))
    np.testing.assert_array_equal(s.ctrl[s.ctrl_off[2]:s.ctrl_off[3]], b.ctrl[b.ctrl_off[17]:b.ctrl_off[18]])
