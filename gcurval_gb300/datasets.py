"""Seeded synthetic curve batches (the five workloads the library is measured on).

The reference ships no benchmark inputs besides its text B-spline bundle; these
generators produce curves with the shapes, sizes and value distributions of the
five measured workloads, from ``numpy.random.default_rng(seed)``:

* ``ellipses``          4,096 2D ellipses, a, b ~ U[0.1, 10], rotation
                        ~ U[0, 2 pi), centre ~ U[-100, 100]^2, one interval
                        t in [0, 2 pi]; 1,000 uniformly spaced samples.
* ``uniform_bsplines``  10,000 clamped uniform cubic 2D B-splines, 64 control
                        points as a random walk with N(0, 1) steps per axis
                        (61 knot intervals); 1,024 samples.
* ``mixed3d_bsplines``  100,000 clamped 3D B-splines, degree 3 or 5, 32-256
                        control points, interior knots sorted U[0, 1] draws,
                        N(0, 0.5) random-walk steps; 2,048 samples.
* ``uneven_batch``      1,000,000 curves: 20 % ellipses, 80 % 2D/3D B-splines of
                        degree 2-5 with log-uniform 4-4,096 control points and 5 %
                        near-duplicate interior knots (gap 1e-6); log-uniform
                        16-8,192 samples per curve.

The batch layout is the one the C ABI takes (``gcv_create_batch`` in
include/gcurval_gb300.h): per-curve kind / degree / dim, CSR offsets into one
knot array and one control array.  Ellipses store ``a, b, rotation, cx, cy`` as
their control data and the knot vector ``{0, 2 pi}``.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

KIND_ELLIPSE = 0
KIND_BSPLINE = 1
TWO_PI = 2.0 * math.pi


@dataclasses.dataclass
class CurveBatch:
    kind: np.ndarray  # uint8[n]
    degree: np.ndarray  # uint8[n]
    dim: np.ndarray  # uint8[n]
    knot_off: np.ndarray  # int64[n + 1]
    knots: np.ndarray  # float64
    ctrl_off: np.ndarray  # int64[n + 1] (in doubles)
    ctrl: np.ndarray  # float64
    n_samples: np.ndarray  # int32[n]
    positions: np.ndarray | None = None  # float64[sum(n_samples)], relative
    name: str = ""
    rtol: float = 1e-10

    @property
    def n_curve(self) -> int:
        return int(self.kind.shape[0])

    @property
    def n_segments(self) -> np.ndarray:
        nk = np.diff(self.knot_off)
        p = self.degree.astype(np.int64)
        return np.where(self.kind == KIND_ELLIPSE, nk - 1, nk - 2 * p - 1)

    @property
    def total_samples(self) -> int:
        return int(self.n_samples.astype(np.int64).sum())

    def sample_positions(self) -> np.ndarray:
        """Uniformly spaced relative positions j / (n - 1) for every curve."""
        if self.positions is None:
            self.positions = uniform_positions(self.n_samples)
        return self.positions

    def subset(self, idx) -> "CurveBatch":
        """A new batch holding curves ``idx`` (in that order)."""
        idx = np.asarray(idx, dtype=np.int64)
        kl = np.diff(self.knot_off)[idx]
        cl = np.diff(self.ctrl_off)[idx]
        ko = np.concatenate([[0], np.cumsum(kl)]).astype(np.int64)
        co = np.concatenate([[0], np.cumsum(cl)]).astype(np.int64)
        knots = np.concatenate([self.knots[self.knot_off[i]:self.knot_off[i + 1]] for i in idx]) if len(idx) else np.zeros(0)
        ctrl = np.concatenate([self.ctrl[self.ctrl_off[i]:self.ctrl_off[i + 1]] for i in idx]) if len(idx) else np.zeros(0)
        ns = self.n_samples[idx].copy()
        pos = None
        if self.positions is not None:
            so = np.concatenate([[0], np.cumsum(self.n_samples.astype(np.int64))])
            pos = np.concatenate([self.positions[so[i]:so[i + 1]] for i in idx]) if len(idx) else np.zeros(0)
        return CurveBatch(self.kind[idx].copy(), self.degree[idx].copy(), self.dim[idx].copy(), ko,
                          np.ascontiguousarray(knots, dtype=np.float64), co,
                          np.ascontiguousarray(ctrl, dtype=np.float64), ns, pos, self.name, self.rtol)

    def nbytes(self) -> int:
        return sum(a.nbytes for a in (self.kind, self.degree, self.dim, self.knot_off, self.knots,
                                      self.ctrl_off, self.ctrl))


def uniform_positions(n_samples: np.ndarray) -> np.ndarray:
    """Relative positions j / (n - 1), j = 0..n-1, for each curve (0 when n == 1)."""
    n_samples = np.asarray(n_samples, dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(n_samples)])
    out = np.empty(int(off[-1]))
    step = 1 << 16
    for i in range(0, n_samples.size, step):
        ns = n_samples[i:i + step]
        lo, hi = int(off[i]), int(off[min(i + step, n_samples.size)])
        j = np.arange(hi - lo, dtype=np.float64) - np.repeat((off[i:i + ns.size] - lo).astype(np.float64), ns)
        out[lo:hi] = j / np.repeat(np.maximum(ns - 1, 1).astype(np.float64), ns)
    return out


def _pack(kind, degree, dim, knot_lists_len, knots, ctrl_len, ctrl, n_samples, name, rtol):
    knot_off = np.concatenate([[0], np.cumsum(knot_lists_len)]).astype(np.int64)
    ctrl_off = np.concatenate([[0], np.cumsum(ctrl_len)]).astype(np.int64)
    return CurveBatch(np.asarray(kind, np.uint8), np.asarray(degree, np.uint8), np.asarray(dim, np.uint8),
                      knot_off, np.ascontiguousarray(knots, np.float64), ctrl_off,
                      np.ascontiguousarray(ctrl, np.float64), np.asarray(n_samples, np.int32), None, name, rtol)


def _ellipse_params(rng, n):
    a = rng.uniform(0.1, 10.0, n)
    b = rng.uniform(0.1, 10.0, n)
    rot = rng.uniform(0.0, TWO_PI, n)
    cx = rng.uniform(-100.0, 100.0, n)
    cy = rng.uniform(-100.0, 100.0, n)
    return np.stack([a, b, rot, cx, cy], axis=1)


def ellipses(n: int = 4096, n_samples: int = 1000, seed: int = 0, rtol: float = 1e-10) -> CurveBatch:
    rng = np.random.default_rng(seed)
    prm = _ellipse_params(rng, n)
    knots = np.tile(np.array([0.0, TWO_PI]), n)
    return _pack(np.zeros(n), np.zeros(n), np.full(n, 2), np.full(n, 2), knots, np.full(n, 5),
                 prm.reshape(-1), np.full(n, n_samples), "ellipses", rtol)


def ellipses_from_axes(a, b, rot=None, cx=None, cy=None, n_samples=0) -> CurveBatch:
    a = np.asarray(a, np.float64)
    n = a.shape[0]
    z = np.zeros(n)
    prm = np.stack([a, np.asarray(b, np.float64), z if rot is None else np.asarray(rot, np.float64),
                    z if cx is None else np.asarray(cx, np.float64), z if cy is None else np.asarray(cy, np.float64)], 1)
    return _pack(np.zeros(n), np.zeros(n), np.full(n, 2), np.full(n, 2), np.tile([0.0, TWO_PI], n),
                 np.full(n, 5), prm.reshape(-1), np.full(n, n_samples), "ellipses", 1e-10)


def clamped_uniform_knots(n_ctrl: int, degree: int) -> np.ndarray:
    n_int = n_ctrl - degree - 1
    inner = np.arange(1, n_int + 1, dtype=np.float64) / (n_int + 1)
    return np.concatenate([np.zeros(degree + 1), inner, np.ones(degree + 1)])


def uniform_bsplines(n: int = 10000, n_ctrl: int = 64, degree: int = 3, dim: int = 2, n_samples: int = 1024,
                     seed: int = 0, step_sigma: float = 1.0, rtol: float = 1e-10) -> CurveBatch:
    rng = np.random.default_rng(seed)
    steps = rng.normal(0.0, step_sigma, size=(n, n_ctrl - 1, dim))
    pts = np.concatenate([np.zeros((n, 1, dim)), np.cumsum(steps, axis=1)], axis=1)
    kv = clamped_uniform_knots(n_ctrl, degree)
    knots = np.tile(kv, n)
    return _pack(np.ones(n), np.full(n, degree), np.full(n, dim), np.full(n, kv.size), knots,
                 np.full(n, n_ctrl * dim), pts.reshape(-1), np.full(n, n_samples), "uniform_bsplines", rtol)


def _segmented_sorted_uniform(rng, counts: np.ndarray) -> np.ndarray:
    """For each count m, m sorted U(0,1) draws (via normalised exponential spacings), flat."""
    counts = np.asarray(counts, np.int64)
    tot = int((counts + 1).sum())
    e = rng.exponential(1.0, tot)
    seg = np.repeat(np.arange(counts.size), counts + 1)
    cs = np.cumsum(e)
    starts = np.concatenate([[0], np.cumsum(counts + 1)])
    base = np.concatenate([[0.0], cs])[starts[:-1]]
    local = cs - base[seg]
    total = local[starts[1:] - 1]
    val = local / total[seg]
    keep = np.ones(tot, bool)
    keep[starts[1:] - 1] = False  # drop the last (== 1) of each group
    return val[keep]


def _ragged_index(starts, lengths):
    """Flat indices starts[i] + 0..lengths[i]-1 for every i, concatenated."""
    lengths = np.asarray(lengths, np.int64)
    tot = int(lengths.sum())
    if tot == 0:
        return np.zeros(0, np.int64)
    first = np.concatenate([[0], np.cumsum(lengths)[:-1]])
    return np.repeat(np.asarray(starts, np.int64) - first, lengths) + np.arange(tot, dtype=np.int64)


_CHUNK = 1 << 16


def _bspline_chunk(rng, degree, dim, n_ctrl, step_sigma, dup_frac, dup_gap):
    n_int = n_ctrl - degree - 1
    inner = _segmented_sorted_uniform(rng, n_int)
    io = np.concatenate([[0], np.cumsum(n_int)])
    if dup_frac > 0.0 and inner.size:
        # a fraction of the interior knots become previous + gap (near-duplicate
        # knots); min() with the next knot keeps every curve's interior sorted
        has = n_int > 0
        first = np.zeros(inner.size, bool)
        first[io[:-1][has]] = True
        nxt = np.append(inner[1:], 1.0)
        nxt[io[1:][has] - 1] = 1.0
        pick = np.nonzero((rng.random(inner.size) < dup_frac) & ~first)[0]
        inner[pick] = np.minimum(inner[pick - 1] + dup_gap, nxt[pick])
    n_knots = n_ctrl + degree + 1
    ko = np.concatenate([[0], np.cumsum(n_knots)])
    knots = np.ones(int(ko[-1]))
    knots[_ragged_index(ko[:-1], degree + 1)] = 0.0
    knots[_ragged_index(ko[:-1] + degree + 1, n_int)] = inner
    # control points: random walk from the origin, one (x, y, z) row per point,
    # z dropped for 2D curves
    po = np.concatenate([[0], np.cumsum(n_ctrl)])
    steps = rng.normal(0.0, step_sigma, (int(po[-1]), 3))
    steps[po[:-1]] = 0.0
    cs = np.cumsum(steps, axis=0)
    cs -= np.repeat(cs[po[:-1]], n_ctrl, axis=0)
    keep = np.arange(3)[None, :] < np.repeat(dim, n_ctrl)[:, None]
    return n_knots, knots, n_ctrl * dim, cs[keep]


def _random_knot_bsplines(rng, degree, dim, n_ctrl, step_sigma, dup_frac=0.0, dup_gap=1e-6):
    """Clamped B-splines with sorted-uniform interior knots and random-walk control
    points; per-curve degree / dim / n_ctrl arrays.  Linear time, in chunks of
    curves, so that a million curves with hundreds of millions of knots fit."""
    degree = np.asarray(degree, np.int64)
    dim = np.asarray(dim, np.int64)
    n_ctrl = np.asarray(n_ctrl, np.int64)
    parts = [_bspline_chunk(rng, degree[i:i + _CHUNK], dim[i:i + _CHUNK], n_ctrl[i:i + _CHUNK], step_sigma,
                            dup_frac, dup_gap) for i in range(0, degree.size, _CHUNK)]
    if not parts:
        return np.zeros(0, np.int64), np.zeros(0), np.zeros(0, np.int64), np.zeros(0)
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(4))


def mixed3d_bsplines(n: int = 100_000, n_samples: int = 2048, seed: int = 0, rtol: float = 1e-8) -> CurveBatch:
    rng = np.random.default_rng(seed)
    degree = np.where(rng.random(n) < 0.5, 3, 5).astype(np.int64)
    n_ctrl = rng.integers(32, 257, n).astype(np.int64)
    dim = np.full(n, 3, np.int64)
    n_knots, knots, clen, ctrl = _random_knot_bsplines(rng, degree, dim, n_ctrl, 0.5)
    return _pack(np.ones(n), degree, dim, n_knots, knots, clen, ctrl, np.full(n, n_samples),
                 "mixed3d_bsplines", rtol)


def _log_uniform_int(rng, lo, hi, n):
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi + 1), n))).astype(np.int64).clip(lo, hi)


def uneven_batch(n: int = 1_000_000, seed: int = 0, rtol: float = 5e-9,
                 max_ctrl: int = 4096, min_samples: int = 16, max_samples: int = 8192) -> CurveBatch:
    """The uneven batch: 20% ellipses, 80% B-splines of degree 2-5 in 2D / 3D
    with log-uniform 4-4,096 control points and 5% near-duplicate knots (gap
    1e-6), log-uniform 16-8,192 samples per curve.  Its accuracy target is
    1e-8 relative error of lengths and sample positions against the FP64
    oracle; the per-interval tolerance it carries is half of that, because
    at 1e-8 itself the sample positions of a few curves with sharp speed
    dips (a factor of 10^4 inside one knot interval) land at up to 1.1e-8."""
    rng = np.random.default_rng(seed)
    is_ell = rng.random(n) < 0.2
    ne = int(is_ell.sum())
    nb = n - ne
    degree = rng.integers(2, 6, nb).astype(np.int64)
    dim = rng.integers(2, 4, nb).astype(np.int64)
    n_ctrl = np.maximum(_log_uniform_int(rng, 4, max_ctrl, nb), degree + 1)
    prm = _ellipse_params(rng, ne)
    n_samp = _log_uniform_int(rng, min_samples, max_samples, n)
    kind = np.where(is_ell, KIND_ELLIPSE, KIND_BSPLINE)
    deg = np.zeros(n, np.int64)
    dm = np.full(n, 2, np.int64)
    deg[~is_ell] = degree
    dm[~is_ell] = dim
    nc = np.zeros(n, np.int64)
    nc[~is_ell] = n_ctrl
    ell_prm = np.zeros((n, 5))
    ell_prm[is_ell] = prm
    klen = np.where(is_ell, 2, nc + deg + 1)
    clen = np.where(is_ell, 5, nc * dm)
    # B-spline data in chunks of curves, interleaved with the ellipses in curve order
    knots_parts, ctrl_parts = [], []
    for i in range(0, n, _CHUNK):
        sl = slice(i, min(i + _CHUNK, n))
        e = is_ell[sl]
        b = ~e
        nk, kb, cl, cb = _bspline_chunk(rng, deg[sl][b], dm[sl][b], nc[sl][b], 1.0, 0.05, 1e-6)
        ko = np.concatenate([[0], np.cumsum(klen[sl])])
        co = np.concatenate([[0], np.cumsum(clen[sl])])
        kn = np.empty(int(ko[-1]))
        ct = np.empty(int(co[-1]))
        kn[_ragged_index(ko[:-1][b], nk)] = kb
        ct[_ragged_index(co[:-1][b], cl)] = cb
        ei = np.nonzero(e)[0]
        kn[ko[ei]] = 0.0
        kn[ko[ei] + 1] = TWO_PI
        ct[_ragged_index(co[ei], np.full(ei.size, 5))] = ell_prm[sl][e].reshape(-1)
        knots_parts.append(kn)
        ctrl_parts.append(ct)
    knots = np.concatenate(knots_parts) if knots_parts else np.zeros(0)
    ctrl = np.concatenate(ctrl_parts) if ctrl_parts else np.zeros(0)
    return _pack(kind, deg, dm, klen, knots, clen, ctrl, n_samp, "uneven_batch", rtol)


# ------------------------------------------------------------ subsets
def cost_proxy(batch: CurveBatch) -> np.ndarray:
    """A per-curve work estimate for stratified sampling: knot intervals
    (weighted as the tens of integrand evaluations each costs) plus samples."""
    return 32.0 * batch.n_segments.astype(np.float64) + batch.n_samples.astype(np.float64)


def stratified_indices(batch: CurveBatch, n: int) -> np.ndarray:
    """n curves spread evenly over the batch sorted by cost_proxy (a
    systematic sample of the cost distribution: its mean cost matches the
    batch's far more closely than a uniform sample of the same size when
    costs are heavy-tailed).  Sorted by descending cost."""
    n = int(min(max(n, 0), batch.n_curve))
    if n == 0:
        return np.zeros(0, np.int64)
    cost = cost_proxy(batch)
    order = np.argsort(cost, kind="stable")
    pick = order[((np.arange(n) + 0.5) * batch.n_curve / n).astype(np.int64)]
    return pick[np.argsort(-cost[pick], kind="stable")]


def near_duplicate_knots(batch: CurveBatch, gap: float = 1e-5) -> np.ndarray:
    """Per curve, the number of consecutive knot pairs closer than `gap`
    but not equal (the uneven batch's near-duplicate knots)."""
    d = np.diff(batch.knots)
    close = (d > 0.0) & (d < gap)
    # pairs that cross a curve boundary do not count
    ends = batch.knot_off[1:-1] - 1
    close[ends[(ends >= 0) & (ends < close.size)]] = False
    cnt = np.zeros(batch.n_curve, np.int64)
    if close.size:
        owner = np.searchsorted(batch.knot_off, np.nonzero(close)[0], side="right") - 1
        np.add.at(cnt, owner, 1)
    return cnt


def hard_case_indices(batch: CurveBatch, k: int = 200, seed: int = 0) -> np.ndarray:
    """The curves where accuracy is hardest to hold, for the accuracy checks:
    the k with the most near-duplicate knots, the k degree-5 curves with the
    most near-duplicate knots, the k with the most knot intervals, the k with
    the most samples, and k / 10 random curves of every curve code."""
    rng = np.random.default_rng(seed)
    dup = near_duplicate_knots(batch)
    nseg = batch.n_segments
    parts = [np.argsort(-dup, kind="stable")[:k]]
    d5 = np.nonzero((batch.kind == KIND_BSPLINE) & (batch.degree == 5))[0]
    parts.append(d5[np.argsort(-dup[d5], kind="stable")[:k]])
    parts.append(np.argsort(-nseg, kind="stable")[:k])
    parts.append(np.argsort(-batch.n_samples.astype(np.int64), kind="stable")[:k])
    code = np.where(batch.kind == KIND_ELLIPSE, -1, batch.degree.astype(np.int64) * 10 + batch.dim)
    for c in np.unique(code):
        idx = np.nonzero(code == c)[0]
        parts.append(rng.choice(idx, size=min(idx.size, max(1, k // 10)), replace=False))
    return np.unique(np.concatenate(parts))


def accuracy_subset_indices(batch: CurveBatch, n_stratified: int = 1000, k_hard: int = 250) -> np.ndarray:
    """A stratified sample of the batch plus its hard cases (sorted indices)."""
    return np.union1d(stratified_indices(batch, n_stratified), hard_case_indices(batch, k_hard))


def control_polygon_length(batch: CurveBatch) -> np.ndarray:
    """Per curve, the length of the control polygon (B-splines; an upper
    bound of the curve's length) or 2 pi max(a, b) (ellipses)."""
    out = np.zeros(batch.n_curve)
    ell = np.nonzero(batch.kind == KIND_ELLIPSE)[0]
    if ell.size:
        a = batch.ctrl[batch.ctrl_off[ell]]
        b = batch.ctrl[batch.ctrl_off[ell] + 1]
        out[ell] = TWO_PI * np.maximum(np.abs(a), np.abs(b))
    for d in (2, 3):
        sel = np.nonzero((batch.kind == KIND_BSPLINE) & (batch.dim == d))[0]
        if not sel.size:
            continue
        npts = (batch.ctrl_off[sel + 1] - batch.ctrl_off[sel]) // d
        idx = _ragged_index(batch.ctrl_off[sel], npts * d)
        pts = batch.ctrl[idx].reshape(-1, d)
        seg = np.linalg.norm(np.diff(pts, axis=0), axis=1)
        first = np.concatenate([[0], np.cumsum(npts)[:-1]])
        # drop the steps that join consecutive curves
        keep = np.ones(seg.size, bool)
        keep[(first[1:] - 1)] = False
        owner = np.repeat(np.arange(sel.size), npts)[1:]
        tot = np.zeros(sel.size)
        np.add.at(tot, owner[keep], seg[keep])
        out[sel] = tot
    return out


WORKLOADS = {
    "ellipses": ellipses,
    "uniform_bsplines": uniform_bsplines,
    "mixed3d_bsplines": mixed3d_bsplines,
    "uneven_batch": uneven_batch,
}


def reference_layout(batch: CurveBatch):
    """(degree, dim, knots_offset int32[n+1], knots, ctrl) for a batch of B-splines that share
    one degree and dimension: the layout of the reference's B-spline sample
    (samples/sample2_bspline/arclength_calculate.h:505-518)."""
    assert np.all(batch.kind == KIND_BSPLINE)
    p = int(batch.degree[0])
    d = int(batch.dim[0])
    assert np.all(batch.degree == p) and np.all(batch.dim == d)
    return p, d, batch.knot_off.astype(np.int32), batch.knots, batch.ctrl
