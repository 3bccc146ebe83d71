"""Generates the golden fixtures in this folder from the reference's own CPU
driver (gcurval::ArclengthCalculateCpu, compiled from the reference tree by
oracle/Makefile into oracle/_ref/libgcv_ref.so).

    python tests/golden/make_golden.py [case ...]

Each ``<case>.npz`` holds the curve batch (CurveBatch arrays), the sample
counts and positions, and the reference's outputs: total lengths
(getAllCurveArclengths), sample parameters and points (arclengthReverse with
gcurvalHost / gcurvalReverseReturnUs and ...Points), at the reference's
default FP64 configuration (MAX_ERROR 1e-14, depth 23).

``bundle_0.npz`` is real data: the text of the first 300 curve records of
the reference's ``dataset/BSpline/Bundle_0.txt`` (``text``) and the arrays the
reference's own loader makes of them (``load_dataset``,
samples/sample2_bspline/dataset_loader.h:40-126, compiled into
oracle/_ref/libgcv_ref.so): the batch arrays of that fixture ARE the
reference loader's output.

``point_rules.npz`` holds the values of the reference's own point-based rule
functors (PolylineMethod, SimpsonMethod, VincentForseyRule,
gcurval/base/functors.inl.h:145-238) on seeded intervals of ellipses and of
cubic 2D B-splines, through the sample plugins' GetPoint.

The reference tree is needed only here; tests read the committed files.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gcurval_gb300 import bundle  # noqa: E402
from gcurval_gb300 import datasets as ds  # noqa: E402
from oracle.oracle import (REF_TREE, Reference, reference_available, reference_load_bundle,  # noqa: E402
                           reference_rule_values)

BUNDLE_CURVES = 300


def _positions(rng, n_curve, n_samp):
    """Uniform relative positions plus the edges 0 and 1 for every curve."""
    pos = ds.uniform_positions(np.full(n_curve, n_samp))
    # perturb interior positions so they do not sit on table entries
    jitter = rng.uniform(-0.3, 0.3, pos.shape) / max(n_samp - 1, 1)
    inner = (pos > 0) & (pos < 1)
    pos[inner] = np.clip(pos[inner] + jitter[inner], 0.0, 1.0)
    return pos


def cases():
    rng = np.random.default_rng(20240601)
    out = {}
    # ellipses without rotation / centre (the reference's ellipse has neither)
    a = rng.uniform(0.1, 10.0, 24)
    b = rng.uniform(0.1, 10.0, 24)
    a[0] = b[0] = 1.0  # a circle
    a[1], b[1] = 2.0, 1.0
    e = ds.ellipses_from_axes(a, b, n_samples=17)
    out["ellipses"] = e
    # cubic 2D uniform B-splines (the reference sample's curve type)
    out["bspline_p3_d2"] = ds.uniform_bsplines(12, n_ctrl=14, degree=3, dim=2, n_samples=33, seed=5)
    # other degrees / dims with random interior knots
    for p, d, seed in ((1, 2, 7), (2, 3, 8), (4, 2, 9), (5, 3, 10)):
        nb = 6
        deg = np.full(nb, p)
        dim = np.full(nb, d)
        n_ctrl = rng.integers(p + 2, p + 12, nb)
        n_knots, knots, clen, ctrl = ds._random_knot_bsplines(np.random.default_rng(seed), deg, dim, n_ctrl, 1.0)
        out[f"bspline_p{p}_d{d}"] = ds._pack(np.ones(nb), deg, dim, n_knots, knots, clen, ctrl, np.full(nb, 9),
                                             f"bspline_p{p}_d{d}", 1e-10)
    # real data: the first 300 curves of the reference's own dataset file,
    # read and normalised by the reference's loader
    bundle_file = os.path.join(REF_TREE, "dataset", "BSpline", "Bundle_0.txt")
    if os.path.exists(bundle_file):
        out["bundle_0"] = reference_bundle(bundle_file, BUNDLE_CURVES)
    return out


def bundle_records_text(path: str, n_curve: int) -> bytes:
    """The bytes of the first n_curve records of a Bundle file (records end
    with a blank line)."""
    data = open(path, "rb").read()
    recs = data.split(b"\n\n")
    if len(recs) <= n_curve:
        raise ValueError("the file holds fewer records")
    return b"\n\n".join(recs[:n_curve]) + b"\n\n"


def reference_bundle(path: str, n_curve: int) -> "ds.CurveBatch":
    """A CurveBatch of the reference loader's arrays (cubic, 2D), carrying the
    records' text in ``.text``."""
    ko, kv, cp = reference_load_bundle(path, n_curve)
    n = n_curve
    knot_off = ko.astype(np.int64)
    n_pts = np.diff(knot_off) - 4
    ctrl_off = np.concatenate([[0], np.cumsum(2 * n_pts)]).astype(np.int64)
    b = ds.CurveBatch(np.full(n, ds.KIND_BSPLINE, np.uint8), np.full(n, 3, np.uint8), np.full(n, 2, np.uint8),
                      knot_off, kv, ctrl_off, cp.reshape(-1), np.full(n, 9, np.int32), None, "bundle_0", 1e-10)
    b.text = bundle_records_text(path, n_curve)
    # the host reader must agree with the reference loader bit for bit
    h = bundle.load(path, n_curve=n_curve, samples_per_curve=9)
    assert np.array_equal(h.knots.view(np.uint64), b.knots.view(np.uint64))
    assert np.array_equal(h.ctrl.view(np.uint64), b.ctrl.view(np.uint64))
    return b


def point_rule_cases():
    """Values of the reference's three rule functors on seeded intervals."""
    rng = np.random.default_rng(99)
    out = {}
    n_iv = 40
    # ellipses: intervals anywhere in [0, 2 pi], widths from 1e-4 to 2
    a = rng.uniform(0.1, 10.0, 6)
    b = rng.uniform(0.1, 10.0, 6)
    t0 = rng.uniform(0.0, 2 * np.pi, (6, n_iv))
    w = np.exp(rng.uniform(np.log(1e-4), np.log(2.0), (6, n_iv)))
    out["ell_a"], out["ell_b"], out["ell_begin"], out["ell_end"] = a, b, t0, t0 + w
    for rule in ("polyline", "simpson", "vincent_forsey"):
        out[f"ell_{rule}"] = np.stack([reference_rule_values(rule, t0[i], t0[i] + w[i], ellipse=(a[i], b[i]))
                                       for i in range(6)])
    # cubic 2D B-splines (random interior knots, random-walk points): intervals
    # inside one knot interval each
    bs = ds._pack(np.ones(4), np.full(4, 3), np.full(4, 2),
                  *ds._random_knot_bsplines(np.random.default_rng(3), np.full(4, 3), np.full(4, 2),
                                            np.array([7, 9, 12, 20]), 1.0), np.full(4, 1), "rules", 1e-10)
    out["bs_knot_off"], out["bs_knots"], out["bs_ctrl_off"], out["bs_ctrl"] = \
        bs.knot_off, bs.knots, bs.ctrl_off, bs.ctrl
    segs, begins, ends = [], [], []
    for c in range(4):
        kv = bs.knots[bs.knot_off[c]:bs.knot_off[c + 1]]
        n_ctrl = (bs.ctrl_off[c + 1] - bs.ctrl_off[c]) // 2
        sid = rng.integers(0, n_ctrl - 3, n_iv)
        lo, hi = kv[sid + 3], kv[sid + 4]
        f0 = rng.uniform(0.0, 1.0, n_iv)
        f1 = np.minimum(1.0, f0 + np.exp(rng.uniform(np.log(1e-4), np.log(1.0), n_iv)))
        segs.append(sid)
        begins.append(lo + f0 * (hi - lo))
        ends.append(lo + f1 * (hi - lo))
    out["bs_seg"], out["bs_begin"], out["bs_end"] = np.stack(segs), np.stack(begins), np.stack(ends)
    for rule in ("polyline", "simpson", "vincent_forsey"):
        vals = np.zeros((4, n_iv))
        for c in range(4):
            kv = bs.knots[bs.knot_off[c]:bs.knot_off[c + 1]]
            cp = bs.ctrl[bs.ctrl_off[c]:bs.ctrl_off[c + 1]].reshape(-1, 2)
            for j in range(n_iv):
                vals[c, j] = reference_rule_values(rule, begins[c][j:j + 1], ends[c][j:j + 1],
                                                   bspline=(kv, cp, int(segs[c][j])))[0]
        out[f"bs_{rule}"] = vals
    return out


def main(names=None):
    """Regenerates every fixture, or only the named ones (the random stream
    of the positions is the same either way)."""
    if not reference_available():
        sys.exit("the reference tree is needed to regenerate the golden fixtures")
    rng = np.random.default_rng(7)
    for name, batch in cases().items():
        pos = _positions(rng, batch.n_curve, int(batch.n_samples[0]))
        if names and name not in names:
            continue
        batch.positions = pos
        ref = Reference(batch)
        lengths, us = ref.run(batch.n_samples, pos, True, 0)
        _, pts = ref.run(batch.n_samples, pos, True, 1)
        # absolute positions: a third of each curve's length, and beyond its end
        abs_pos = np.repeat(lengths, 2) * np.tile([1.0 / 3.0, 1.5], batch.n_curve)
        _, us_abs = ref.run(np.full(batch.n_curve, 2), abs_pos, False, 0)
        extra = {"text": np.frombuffer(batch.text, np.uint8),
                 "loader": "reference load_dataset"} if hasattr(batch, "text") else {}
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            kind=batch.kind, degree=batch.degree, dim=batch.dim, knot_off=batch.knot_off, knots=batch.knots,
            ctrl_off=batch.ctrl_off, ctrl=batch.ctrl, n_samples=batch.n_samples, positions=pos,
            ref_lengths=lengths, ref_us=us, ref_points=pts, abs_positions=abs_pos, ref_us_abs=us_abs,
            max_error=1e-14, max_depth=23, **extra)
        print(name, batch.n_curve, "curves", us.shape[0], "samples")
    if not names or "point_rules" in names:
        np.savez_compressed(os.path.join(HERE, "point_rules.npz"), **point_rule_cases())
        print("point_rules")


if __name__ == "__main__":
    main(sys.argv[1:])
