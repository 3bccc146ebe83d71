"""Generates the golden fixtures in this folder from the reference's own CPU
driver (gcurval::ArclengthCalculateCpu, compiled from the reference tree by
oracle/Makefile into oracle/_ref/libgcv_ref.so).

    python tests/golden/make_golden.py [case ...]

Each ``<case>.npz`` holds the curve batch (CurveBatch arrays), the sample
counts and positions, and the reference's outputs: total lengths
(getAllCurveArclengths), sample parameters and points (arclengthReverse with
gcurvalHost / gcurvalReverseReturnUs and ...Points), at the reference's
default FP64 configuration (MAX_ERROR 1e-14, depth 23).  The reference tree
is needed only here; tests read the committed files.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_TREE = "/root/reference"
sys.path.insert(0, ROOT)

from gcurval_gb300 import bundle  # noqa: E402
from gcurval_gb300 import datasets as ds  # noqa: E402
from oracle.oracle import Reference, reference_available  # noqa: E402


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
    # read and normalised like its loader (samples/sample2_bspline/dataset_loader.h)
    bundle_file = os.path.join(REF_TREE, "dataset", "BSpline", "Bundle_0.txt")
    if os.path.exists(bundle_file):
        out["bundle_0"] = bundle.load(bundle_file, n_curve=300, samples_per_curve=9)
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
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            kind=batch.kind, degree=batch.degree, dim=batch.dim, knot_off=batch.knot_off, knots=batch.knots,
            ctrl_off=batch.ctrl_off, ctrl=batch.ctrl, n_samples=batch.n_samples, positions=pos,
            ref_lengths=lengths, ref_us=us, ref_points=pts, abs_positions=abs_pos, ref_us_abs=us_abs,
            max_error=1e-14, max_depth=23)
        print(name, batch.n_curve, "curves", us.shape[0], "samples")


if __name__ == "__main__":
    main(sys.argv[1:])
