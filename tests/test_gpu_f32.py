"""FP32 data (the reference's ArclengthCalculateGpu<float>, the samples'
default): float curve data, positions and results through the *_f32 entry
points give exactly the double path's results on the widened data, rounded
to float."""
import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import datasets as ds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def double_reference(make, pos64, counts, what=g.GCV_RETURN_US, **kw):
    calc = make()
    calc.createArclengthTable()
    L = calc.getAllCurveArclengths()
    r = calc.arclengthReverse(counts, pos64, True, g.GCV_HOST, what)
    out = r.us if what == g.GCV_RETURN_US else r.points
    calc.close()
    return L.astype(np.float32), out.astype(np.float32)


@pytest.mark.parametrize("precision", [g.GCV_PLAIN_FP64, g.GCV_MIXED])
def test_ellipses_f32(gpu_lib, precision):
    rng = np.random.default_rng(3)
    n = 300
    a = rng.uniform(0.1, 10, n).astype(np.float32)
    b = rng.uniform(0.1, 10, n).astype(np.float32)
    rot = rng.uniform(0, 6.28, n).astype(np.float32)
    counts = rng.integers(0, 40, n).astype(np.int32)
    pos = rng.random(int(counts.sum())).astype(np.float32)
    for what in (g.GCV_RETURN_US, g.GCV_RETURN_POINTS):
        L_ref, u_ref = double_reference(
            lambda: g.ArclengthCalculateGpu.ellipses(a.astype(np.float64), b.astype(np.float64),
                                                     rot.astype(np.float64), precision=precision),
            pos.astype(np.float64), counts, what)
        calc = g.ArclengthCalculateGpu.ellipses(a, b, rot, precision=precision)
        assert calc.f32
        calc.createArclengthTable()
        L = calc.getAllCurveArclengths()
        assert L.dtype == np.float32
        np.testing.assert_array_equal(L, L_ref)
        assert calc.getArclength(7) == L_ref[7]
        r = calc.arclengthReverse(counts, pos, True, g.GCV_HOST, what)
        res = r.us if what == g.GCV_RETURN_US else r.points
        assert res.dtype == np.float32
        np.testing.assert_array_equal(res, u_ref)
        calc.close()


@pytest.mark.parametrize("where", ["host", "device"])
def test_bsplines_f32(gpu_lib, where):
    bb = ds.uniform_bsplines(120, n_ctrl=20, n_samples=33, seed=12)
    pos = bb.sample_positions().astype(np.float32)
    ko = bb.knot_off.astype(np.int32)
    kv = bb.knots.astype(np.float32)
    cp = bb.ctrl.astype(np.float32)
    counts = bb.n_samples.astype(np.int32)
    L_ref, u_ref = double_reference(
        lambda: g.ArclengthCalculateGpu.bsplines(3, 2, ko, kv.astype(np.float64), cp.astype(np.float64),
                                                 precision=g.GCV_MIXED),
        pos.astype(np.float64), counts)
    if where == "host":
        calc = g.ArclengthCalculateGpu.bsplines(3, 2, ko, kv, cp, precision=g.GCV_MIXED)
    else:
        calc = g.ArclengthCalculateGpu.bsplines(3, 2, torch.from_numpy(ko).cuda(), torch.from_numpy(kv).cuda(),
                                                torch.from_numpy(cp).cuda(), precision=g.GCV_MIXED)
    calc.createArclengthTable()
    np.testing.assert_array_equal(calc.getAllCurveArclengths(), L_ref)
    # into host and device buffers
    out = np.empty(pos.size, np.float32)
    calc.arclengthReverseInto(counts, pos, out, True)
    np.testing.assert_array_equal(out, u_ref)
    d_out = torch.empty(pos.size, dtype=torch.float32, device="cuda")
    calc.arclengthReverseInto(torch.from_numpy(counts).cuda(), torch.from_numpy(pos).cuda(), d_out, True)
    np.testing.assert_array_equal(d_out.cpu().numpy(), u_ref)
    d_len = torch.empty(calc.n_curve, dtype=torch.float32, device="cuda")
    calc.getAllCurveArclengths(out=d_len)
    np.testing.assert_array_equal(d_len.cpu().numpy(), L_ref)
    r = calc.arclengthReverse(counts, pos, True, g.GCV_DEVICE)
    np.testing.assert_array_equal(r.us, u_ref)
    with pytest.raises(ValueError):
        calc.arclengthReverseInto(counts, pos, np.empty(pos.size, np.float64), True)
    calc.close()
