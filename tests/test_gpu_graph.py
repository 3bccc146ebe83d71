"""gcv_step_graph: the table build and the sampling captured as one CUDA
graph give the ordinary path's results bit for bit, replay with new sample
counts, and are captured again when the options change."""
import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import datasets as ds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(b):
    tk = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).cuda().to(dt)
    arrs = (tk(b.kind, torch.uint8), tk(b.degree, torch.uint8), tk(b.dim, torch.uint8), tk(b.knot_off, torch.int64),
            tk(b.knots, torch.float64), tk(b.ctrl_off, torch.int64), tk(b.ctrl, torch.float64))
    return arrs, tk(b.n_samples, torch.int32), tk(b.sample_positions(), torch.float64)


def _ordinary(arrs, cnt, pos, **kw):
    calc = g.ArclengthCalculateGpu.from_device_batch(*arrs, **kw)
    calc.createArclengthTable()
    out = torch.empty(pos.shape[0], dtype=torch.float64, device="cuda")
    calc.arclengthReverseInto(cnt, pos, out, True, g.GCV_RETURN_US)
    L = calc.getAllCurveArclengths()
    calc.close()
    return L, out.cpu().numpy()


@pytest.mark.parametrize("kind", ["uniform", "uneven_mixed", "uneven_learned"])
def test_graph_step_matches_ordinary_path(gpu_lib, kind):
    if kind == "uniform":
        b = ds.uniform_bsplines(3000, n_ctrl=40, n_samples=100, seed=3)
        kw = dict(precision=g.GCV_PLAIN_FP64)
    else:
        b = ds.uneven_batch(3000, seed=4, max_samples=256)
        kw = dict(precision=g.GCV_MIXED, rtol=b.rtol, learned=kind == "uneven_learned")
    arrs, cnt, pos = _dev(b)
    calc = g.ArclengthCalculateGpu.from_device_batch(*arrs, collect_stats=True, **kw)
    if kw.get("learned"):
        from gcurval_gb300 import learned
        calc.set_learned_model(learned.load_model())
    out = torch.empty(pos.shape[0], dtype=torch.float64, device="cuda")
    for _ in range(3):  # capture, then replays
        out.fill_(-7.0)
        calc.stepGraph(cnt, pos, out)
        got = out.cpu().numpy()
        L = calc.getAllCurveArclengths()
        if kw.get("learned"):
            ref_L, ref_u = L, got  # compared with the ordinary learned path below
        else:
            ref_L, ref_u = _ordinary(arrs, cnt, pos, **kw)
        np.testing.assert_array_equal(L, ref_L)
        np.testing.assert_array_equal(got, ref_u)
    st = calc.stats()
    assert st["n_panels"] > 0 and st["n_samples"] >= 0
    if kw.get("learned"):
        calc2 = g.ArclengthCalculateGpu.from_device_batch(*arrs, **kw)
        from gcurval_gb300 import learned
        calc2.set_learned_model(learned.load_model())
        calc2.createArclengthTable()
        o2 = torch.empty_like(out)
        calc2.arclengthReverseInto(cnt, pos, o2, True, g.GCV_RETURN_US)
        np.testing.assert_array_equal(calc2.getAllCurveArclengths(), calc.getAllCurveArclengths())
        np.testing.assert_array_equal(o2.cpu().numpy(), out.cpu().numpy())
        calc2.close()
    calc.close()


def test_graph_replay_with_new_counts(gpu_lib):
    b = ds.uneven_batch(2000, seed=5, max_samples=128)
    arrs, cnt, pos = _dev(b)
    calc = g.ArclengthCalculateGpu.from_device_batch(*arrs, precision=g.GCV_MIXED, rtol=b.rtol)
    out = torch.empty(pos.shape[0], dtype=torch.float64, device="cuda")
    calc.stepGraph(cnt, pos, out)
    # the same total, other curves: permuted counts in the same buffer
    perm = np.random.default_rng(0).permutation(b.n_curve)
    cnt.copy_(torch.from_numpy(b.n_samples[perm].astype(np.int32)).cuda())
    calc.stepGraph(cnt, pos, out)
    got = out.cpu().numpy()
    ref = torch.empty_like(out)
    calc.arclengthReverseInto(cnt, pos, ref, True, g.GCV_RETURN_US)
    np.testing.assert_array_equal(got, ref.cpu().numpy())
    calc.close()


def test_graph_captures_again_after_an_option_change(gpu_lib):
    b = ds.uniform_bsplines(500, n_ctrl=30, n_samples=20, seed=6)
    arrs, cnt, pos = _dev(b)
    calc = g.ArclengthCalculateGpu.from_device_batch(*arrs, precision=g.GCV_PLAIN_FP64, rtol=1e-4)
    out = torch.empty(pos.shape[0], dtype=torch.float64, device="cuda")
    calc.stepGraph(cnt, pos, out)
    # a tighter tolerance: a new table (more leaves), a new capture
    calc.set_options(g.GCV_PLAIN_FP64, rtol=1e-13)
    calc.stepGraph(cnt, pos, out)
    ref_L, ref_u = _ordinary(arrs, cnt, pos, precision=g.GCV_PLAIN_FP64, rtol=1e-13)
    np.testing.assert_array_equal(calc.getAllCurveArclengths(), ref_L)
    np.testing.assert_array_equal(out.cpu().numpy(), ref_u)
    calc.close()


def test_autotuner_settles_after_three_builds(gpu_lib):
    # a batch shape of its own (interval count) so that no earlier test tuned it
    b = ds.uniform_bsplines(777, n_ctrl=23, degree=4, dim=3, n_samples=11, seed=8)
    arrs, cnt, pos = _dev(b)
    calc = g.ArclengthCalculateGpu.from_device_batch(*arrs, precision=g.GCV_MIXED)
    out = torch.empty(pos.shape[0], dtype=torch.float64, device="cuda")
    results = []
    for i in range(5):
        calc.createArclengthTable()
        calc.arclengthReverseInto(cnt, pos, out, True, g.GCV_RETURN_US)
        results.append(out.cpu().numpy().copy())
        st = calc.stats()
        assert st["tuned"] == (1 if i >= 2 else 0), (i, st)
    for r in results[1:]:
        np.testing.assert_array_equal(r, results[0])  # shapes change scheduling only
    assert st["length_blocks_per_sm"] in (4, 6, 32) and st["sample_threads"] in (128, 256, 512)
    # a second context of the same shape starts tuned
    calc2 = g.ArclengthCalculateGpu.from_device_batch(*arrs, precision=g.GCV_MIXED)
    calc2.createArclengthTable()
    assert calc2.stats()["tuned"] == 1
    calc2.close()
    calc.close()
