"""The learned form on the GPU: FP32 training gradients against the CPU
oracle (oracle/mlp.py), the BF16 tensor-core inference against the FP32
forward pass, and the learned table against the FP64 oracle with the panels
it saves over the same walk without the network."""
import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import datasets as ds
from gcurval_gb300 import learned
from oracle import mlp
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 16)).astype(np.float32)
    depth = rng.integers(0, 13, n).astype(np.int32)
    share = rng.dirichlet(np.ones(4), n).astype(np.float32)
    tg = rng.uniform(-1, 1, (n, 8)).astype(np.float32)
    return X, depth, share, tg


def _cuda(*arrs):
    return [torch.from_numpy(a).cuda() for a in arrs]


def test_training_gradients_match_cpu_oracle(gpu_lib):
    w = (mlp.he_init(7) * 0.5).astype(np.float32)
    X, d, s, t = _data(300, 8)
    tr = learned.Trainer(512, weights=w)
    gg, loss = tr.gradients(*_cuda(X, d, s, t))
    tr.close()
    lo, go = mlp.loss_and_grad(w.astype(np.float64), X, d, s, t)
    np.testing.assert_allclose(loss, lo, rtol=2e-5)
    scale = np.abs(go).max()
    assert np.max(np.abs(gg - go)) <= 2e-4 * scale
    # per layer, relative to the layer's own gradient size
    o = 0
    for name, shp in mlp.SHAPES:
        n = int(np.prod(shp))
        gl, ol = gg[o:o + n], go[o:o + n]
        assert np.linalg.norm(gl - ol) <= 1e-4 * np.linalg.norm(ol) + 1e-7, name
        o += n


def test_forward_matches_cpu_oracle(gpu_lib):
    w = (mlp.he_init(9) * 0.5).astype(np.float32)
    X, _, _, _ = _data(1000, 10)
    tr = learned.Trainer(1024, weights=w)
    out = tr.forward(torch.from_numpy(X).cuda()).cpu().numpy()
    tr.close()
    ref, _, _ = mlp.forward(w.astype(np.float64), X)
    np.testing.assert_allclose(out, ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 40000])
def test_tensor_core_inference_matches_fp32(gpu_lib, n):
    # BF16 operands, FP32 accumulation: compare with the FP32 forward pass
    w = (mlp.he_init(11) * 0.5).astype(np.float32)
    X, _, _, _ = _data(n, 12)
    Xd = torch.from_numpy(X).cuda()
    tc = learned.infer(w, Xd).cpu().numpy()
    ref, _, _ = mlp.forward(w.astype(np.float64), X)
    err = np.abs(tc - ref)
    assert np.max(err) <= 0.05 * np.abs(ref).max(), np.max(err)
    assert np.mean(err) <= 0.01 * np.abs(ref).mean() + 1e-3


def test_short_training_reduces_the_loss(gpu_lib):
    b = ds.uneven_batch(300, seed=21)
    calc = g.ArclengthCalculateGpu.from_batch(b, precision=g.GCV_PLAIN_FP64, rtol=b.rtol)
    calc.createArclengthTable()
    n = calc.n_segments
    X = torch.empty((n, 16), dtype=torch.float32, device="cuda")
    D = torch.empty(n, dtype=torch.int32, device="cuda")
    S = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    T = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    calc.learned_features(X)
    calc.learned_labels(D, S, T)
    calc.close()
    keep = (X[:, 0] > 0) & (X[:, 11] > 0)
    X, D, S, T = X[keep].contiguous(), D[keep].contiguous(), S[keep].contiguous(), T[keep].contiguous()
    assert int(D.min()) >= 0 and int(D.max()) <= 12
    np.testing.assert_allclose(S.sum(dim=1).cpu().numpy(), 1.0, rtol=1e-6)
    tr = learned.Trainer(4096, seed=3)
    first = tr.gradients(X[:4096], D[:4096], S[:4096], T[:4096])[1].sum()
    for _ in range(4):
        for i in range(0, X.shape[0] - 4096 + 1, 4096):
            tr.step(X[i:i + 4096], D[i:i + 4096], S[i:i + 4096], T[i:i + 4096], 2e-3)
    last = tr.gradients(X[:4096], D[:4096], S[:4096], T[:4096])[1].sum()
    tr.close()
    assert last < 0.8 * first


def _table(b, learned_on, w=None):
    calc = g.ArclengthCalculateGpu.from_batch(b, precision=g.GCV_MIXED, rtol=b.rtol, collect_stats=True,
                                             learned=learned_on)
    if w is not None:
        calc.set_learned_model(w)
    calc.createArclengthTable()
    L = calc.getAllCurveArclengths()
    u = calc.arclengthReverse(b.n_samples, b.positions, True, g.GCV_HOST).us
    st = calc.stats()
    calc.close()
    return L, u, st


def test_learned_table_meets_tolerance_and_saves_panels(gpu_lib):
    w = learned.load_model()
    b = ds.uneven_batch(400, seed=31)
    b.sample_positions()
    L0, u0, st0 = _table(b, False)
    L1, u1, st1 = _table(b, True, w)
    o = Oracle(b)
    Lo = o.lengths()
    assert np.max(np.abs(L1 - Lo) / Lo) <= 1e-8
    s = o.s_at(b.n_samples, u1)
    tgt = b.positions * np.repeat(Lo, b.n_samples)
    assert np.max(np.abs(s - tgt) / np.repeat(Lo, b.n_samples)) <= 1e-8
    # the gain: panels of the length walk with the network against without it
    assert st1["n_panels"] < st0["n_panels"], (st1["n_panels"], st0["n_panels"])
    assert st1["ms_learned"] > 0.0


def test_learned_model_is_validated(gpu_lib):
    b = ds.uneven_batch(20, seed=32)
    calc = g.ArclengthCalculateGpu.from_batch(b, precision=g.GCV_MIXED, learned=True)
    with pytest.raises(ValueError):
        calc.set_learned_model(np.zeros(10, np.float32))
    bad = np.full(learned.N_PARAM, np.nan, np.float32)
    with pytest.raises(g.GcvError):
        calc.set_learned_model(bad)
    calc.set_learned_model(None)
    calc.createArclengthTable()  # no network: the plain start
    calc.close()
