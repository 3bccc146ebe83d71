"""The CPU oracle of the learned form's network: its analytic gradients
against central finite differences (this pins the oracle that the GPU
training kernels are checked against)."""
import numpy as np

from oracle import mlp


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, mlp.IN))
    depth = rng.integers(0, 13, n)
    share = rng.dirichlet(np.ones(4), n)
    tg = rng.uniform(-1, 1, (n, 8))
    return X, depth, share, tg


def test_oracle_gradient_matches_finite_differences():
    w = mlp.he_init(3) * 0.5
    X, d, s, t = _data(6, 4)
    _, g = mlp.loss_and_grad(w, X, d, s, t)
    rng = np.random.default_rng(5)
    idx = rng.choice(mlp.N_PARAM, 60, replace=False)
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (mlp.loss_and_grad(wp, X, d, s, t)[0].sum() - mlp.loss_and_grad(wm, X, d, s, t)[0].sum()) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_pack_layout_matches_header():
    assert mlp.N_PARAM == 39328
    offs, o = {}, 0
    for name, shp in mlp.SHAPES:
        offs[name] = o
        o += int(np.prod(shp))
    assert offs["b1"] == 2048 and offs["W2"] == 2176 and offs["W4"] == 35200 and offs["b4"] == 39296
