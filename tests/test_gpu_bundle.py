"""The GPU Bundle reader (gcv_bundle_parse / gcv_bundle_fill): the same
numbers as the host reader (gcurval_gb300.bundle.parse / load), bit for bit,
on the real curves of the reference's first dataset file, on synthetic texts
in every number form the format allows, across several files, and with the
reference loader's normalisation; malformed input fails with a message."""
import ctypes

import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import _lib, bundle
from conftest import load_golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def bundle_text(degrees, ctrls, knots, fmt=repr) -> str:
    out = []
    for p, c, k in zip(degrees, ctrls, knots):
        out.append(f"{p} {c.shape[0]} {k.size}\n" + " ".join(fmt(float(v)) for v in c[:, 0]) + " \n" +
                   " ".join(fmt(float(v)) for v in c[:, 1]) + " \n" + " ".join(fmt(float(v)) for v in k) + " \n\n")
    return "".join(out)


def golden_curves():
    b, z = load_golden("bundle_0")
    degrees = [int(p) for p in b.degree]
    ctrls = [b.ctrl[b.ctrl_off[i]:b.ctrl_off[i + 1]].reshape(-1, 2) for i in range(b.n_curve)]
    knots = [b.knots[b.knot_off[i]:b.knot_off[i + 1]] for i in range(b.n_curve)]
    return b, z, degrees, ctrls, knots


def host_arrays(texts, dim=2, normalize=True, n_curve=None):
    """The host reader's arrays for the same texts (files in order)."""
    degrees, ctrls, knots = [], [], []
    for t in texts:
        d, c, k = bundle.parse(t if isinstance(t, str) else t.decode())
        degrees += d
        ctrls += c
        knots += k
    if n_curve is not None:
        degrees, ctrls, knots = degrees[:n_curve], ctrls[:n_curve], knots[:n_curve]
    pts = [bundle.normalize(c) if normalize else c for c in ctrls]
    if dim == 3:
        pts = [np.concatenate([q, np.zeros((q.shape[0], 1))], axis=1) for q in pts]
    n = len(degrees)
    ko = np.concatenate([[0], np.cumsum([k.size for k in knots])]).astype(np.int64)
    co = np.concatenate([[0], np.cumsum([q.size for q in pts])]).astype(np.int64)
    return (np.full(n, 1, np.uint8), np.asarray(degrees, np.uint8), np.full(n, dim, np.uint8), ko,
            np.concatenate(knots) if n else np.zeros(0), co,
            np.concatenate([q.reshape(-1) for q in pts]) if n else np.zeros(0))


def assert_same(dev, host):
    names = ("kind", "degree", "dim", "knot_off", "knots", "ctrl_off", "ctrl")
    for name, a, h in zip(names, dev, host):
        a = a.cpu().numpy()
        assert a.shape == h.shape, name
        # bit for bit (NaN-free inputs; -0.0 and 0.0 told apart)
        assert np.array_equal(a.view(np.uint8), np.ascontiguousarray(h, a.dtype).view(np.uint8)), name


def test_real_curves_unnormalised_give_the_fixture_arrays(gpu_lib):
    b, z, degrees, ctrls, knots = golden_curves()
    text = bundle_text(degrees, ctrls, knots).encode()
    dev = bundle.load_device(text, normalize=False)
    assert_same(dev, (b.kind, b.degree, b.dim, b.knot_off, b.knots, b.ctrl_off, b.ctrl))
    # and the table built from them reproduces the reference's lengths
    calc = g.ArclengthCalculateGpu.from_device_batch(*dev)
    calc.createArclengthTable()
    L = calc.getAllCurveArclengths()
    calc.close()
    assert np.max(np.abs(L - z["ref_lengths"]) / z["ref_lengths"]) <= 1e-9


def test_real_curves_give_the_reference_loaders_arrays(gpu_lib):
    """The device reader on the text of the reference's first 300 dataset
    records (kept in the fixture) gives, bit for bit, what the reference's
    own load_dataset made of them (the fixture's arrays)."""
    b, z = load_golden("bundle_0")
    assert str(z["loader"]) == "reference load_dataset"
    dev = bundle.load_device(z["text"].tobytes(), normalize=True)
    assert_same(dev, (b.kind, b.degree, b.dim, b.knot_off, b.knots, b.ctrl_off, b.ctrl))


@pytest.mark.parametrize("dim", [2, 3])
def test_real_curves_normalised_like_the_host_reader(gpu_lib, dim):
    _, _, degrees, ctrls, knots = golden_curves()
    # printed with 6 significant digits, as the dataset files are
    text = bundle_text(degrees, [c * 7.3 + 11.0 for c in ctrls], knots, fmt=lambda v: f"{v:.6g}")
    dev = bundle.load_device(text.encode(), dim=dim)
    assert_same(dev, host_arrays([text], dim=dim))


def test_number_forms_files_and_limits(gpu_lib):
    f1 = "3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n"
    f2 = ("2\t4\t7\r\n+1.5 -2.25e0 3E+1 .5\r\n-0 4.000 5e-3 1234567890123456789e-18\r\n"
          "0 0 0 0.3333333333333333 1 1 1")  # no newline at the end
    f3 = ""  # an empty file between two others
    rng = np.random.default_rng(3)
    x = rng.normal(size=6) * 10.0 ** rng.integers(-15, 15, 6)
    y = rng.normal(size=6)
    f4 = ("5 6 12\n" + " ".join(f"{v:.17g}" for v in x) + "\n" + " ".join(f"{v:.18e}" for v in y) +
          "\n0 0 0 0 0 0 1 1 1 1 1 1\n")
    texts = [f1, f2, f3, f4]
    for normalize in (False, True):
        dev = bundle.load_device([t.encode() for t in texts], normalize=normalize)
        assert_same(dev, host_arrays(texts, normalize=normalize))
    dev = bundle.load_device([t.encode() for t in texts], n_curve=2, normalize=False)
    assert_same(dev, host_arrays(texts, normalize=False, n_curve=2))
    dev = bundle.load_device([t.encode() for t in texts], n_curve=0)
    assert dev[0].numel() == 0 and dev[3].cpu().tolist() == [0]


def test_many_files_of_many_curves(gpu_lib):
    rng = np.random.default_rng(5)
    texts = []
    for f in range(40):
        degrees, ctrls, knots = [], [], []
        for c in range(int(rng.integers(50, 300))):
            p = int(rng.integers(1, 6))
            n = int(rng.integers(p + 1, 40))
            degrees.append(p)
            ctrls.append(np.round(rng.normal(size=(n, 2)) * 20, 4))
            inner = np.sort(np.round(rng.random(n - p - 1), 6))
            knots.append(np.concatenate([np.zeros(p + 1), inner, np.ones(p + 1)]))
        texts.append(bundle_text(degrees, ctrls, knots, fmt=lambda v: f"{v:g}"))
    dev = bundle.load_device([t.encode() for t in texts])
    assert_same(dev, host_arrays(texts))


@pytest.mark.parametrize("bad, what", [
    ("3 4 9\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n", "malformed"),
    ("3 4 8\n0 1 2\n", "malformed"),
    ("3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1 7\n", "malformed"),
    ("3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1.2.3\n", "decimal"),
    ("3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 x\n", "decimal"),
    ("3.5 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n", "malformed"),
])
def test_malformed_text_is_rejected(gpu_lib, bad, what):
    with pytest.raises(_lib.GcvError) as e:
        bundle.load_device(["3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n".encode(), bad.encode()])
    assert e.value.status == _lib.GCV_ERR_INVALID
    assert what in str(e.value) and "file 1" in str(e.value)


def test_files_must_not_share_a_number(gpu_lib):
    lib = g.load()
    text = b"3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 13 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n"
    cut = text.index(b"13 4") + 1
    off = (ctypes.c_int64 * 3)(0, cut, len(text))
    h = ctypes.c_void_p()
    st = lib.gcv_bundle_parse(text, len(text), off, 2, -1, 2, _lib.GCV_HOST, None, ctypes.byref(h))
    assert st == _lib.GCV_ERR_INVALID and b"across" in lib.gcv_last_error()
    # host text, one file: parses
    good = b"3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n"
    st = lib.gcv_bundle_parse(good, len(good), (ctypes.c_int64 * 2)(0, len(good)), 1, -1, 2, _lib.GCV_HOST, None,
                              ctypes.byref(h))
    assert st == 0
    n = ctypes.c_int64()
    assert lib.gcv_bundle_sizes(h, ctypes.byref(n), None, None) == 0 and n.value == 1
    lib.gcv_bundle_destroy(h)
