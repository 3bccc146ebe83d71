"""The Bundle text format of the reference's dataset files
(samples/sample2_bspline/dataset_loader.h:40-126): parsing and the
reference loader's normalisation, on a synthetic text."""
import numpy as np
import pytest

from gcurval_gb300 import bundle


TEXT = """3 4 8
0 1 2 3
0 1 0 1
0 0 0 0 1 1 1 1

3 5 9
1 2 4 5 7
2 2 3 3 6
0 0 0 0 0.5 1 1 1 1
"""


def test_parse_records():
    d, c, k = bundle.parse(TEXT)
    assert d == [3, 3]
    np.testing.assert_array_equal(c[0], [[0, 0], [1, 1], [2, 0], [3, 1]])
    np.testing.assert_array_equal(k[1], [0, 0, 0, 0, 0.5, 1, 1, 1, 1])


def test_normalisation_like_the_reference_loader(tmp_path):
    f = tmp_path / "b.txt"
    f.write_text(TEXT)
    b = bundle.load(str(f), samples_per_curve=5)
    assert b.n_curve == 2 and np.all(b.degree == 3) and np.all(b.dim == 2)
    for i in range(2):
        q = b.ctrl[b.ctrl_off[i]:b.ctrl_off[i + 1]].reshape(-1, 2)
        np.testing.assert_allclose(q.mean(axis=0), 0.0, atol=1e-15)
        assert np.abs(q).max() == pytest.approx(1.0)
    b3 = bundle.load(str(f), dim=3)
    assert np.all(b3.ctrl.reshape(-1, 3)[:, 2] == 0.0)


@pytest.mark.parametrize("bad", ["3 4 9\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n", "3 4 8\n0 1 2\n"])
def test_malformed_records_are_rejected(bad):
    with pytest.raises(ValueError):
        bundle.parse(bad)


def test_device_number_conversion_matches_strtod(tmp_path):
    """The GPU reader's decimal conversion (gcv_decimal.cuh, host and device
    code) against the C library's correctly rounded strtod, on the host."""
    import os
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(here, "bundle", "decimal_check.cpp")
    inc = os.path.join(os.path.dirname(here), "gcurval_gb300", "csrc")
    exe = str(tmp_path / "decimal_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", inc, src, "-o", exe], check=True)
    r = subprocess.run([exe, "200000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "mismatched 0" in r.stdout


def test_host_reader_equals_the_reference_loader_on_real_curves(tmp_path):
    """tests/golden/bundle_0.npz holds the text of the first 300 records of
    the reference's dataset/BSpline/Bundle_0.txt and the arrays the
    reference's own load_dataset made of them (compiled from the reference
    by make_golden.py): the host reader gives the same bits."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "bundle_0.npz"))
    assert str(z["loader"]) == "reference load_dataset"
    f = tmp_path / "bundle_0_head.txt"
    f.write_bytes(z["text"].tobytes())
    b = bundle.load(str(f), samples_per_curve=9)
    assert b.n_curve == 300
    np.testing.assert_array_equal(b.knot_off, z["knot_off"])
    np.testing.assert_array_equal(b.ctrl_off, z["ctrl_off"])
    assert np.array_equal(b.knots.view(np.uint64), z["knots"].view(np.uint64))
    assert np.array_equal(b.ctrl.view(np.uint64), z["ctrl"].view(np.uint64))
