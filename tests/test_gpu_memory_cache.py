"""The device memory cache: a destroyed context's buffers serve the next
context of the same shape, results stay bit for bit the same, the cache can
be emptied, and GCV_NO_MEMORY_CACHE=1 turns it off."""
import os
import subprocess
import sys

import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import datasets as ds

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def one_pass(b, pos, **kw):
    calc = g.ArclengthCalculateGpu.from_batch(b, **kw)
    calc.createArclengthTable()
    L = calc.getAllCurveArclengths()
    u = calc.arclengthReverse(b.n_samples, pos, True, g.GCV_HOST, g.GCV_RETURN_US).us.copy()
    calc.close()
    return L, u


@pytest.mark.parametrize("precision", [g.GCV_PLAIN_FP64, g.GCV_MIXED])
def test_reused_buffers_give_the_same_results(gpu_lib, precision):
    b = ds.uneven_batch(600, seed=21)
    pos = b.sample_positions()
    g.release_cached_memory()
    L0, u0 = one_pass(b, pos, precision=precision)
    cached = g.release_cached_memory()
    assert cached > 0  # the context's buffers went to the cache, and are freed now
    L1, u1 = one_pass(b, pos, precision=precision)  # fresh allocations
    L2, u2 = one_pass(b, pos, precision=precision)  # buffers from the cache
    for L, u in ((L1, u1), (L2, u2)):
        np.testing.assert_array_equal(L, L0)
        np.testing.assert_array_equal(u, u0)
    assert g.release_cached_memory() > 0


def test_cache_can_be_turned_off(gpu_lib):
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import gcurval_gb300 as g\nfrom gcurval_gb300 import datasets as ds\n"
            "b = ds.uniform_bsplines(50, n_ctrl=12, n_samples=5, seed=2)\n"
            "c = g.ArclengthCalculateGpu.from_batch(b); c.createArclengthTable(); c.close()\n"
            "print(g.release_cached_memory())\n") % ROOT
    env = dict(os.environ, GCV_NO_MEMORY_CACHE="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-1] == "0"
