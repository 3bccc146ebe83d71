import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


# fixtures that are not curve batches with reference outputs
NOT_CURVE_CASES = {"point_rules"}


def golden_names():
    """The curve-batch fixtures (batch + the reference's lengths and samples)."""
    names = (os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    return sorted(n for n in names if n not in NOT_CURVE_CASES)


def load_golden(name):
    """(CurveBatch, npz dict) of a committed golden case."""
    from gcurval_gb300 import datasets as ds
    z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    b = ds.CurveBatch(z["kind"], z["degree"], z["dim"], z["knot_off"], z["knots"], z["ctrl_off"], z["ctrl"],
                      z["n_samples"], z["positions"], name, 1e-10)
    return b, z


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library on a GPU host; a GPU test fails (not skips) when it cannot load."""
    import gcurval_gb300 as g
    return g.load()
