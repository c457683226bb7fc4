import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "ski-lls_gb300", os.path.join("tests", "golden")):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def fixtures():
    return np.load(os.path.join(GOLDEN, "fixtures.npz"))


def fixture_csc(z, name):
    n, d = (int(v) for v in z[name + "/shape"])
    return n, d, z[name + "/indptr"], z[name + "/indices"], z[name + "/data"]


RANK_DEF_NAMES = ["lp_ship12l", "Franz1", "GL7d26", "cis-n4c6-b2", "lp_modszk1", "rel5",
                  "ch5-5-b1", "n3c5-b2", "ch4-4-b1", "n3c5-b1", "n3c4-b1", "cis-n4c6-b3"]
FULL_RANK_TAGS = ["50by15", "50by20", "100by15", "100by20", "120by15", "120by20"]


def residual_matches(res, expected):
    """test/test_solvers.sh prints residuals to 6 significant digits; values
    below 1e-12 are round-off of a consistent system."""
    if expected < 1e-12:
        return res < 1e-11
    return abs(res - expected) <= 1e-5 * expected + 1e-12
