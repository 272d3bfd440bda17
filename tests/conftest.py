import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden():
    """{case: {values, keys, offsets, index, merged}} from the committed fixtures."""
    z = np.load(GOLDEN)
    out = {}
    for key in z.files:
        case, field = key.split("/")
        out.setdefault(case, {})[field] = z[key]
    return out


@pytest.fixture(scope="session")
def golden():
    return load_golden()
