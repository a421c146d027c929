import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def known():
    with open(os.path.join(GOLDEN, "known.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def rsuite():
    return dict(np.load(os.path.join(GOLDEN, "random_suite.npz")))


@pytest.fixture(scope="session")
def csuite():
    return dict(np.load(os.path.join(GOLDEN, "configs.npz")))


@pytest.fixture(scope="session")
def gpu():
    """The drop-in GPU module; builds the library if needed and requires a GPU."""
    from editdist_bench_gb300 import _build
    _build.build()
    from editdist_bench_gb300 import gpu as g
    assert g.available(), "no CUDA device visible: GPU tests need one"
    return g
