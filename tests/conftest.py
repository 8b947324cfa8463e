import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libhdg.so")


@pytest.fixture(scope="session")
def kats():
    import json
    with open(os.path.join(GOLDEN, "reference_kats.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def oracle():
    import hdgref
    hdgref.build()
    return hdgref


@pytest.fixture(scope="session")
def figure_root():
    return os.path.join(GOLDEN, "mesh", "figure2.1")
