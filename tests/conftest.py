import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden", "hard_leaves.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ora():
    import oracle as o
    o.load()
    return o


@pytest.fixture(scope="session")
def pcg():
    import primecount_gb300 as p
    if not os.path.exists(p.LIB_PATH):
        from primecount_gb300 import build
        build.build_lib()
    p.load()
    return p
