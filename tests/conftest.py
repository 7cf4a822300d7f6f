import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def emv():
    """The product package with its native library built and loaded."""
    import steiner_edge_linear_gb300 as E

    E.build()
    E.load_library()
    return E


@pytest.fixture(scope="session")
def orc():
    """The oracle package (C restatement built; reference leg when its source is present)."""
    import oracle

    oracle.build(reference=True)
    return oracle


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)
