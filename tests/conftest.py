import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    """The CPU oracle (plain-C restatement of htool's hot path)."""
    from oracle.oracle import Oracle, build_port

    build_port()
    return Oracle("port")


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np

    def load(name):
        return np.load(os.path.join(GOLDEN, name + ".npz")), json.load(open(os.path.join(GOLDEN, name + ".json")))

    return load
