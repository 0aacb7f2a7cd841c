import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build(reference=False)
    return oracle.Oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle
    if not oracle.Reference.available():
        if os.path.isdir(os.path.join(oracle.REFERENCE_TREE, "src", "tools")):
            oracle.build(reference=True)
    if not oracle.Reference.available():
        pytest.skip("reference harness not built (reference tree absent)")
    return oracle.Reference()


@pytest.fixture(scope="session")
def golden():
    import json
    d = os.path.join(ROOT, "tests", "golden")

    def load(name):
        with open(os.path.join(d, name)) as f:
            return json.load(f)
    return load
