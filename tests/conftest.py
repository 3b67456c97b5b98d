import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib


@pytest.fixture(scope="session")
def kats():
    import json
    with open(os.path.join(HERE, "golden", "userguide_kats.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu():
    import jadamilu_gb300 as J
    L = J.load()
    if L.jdgpu_device_count() <= 0:
        pytest.fail("GPU test selected but no CUDA device is visible")
    return J
