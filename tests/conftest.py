import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libosb_gb300.so")


@pytest.fixture(scope="session")
def built_lib():
    from opensbli_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    import harness
    return harness.build_oracle()
