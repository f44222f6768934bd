import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built librgf_gb300.so")


@pytest.fixture(scope="session")
def rgf():
    import rgf_gb300
    rgf_gb300.load_library()
    return rgf_gb300
