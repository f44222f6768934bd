import os
import sys

import numpy as np
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


@pytest.fixture(scope="session")
def pinned():
    """Page-locked copies of host arrays (what the asynchronous upload needs):
    pinned(ia, ja, a) -> the same arrays in pinned memory, same dtypes."""
    torch = pytest.importorskip("torch")

    def pin(*arrays):
        out = []
        for x in arrays:
            x = np.ascontiguousarray(x)
            v = x.view(np.int64) if x.dtype == np.uint64 else x
            out.append(torch.from_numpy(v).pin_memory().numpy().view(x.dtype))
        return tuple(out)
    return pin
