import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_PATH = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity / solver tests)")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """The C-ABI library is built in-tree before any test runs (no fallback)."""
    from tatva_gb300 import _build

    return _build.build()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN_PATH))


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch.device("cuda")
