import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(TESTS, "golden")


@pytest.fixture(scope="session")
def runs(golden_dir):
    import numpy as np

    return dict(np.load(os.path.join(golden_dir, "runs.npz")))


@pytest.fixture(scope="session")
def kat(golden_dir):
    import numpy as np

    return dict(np.load(os.path.join(golden_dir, "kat.npz")))


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, required to load where a GPU is visible (no fallback)."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    import euler2d_kokkos_gb300 as e2d

    return e2d.load_library()
