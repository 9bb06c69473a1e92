import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU oracle runs")


@pytest.fixture(scope="session")
def built_lib():
    """Path of the C-ABI library, building it in-tree when it is missing."""
    from phinfortran_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    return build.LIB


@pytest.fixture(scope="session")
def cuda_ready(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True


@pytest.fixture(scope="session")
def sisi():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "sisi.npz")))
