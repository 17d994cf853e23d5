import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
REF_ROOT = "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger parity case")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build_oracle()
    return O


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; a GPU test must run on the native path."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from annfmp_gb300 import build as B
    B.build()
    from annfmp_gb300 import _lib
    return _lib.load()
