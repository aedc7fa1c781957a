import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libqltg.so")
    config.addinivalue_line("markers", "slow: full-size cases (seconds of CPU oracle work)")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture(scope="session")
def gpu():
    """Skip unless a CUDA device and libqltg.so are present; fail loudly if the device is there
    but the library is not (no CPU fallback exists)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensortoolkit_gb300 import _native
    if not os.path.exists(_native.LIB_QLTG):
        raise RuntimeError("libqltg.so missing on a GPU host: run __graft_entry__.build()")
    return 0
