import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and liblvrgb.so")
    config.addinivalue_line("markers", "slow: full-size workload")


def gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    """liblvrgb.so, built in-tree if needed (the GPU tests call through the C ABI)."""
    from lvr2_gb300 import build as B
    B.build()
    import lvr2_gb300
    return lvr2_gb300.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O
