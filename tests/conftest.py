import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")
    config.addinivalue_line("markers", "slow: full-size workload check")


@pytest.fixture(scope="session")
def built_lib():
    """libt1m_cuda.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from t1m_gb300 import build as b
    return b.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    import t1m_gb300 as t1m
    c = t1m.Context()
    yield c
    c.close()


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch
