import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libpyre_cuda.so")
    config.addinivalue_line("markers", "slow: larger parity cases")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    if not _has_gpu():
        pytest.skip("no CUDA device")
    from pyre_gb300 import build as B
    B.build()
    from pyre_gb300 import CudaIntegrator
    ctx = CudaIntegrator(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.lib()
    return O
