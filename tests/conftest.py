"""Shared test set-up: repository root on sys.path, the `gpu` marker, and the
native library built on demand (CPU tests only need it loaded, not run)."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def native():
    """Build (if stale) and load librmq.so."""
    from rtxrmq_gb300 import build as b
    b.build()
    import rtxrmq_gb300
    return rtxrmq_gb300.load()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(with_ref=None)
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
