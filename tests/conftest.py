import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "lbdemcoupling-public_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")
    config.addinivalue_line("markers", "slow: full-size cases that take tens of seconds")


def _gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle import psm_oracle
    psm_oracle.load()
    return psm_oracle


@pytest.fixture(scope="session")
def lbdem_lib():
    """The CUDA library, built in-tree if needed.  GPU tests fail loudly without it."""
    import build as pkg_build
    pkg_build.build()
    import lbdem
    lbdem.load()
    return lbdem


@pytest.fixture(scope="session")
def gpu(lbdem_lib):
    if not _gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return lbdem_lib
