import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long CPU statistics test")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def dsm_mod():
    """The native library, built in-tree; GPU tests fail (not skip) if it is missing."""
    import gpu_dsm_gb300 as g
    from gpu_dsm_gb300 import build as b
    b.build()
    g.load_library()
    return g
