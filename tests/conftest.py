import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer-running test")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build_port()
    return oracle


@pytest.fixture(scope="session")
def tsph():
    from tinysph_old_gb300 import sph

    sph.load()
    return sph


@pytest.fixture(scope="session")
def gpu_tsph(tsph):
    if tsph.device_count() < 1:
        pytest.fail("GPU test run without a visible CUDA device")
    return tsph
