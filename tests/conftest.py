import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300", "python"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib

    oracle_lib.build()
    # the oracle's sparse rows on OpenMP threads: no result changes (each row keeps its
    # own summation order); bench.py's CPU baseline keeps them serial
    oracle_lib.set_parallel_rows(True)
    return oracle_lib


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library; built if needed.  No CPU fallback exists."""
    sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300"))
    import build_ext

    build_ext.build()
    import cpm_gb300

    info = cpm_gb300.device_info()
    return cpm_gb300
