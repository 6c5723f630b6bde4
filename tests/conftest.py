import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session", autouse=True)
def native_library():
    """libgmhd.so (the kernels, the C ABI and the host leaf forest the AMR mesh builders call);
    compiled here when missing or stale (nvcc cross-compiles without a GPU)."""
    from godunov_mhd_ct_gb300.csrc import build

    build.build()
