import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pnfft_oracle
    return pnfft_oracle


@pytest.fixture(scope="session")
def lib():
    import pnfft_gb300
    from pnfft_gb300 import build as _b
    _b.build()
    return pnfft_gb300
