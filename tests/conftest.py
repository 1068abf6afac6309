import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)



def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libqmiv_gb300.so")
    config.addinivalue_line("markers", "reference: needs the reference sources and the oracle/_ref build")


@pytest.fixture(scope="session")
def oq():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The native library on a CUDA device; fails (not skips) when the library is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ivpsnr_gb300
    from ivpsnr_gb300 import _abi
    _abi.load()
    torch.cuda.init()
    return ivpsnr_gb300
