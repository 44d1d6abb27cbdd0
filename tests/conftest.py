import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    """The FP64 oracle (psv_oracle.c), built on first use, single-threaded
    so its reductions are in a fixed order."""
    from oracle import oracle as O
    O.build()
    o = O.oracle()
    o.set_threads(1)
    return o


@pytest.fixture(scope="session")
def gpu():
    """Fails (does not skip) when the engine cannot see a GPU: GPU tests must
    run the CUDA path or fail loudly."""
    from fwi_cuda_gb300 import _lib
    assert _lib.device_available(), "no CUDA device visible to libfwi_psv.so"
    return _lib
