import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def native_lib():
    from vmps_gb300 import build
    build.build()
    from vmps_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def gpu_ctx(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vmps_gb300.pivot import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
