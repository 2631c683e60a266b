import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    from streamparanumal_gb300 import _build, capi
    _build.build_library()
    return capi.load()


@pytest.fixture(scope="session")
def orc():
    from streamparanumal_gb300 import _build
    _build.build_oracle()
    from oracle import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def cuda(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
