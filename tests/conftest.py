"""Shared fixtures: the skeleton library (CUDA), the oracle (CPU restatement)."""
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size cases (2^28 elements and up)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def acc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as ge
    ge._load_build().build()
    pkg = ge.load_package()
    pkg.load()
    return pkg


@pytest.fixture(scope="session")
def dev(acc):
    import torch
    return torch.device("cuda:0")
