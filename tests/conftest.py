import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def ads():
    import __graft_entry__ as g

    pkg = g.load_package()
    if not os.path.exists(pkg.LIB_PATH):  # a fresh checkout: compile the library first
        pkg.build_library()
    return pkg


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def golden(name):
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", name))
