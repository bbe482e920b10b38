import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu on a GB300)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def built_library():
    from gpucell_gb300.build import build_library
    return build_library()


@pytest.fixture(scope="session")
def oracle_lib():
    from gpucell_gb300.build import build_oracle
    build_oracle()
    from oracle import binding
    return binding.load()


@pytest.fixture(scope="session")
def cuda_device(built_library):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
