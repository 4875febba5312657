import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "cupdlp.jl_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs through libgpdhg.so")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def lib():
    import build as pkg_build
    pkg_build.build()
    import cupdlp
    return cupdlp._abi.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.load()
    oracle.set_threads(min(8, os.cpu_count() or 1))
    return oracle
