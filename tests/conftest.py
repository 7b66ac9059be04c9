import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build(with_ref=False)
    return O


@pytest.fixture(scope="session")
def cglib():
    """libconvGemm.so, built in-tree if missing or stale."""
    from convgemm_gb300 import build
    build.build()
    import convgemm_gb300 as cg
    return cg
