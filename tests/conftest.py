import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def lib():
    """The CUDA library, built in-tree if missing (fails loudly without nvcc)."""
    from scalit_gb300 import capi
    return capi.load(build_if_missing=True)


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle


# GPU modules whose device path has not yet passed on a GB300 run after the
# others, so that under -x a failure in one of them does not hide the rest;
# test_zz_no_alloc.py stays last (its docstring says why).
_NOT_YET_VALIDATED = ("test_gpu_window.py", "test_gpu_complex.py")


def pytest_collection_modifyitems(config, items):
    def rank(item):
        name = os.path.basename(str(item.fspath))
        if name == "test_zz_no_alloc.py":
            return 2
        return 1 if name in _NOT_YET_VALIDATED else 0
    items.sort(key=rank)
