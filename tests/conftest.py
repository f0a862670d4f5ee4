import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_golden.npz"))


@pytest.fixture(scope="session")
def golden_meta():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "reference_golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def engine_lib():
    """The C-ABI library, built in-tree when missing (nvcc cross-compiles without a GPU)."""
    from pyramaterised_gb300 import _lib, build

    if not os.path.exists(build.lib_path()):
        build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyramaterised_gb300 import _lib, build

    if not os.path.exists(build.lib_path()):
        build.build()
    _lib.load()
    return torch.device("cuda", 0)


@pytest.fixture(scope="session")
def oracle_pool():
    """Spawned single-threaded oracle workers for parity checks at benchmark sizes (started on first use)."""
    from oracle_pool import OraclePool

    pool = OraclePool()
    yield pool
    pool.close()
