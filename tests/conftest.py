import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "nextla.jl_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "lapack_golden.npz"))


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def tq():
    """The CUDA library front end; builds libtileqr.so when it is stale."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tileqr_build as B
    B.build()
    import tileqr
    tileqr.set_blocking(True)
    return tileqr
