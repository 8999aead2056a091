import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        data = {k: z[k] for k in z.files}
    cases = sorted({k.split(".")[0] for k in data if not k.startswith("seq.")})
    return data, cases


@pytest.fixture(scope="session")
def mdsx_lib():
    """libmdsx.so, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from massivemds_gb300 import build

    build.build()
    from massivemds_gb300 import _lib

    return _lib.load()
