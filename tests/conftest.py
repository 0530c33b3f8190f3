import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "reference_tests.npz"))


@pytest.fixture(scope="session")
def golden_sh():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "sh_adam.npz"))


@pytest.fixture(scope="session")
def gray_lib():
    """The CUDA library, built in-tree for sm_103a (nvcc cross-compiles without a GPU)."""
    from gray_gb300 import build as B
    from gray_gb300 import _lib

    B.build()
    return _lib.load()
