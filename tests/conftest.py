import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C-ABI")


def pytest_collection_modifyitems(config, items):
    # order: CPU tests first, then GPU tests, files in name order (pytest default)
    pass


@pytest.fixture(scope="session")
def golden_int():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_int.npz")))


@pytest.fixture(scope="session")
def golden_pfb():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_pfb.npz")))


@pytest.fixture(scope="session")
def oc():
    from oracle import c_oracle
    return c_oracle()
