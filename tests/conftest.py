import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def golden(name):
    import numpy as np
    return np.load(os.path.join(REPO, "tests", "golden", name))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build_oracle()
    return O
