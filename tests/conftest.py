import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "vnm-graph-reordering_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ctx():
    import vnm_gb300
    c = vnm_gb300.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def goldens():
    import numpy as np
    return np.load(os.path.join(REPO, "tests", "golden", "nm_ref_goldens.npz"))
