import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "e1039-gpu_gb300"), os.path.join(REPO, "tests"),
          os.path.join(REPO, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def geometry():
    from oracle import pyoracle as O
    from orgpu import GEOMETRY_E906
    return O.parse_geometry(GEOMETRY_E906)
