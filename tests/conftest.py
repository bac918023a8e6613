import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def lib_built():
    from umwm_gb300 import build

    build.build()
    import umwm_gb300

    umwm_gb300.lib()
    return umwm_gb300
