import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built libvgpu (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from engines import OracleEngine
    return OracleEngine()


@pytest.fixture(scope="session")
def ref():
    from engines import RefEngine, ref_available
    if not ref_available():
        pytest.skip("reference engine not buildable here (no reference checkout)")
    return RefEngine()


@pytest.fixture(scope="session")
def gpu():
    import vectra_gb300
    return vectra_gb300.engine(0)
