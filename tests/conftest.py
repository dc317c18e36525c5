import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def built():
    """Builds the native libraries (and the oracle) once per session."""
    import oracle
    import stcdb_gb300.build as b
    b.build_tracegen()
    oracle.build(reference=False)
    return True


@pytest.fixture(scope="session")
def built_cuda(built):
    import stcdb_gb300.build as b
    b.build_cuda()
    return True
