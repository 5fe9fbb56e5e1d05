import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Builds libppgpu.so and the oracle restatement once per session."""
    from patchyparticles_gb300 import build
    from oracle import pyoracle

    build.build()
    pyoracle.build(with_reference=False)
    return True
