import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _native_builds():
    """Builds what the tests load: the host synthetic helper and the CPU oracle (cheap, g++);
    the CUDA library is built by __graft_entry__.build()."""
    from biospring_gb300 import build
    from oracle import pyoracle
    build.build_synth()
    pyoracle.build_oracle()
    yield
