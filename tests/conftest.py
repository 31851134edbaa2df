import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ref_backend():
    """The reference's own kernels compiled for the CPU (only where the reference checkout exists:
    oracle/build_ref.sh locates it and builds nothing without one)."""
    from oracle import volrend as V
    if not V.ref_available():
        V.build_ref()
    if not V.ref_available():
        pytest.skip("reference checkout not present")
    return "ref"
