import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


REFERENCE_ROOT = os.environ.get("NGP_REFERENCE_ROOT", "/root/reference")


@pytest.fixture(scope="session")
def ref_backend():
    """The reference's own kernels compiled for the CPU (only where the checkout exists)."""
    from oracle import volrend as V
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "deps", "volume-rendering-jax")):
        pytest.skip("reference checkout not present")
    if not V.ref_available():
        V.build_ref(REFERENCE_ROOT)
    return "ref"
