import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference source tree (vulkpy): $VULKPY_REFERENCE_ROOT, else a
# directory named "reference" beside this repository.
REFERENCE_ROOT = os.environ.get("VULKPY_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def gpu():
    import vulkpy_gb300 as vk
    return vk.GPU()


@pytest.fixture(scope="session")
def reference_vk():
    """The reference's own Python package over the oracle's fake native
    module (only where the reference source tree is present)."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "vulkpy")):
        pytest.skip("reference source tree not available")
    from oracle.fake_vkarray import load_reference
    return load_reference(REFERENCE_ROOT)
