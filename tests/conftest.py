import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


from oracle.ref_f2c import reference_dir as _reference_dir  # noqa: E402

# the reference checkout ($CLIFFS_REFERENCE or the recipe's default), present
# only in the build container
REFERENCE = _reference_dir("Examples")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def reference_dir():
    """The reference checkout; present only in the build container."""
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "Examples")):
        pytest.skip("reference checkout not present on this host")
    return REFERENCE
