import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _reference_path():
    """The reference checkout: $CLIFFS_REFERENCE, else the `reference_path`
    recorded beside the benchmark description at the repository root, else
    none (the GPU hosts have no checkout)."""
    env = os.environ.get("CLIFFS_REFERENCE")
    if env:
        return env
    p = os.path.join(ROOT, "BASELINE.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                return json.load(f).get("reference_path")
        except (OSError, ValueError):
            return None
    return None


REFERENCE = _reference_path()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def reference_dir():
    """The reference checkout; present only in the build container."""
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "Examples")):
        pytest.skip("reference checkout not present on this host")
    return REFERENCE
