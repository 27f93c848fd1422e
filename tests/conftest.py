import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the CUDA library and the oracle once per session (no-op when up to date)."""
    import __graft_entry__

    __graft_entry__.build()


@pytest.fixture(scope="session")
def anchors():
    with open(os.path.join(ROOT, "tests", "golden", "anchors.json")) as f:
        return json.load(f)


def has_gpu() -> bool:
    try:
        import flock_gb300

        return flock_gb300.load().flock_gb300_device_count() > 0
    except Exception:
        return False
