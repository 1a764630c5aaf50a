import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


# The Nyx source tree, for the few CPU tests that read its own input files: its
# location comes from the NYX_REFERENCE environment variable; without it those
# tests are skipped.
REFERENCE_TREE = os.environ.get("NYX_REFERENCE") or None


def reference_file(*parts):
    """Path of a file inside the Nyx source tree, or None when NYX_REFERENCE is
    unset or the file is absent."""
    if not REFERENCE_TREE:
        return None
    p = os.path.join(REFERENCE_TREE, *parts)
    return p if os.path.exists(p) else None


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    if not gpu_available():
        pytest.skip("no GPU")
    from nyx_gb300.pm import Context
    c = Context()
    yield c
    c.close()
