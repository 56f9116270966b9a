import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _have_gpu():
    try:
        import voro_gb300 as vg
        return vg.device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """Skips nothing: a gpu-marked test that finds no GPU fails loudly."""
    import voro_gb300 as vg
    n = vg.device_count()
    assert n > 0, "no CUDA device visible to the engine"
    return n
