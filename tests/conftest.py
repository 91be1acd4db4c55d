import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA kernels)")


def _gpu_available() -> bool:
    try:
        import pdl_gb300 as P
        return P.device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not _gpu_available():
        pytest.fail("a -m gpu test ran without a usable GPU (or libpdlgb300.so failed to load)")
    import pdl_gb300 as P
    return P
