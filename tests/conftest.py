import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def native_lib():
    from quicksilver_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def has_gpu(native_lib):
    from quicksilver_gb300 import _native
    return _native.device_count() > 0


@pytest.fixture
def gpu(has_gpu):
    if not has_gpu:
        pytest.fail("GPU test selected but no CUDA device is visible")
