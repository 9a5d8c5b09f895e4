import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libquantr_gpu")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library on a GPU machine; a missing build or device fails the test loudly."""
    from quantr_gb300 import _native

    if not _native.LIB_PATH.exists():
        from quantr_gb300 import build

        build.build()
    return _native.load()
