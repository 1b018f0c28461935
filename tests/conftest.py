import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests" / "golden"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libsocgpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library on a GPU machine; builds it when stale."""
    import torch  # noqa: F401  (device plumbing on the GPU machine)
    from socrates_gb300 import build, radiance
    build.build()
    return radiance.load_library()
