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


@pytest.fixture(params=["scan", "phased"])
def kernel(request, gpu_lib):
    """Runs a test on each clear-sky kernel family: the scan kernels (the
    built-in tile) and the phased kernel (lanes_per_solve = 1), for both
    precisions and the no-scatter and full-scattering modes."""
    lanes, warps = (1, 8) if request.param == "phased" else (0, 0)
    for prec in (0, 1):
        for mode in (0, 1):
            assert gpu_lib.socgpu_set_tile_config(prec, mode, lanes, warps) == 0
    yield request.param
    for prec in (0, 1):
        for mode in (0, 1):
            gpu_lib.socgpu_set_tile_config(prec, mode, 0, 0)
