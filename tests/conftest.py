import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


@pytest.fixture(scope="session")
def host_built():
    from farm_gb300 import build
    build.build_host()
    build.build_oracle()
    return True


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib(host_built):
    if not _cuda_available():
        pytest.fail("GPU test on a machine without CUDA")
    from farm_gb300 import build
    build.build_cuda()
    from farm_gb300 import _native
    return _native.gpu()
