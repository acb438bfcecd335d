import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built libbrr_gpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load libbrr_gpu.so; fail loudly when it cannot be built."""
    from bayesrrcmd_gb300.build import build_gpu
    from bayesrrcmd_gb300 import gpu
    build_gpu()
    return gpu.load_library()
