"""Shared fixtures.  Tests marked `gpu` need a CUDA GPU; the rest run on CPU.

The native library and the CPU oracle are (re)built once per session when a
source is newer than the build (nvcc cross-compiles without a GPU).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _native_built():
    from raydar_gb300 import build
    build.build_all()


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


@pytest.fixture()
def renderer():
    """A CudaRenderer on device 0 (gpu tests only)."""
    from raydar_gb300 import CudaRenderer, RendererConfig
    r = CudaRenderer(RendererConfig(), device=0, seed=0)
    yield r
    r.close()
