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


@pytest.fixture(params=["megakernel", "wavefront"])
def renderer(request):
    """A CudaRenderer on device 0 (gpu tests only) whose rdc_render is held to
    one form, so the parity tests run through the megakernel and through the
    wavefront form alike (RDC_FORM_AUTO would pick the wavefront for most of
    their small images)."""
    from raydar_gb300 import CudaRenderer, RendererConfig, native
    r = CudaRenderer(RendererConfig(), device=0, seed=0)
    form = native.FORM_MEGAKERNEL if request.param == "megakernel" else native.FORM_WAVEFRONT
    r._check(r.lib.rdc_set_render_form(r.ctx, form), "rdc_set_render_form")
    yield r
    r.close()
