"""The C ABI surface: the library loads and exports every entry point that
include/raydar_cuda.h declares, and argument checks fail cleanly (no GPU needed)."""
import ctypes as C
import re

import pytest

from raydar_gb300 import native
from tests.conftest import ROOT


def _declared():
    text = (ROOT / "include" / "raydar_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rdc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = native.load()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), f"{n} not exported by libraydar_cuda.so"
        assert n in native.SIGNATURES, f"{n} has no ctypes signature"
    assert set(native.SIGNATURES) == set(names)


def test_the_rust_binding_declares_every_entry_point():
    """INTEGRATION.md's extern block (the FFI a maintainer adds on the Rust
    side) names every function the header declares, and nothing else."""
    text = (ROOT / "INTEGRATION.md").read_text()
    bound = set(re.findall(r"pub fn (rdc_[a-z0-9_]+)\(", text))
    assert bound == set(_declared())


def test_version_string():
    assert b"sm_103a" in native.load().rdc_version()


def test_create_on_a_missing_device_fails_with_a_message():
    lib = native.load()
    ctx = C.c_void_p()
    st = lib.rdc_create(C.byref(ctx), 999)
    assert st != native.RDC_OK and not ctx.value
    assert len(lib.rdc_last_error(None)) > 0


@pytest.mark.parametrize("name,args", [
    ("rdc_render", (None, 0, 1, 1, 0)),
    ("rdc_reset", (None,)),
    ("rdc_scene_upload", (None, None)),
    ("rdc_synchronize", (None,)),
])
def test_null_context_is_rejected(name, args):
    lib = native.load()
    assert getattr(lib, name)(*args) == 1  # RDC_ERR_INVALID_ARGUMENT


def test_destroy_accepts_null():
    native.load().rdc_destroy(None)


def test_camera_update_rejects_bad_input():
    lib = native.load()
    cam = native.RdcCamera()
    assert lib.rdc_camera_update_matrices(None) == 1
    assert lib.rdc_camera_update_matrices(C.byref(cam)) == 1  # zero resolution
