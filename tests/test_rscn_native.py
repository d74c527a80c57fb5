"""The library's .rscn reader and writer (rdc_scene_parse_rscn /
rdc_scene_write_rscn, C++) against the Python loader: the reference's own
scene files read to the same bytes, and written scenes read back unchanged.
No GPU is involved."""
import ctypes as C
import json

import numpy as np
import pytest

from raydar_gb300 import native, scenegen
from raydar_gb300.scene import Scene


@pytest.fixture(scope="module")
def lib():
    return native.load()


def _parse(lib, text: bytes):
    desc = native.RdcSceneDesc()
    n = C.c_uint32(0)
    st = lib.rdc_scene_parse_rscn(text, len(text), C.byref(desc), None, 0, C.byref(n))
    if st != 0:
        return st, None, None
    objs = (native.RdcObject * max(n.value, 1))()
    st = lib.rdc_scene_parse_rscn(text, len(text), C.byref(desc), objs, n.value, C.byref(n))
    return st, desc, objs


def _write(lib, desc) -> bytes:
    ln = C.c_size_t(0)
    assert lib.rdc_scene_write_rscn(C.byref(desc), None, 0, C.byref(ln)) == 0
    buf = C.create_string_buffer(ln.value + 1)
    assert lib.rdc_scene_write_rscn(C.byref(desc), buf, ln.value + 1, C.byref(ln)) == 0
    return buf.raw[: ln.value]


def _camera_bytes(cam):
    """The camera without the inactive projection parameter (the reference's
    Projection enum holds only fov or only size)."""
    c = native.RdcCamera.from_buffer_copy(bytes(cam))
    if c.projection == native.PROJECTION_PERSPECTIVE:
        c.ortho_size = 0.0
    else:
        c.fov_degrees = 0.0
    return bytes(c)


def _world_bytes(w):
    """The world without the colours its variant does not hold."""
    c = native.RdcWorld.from_buffer_copy(bytes(w))
    if c.kind != native.WORLD_SKY_COLOR:
        c.top_color[:] = [0.0] * 3
        c.bottom_color[:] = [0.0] * 3
    if c.kind != native.WORLD_SOLID_COLOR:
        c.solid_color[:] = [0.0] * 3
    return bytes(c)


def _same(desc, objs, sc):
    assert _camera_bytes(desc.camera) == _camera_bytes(sc.desc.camera)
    assert _world_bytes(desc.world) == _world_bytes(sc.desc.world)
    assert desc.object_count == sc.desc.object_count
    n = sc.desc.object_count * C.sizeof(native.RdcObject)
    assert bytes(objs)[:n] == bytes(sc.objects)[:n]


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_reference_scene_files_read_like_the_python_loader(lib, golden_dir, name):
    text = (golden_dir / f"{name}.rscn").read_bytes()
    st, desc, objs = _parse(lib, text)
    assert st == 0, lib.rdc_last_error(None)
    _same(desc, objs, Scene.load(golden_dir / f"{name}.rscn").to_c())


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_written_scene_reads_back_unchanged(lib, golden_dir, name, tmp_path):
    st, desc, objs = _parse(lib, (golden_dir / f"{name}.rscn").read_bytes())
    out = _write(lib, desc)
    json.loads(out)  # valid JSON
    st2, desc2, objs2 = _parse(lib, out)
    assert st2 == 0
    assert bytes(desc2.camera) == bytes(desc.camera) and bytes(desc2.world) == bytes(desc.world)
    assert bytes(objs2) == bytes(objs)
    p = tmp_path / "s.rscn"
    p.write_bytes(out)
    _same(desc, objs, Scene.load(p).to_c())  # the Python loader reads the C++ output


def test_generated_scene_with_ortho_and_solid_world_round_trips(lib, tmp_path):
    from raydar_gb300.scene import World
    s = scenegen.c1_plain().scene
    s.camera.projection = "Orthographic"
    s.camera.size = 7.25
    s.camera.update_matrices()
    s.world = World("SolidColor", color=np.array([0.1, 0.2, 1e-7], np.float32))
    sc = s.to_c()
    out = _write(lib, sc.desc)
    st, desc, objs = _parse(lib, out)
    assert st == 0
    _same(desc, objs, sc)
    p = tmp_path / "g.rscn"
    s.save(p)
    st, desc, objs = _parse(lib, p.read_bytes())
    assert st == 0
    _same(desc, objs, sc)


@pytest.mark.parametrize("text", [b"", b"{", b"[]", b'{"camera": 1}', b'{"camera":{},"world":"Transparent","objects":[]}',
                                  b"{} x"])
def test_malformed_input_is_rejected_with_a_message(lib, text):
    st, _, _ = _parse(lib, text)
    assert st == 1  # RDC_ERR_INVALID_ARGUMENT
    assert len(lib.rdc_last_error(None)) > 0


def test_capacity_below_count_is_a_limit_error(lib, golden_dir):
    text = (golden_dir / "benchmark.rscn").read_bytes()
    desc = native.RdcSceneDesc()
    n = C.c_uint32(0)
    objs = (native.RdcObject * 4)()
    assert lib.rdc_scene_parse_rscn(text, len(text), C.byref(desc), objs, 4, C.byref(n)) == 3
    assert n.value == 183
