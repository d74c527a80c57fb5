"""rdc_render_static, the entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (device memory owned by an
engine or interop layer, allocation-free real-time loops, fixed-budget
plugins): they own the accumulator and pass a device pointer; the library's
scratch is a fixed device array.  This test plays such a caller (torch
allocates the caller's accumulator) and checks, through the C ABI, that two
calls in a row give bit-identical accumulators and segment counts to the
context entry points (rdc_scene_upload + rdc_render) -- the bar every other
parity test here uses.  The second call also proves the shared counters are
cleared between calls.  Collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _static_call(lib, sc, accum_ptr, s0, n, bounces, seed, stream):
    segs = C.c_uint64(0)
    err = C.create_string_buffer(512)
    st = lib.rdc_render_static(sc.ref(), C.c_void_p(accum_ptr), s0, n, bounces, seed, C.c_void_p(stream),
                               C.byref(segs), err, len(err))
    return st, segs.value, err.value.decode()


def test_static_render_matches_context_render_twice():
    torch = pytest.importorskip("torch")
    lib = native.load()
    scene = shrink(scenegen.c2_default().scene, 160, 90)
    bounces, seed = 12, 4242

    # Existing entry points: a context that allocates its own memory.
    r = CudaRenderer(RendererConfig(max_bounces=bounces), device=0, seed=seed)
    r.upload(scene)
    r._check(lib.rdc_reset(r.ctx), "rdc_reset")
    r.render_range(0, 3)
    ref1, seg1 = r.accumulator(scene), r.stats().segments
    r.render_range(3, 2)
    ref2, seg2 = r.accumulator(scene), r.stats().segments
    r.close()

    # The no-allocation entry point, fed a caller-owned device accumulator.
    torch.cuda.set_device(0)
    acc = torch.zeros(scene.height * scene.width * 4, dtype=torch.float32, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    sc = scene.to_c()
    st, s1, msg = _static_call(lib, sc, acc.data_ptr(), 0, 3, bounces, seed, stream)
    assert st == 0, msg
    out1 = acc.cpu().numpy().reshape(scene.height, scene.width, 4)
    st, s2, msg = _static_call(lib, sc, acc.data_ptr(), 3, 2, bounces, seed, stream)
    assert st == 0, msg
    out2 = acc.cpu().numpy().reshape(scene.height, scene.width, 4)

    assert s1 == seg1 and s2 == seg2
    assert bits_equal(out1, ref1)
    assert bits_equal(out2, ref2)
    assert np.all(out2[..., 3] == 5.0)


def test_static_render_rejects_scenes_beyond_its_fixed_scratch():
    torch = pytest.importorskip("torch")
    lib = native.load()
    scene = shrink(scenegen.c1_plain().scene, 8, 8)
    sc = scene.to_c()
    acc = torch.zeros(8 * 8 * 4, dtype=torch.float32, device="cuda:0")
    sc.desc.object_count = 1025  # above RDC_STATIC_MAX_OBJECTS; nothing is read past the real array
    st, _, msg = _static_call(lib, sc, acc.data_ptr(), 0, 1, 4, 1, 0)
    assert st == 3 and "RDC_STATIC_MAX_OBJECTS" in msg


def _alternating_scene(n=1024, width=48, height=27):
    """n objects alternating sphere / cube (every run one object long: the
    densest flattened layout, 3.5 intersection records per object) on a
    32 x 32 grid, seen from above at an angle."""
    from raydar_gb300.scene import Camera, Material, Object, Scene, World
    rng = np.random.default_rng(1024)
    objs = []
    for i in range(n):
        gx, gz = i % 32, i // 32
        c = np.array([(gx - 15.5) * 0.6, 0.2, (gz - 15.5) * 0.6], np.float32)
        kind = "ABCD"[i % 4]
        m = Material(albedo=rng.uniform(0.1, 0.9, 3).astype(np.float32),
                     roughness={"A": 1.0, "B": 0.5, "C": 0.2, "D": 0.0}[kind],
                     metallic=1.0 if kind == "C" else 0.0, transmission=1.0 if kind == "D" else 0.0)
        if i % 2 == 0:
            objs.append(Object("Sphere", c, float(np.float32(rng.uniform(0.1, 0.28))), m))
        else:
            objs.append(Object("Cube", c, float(np.float32(rng.uniform(0.15, 0.5))), m))
    cam = Camera.new([0.0, 9.0, -14.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], width, height, 0.01, 1000.0, fov=50.0)
    return Scene(cam, World("SkyColor", np.array([0.53, 0.8, 0.92], np.float32), np.ones(3, np.float32)), objs)


def test_static_render_of_the_densest_layout_matches_context_render():
    """1024 objects alternating sphere / cube fill the fixed scratch's record
    region to its worst case; the render must equal the context's brute-force
    render bit for bit, on two calls in a row."""
    torch = pytest.importorskip("torch")
    lib = native.load()
    scene = _alternating_scene()
    bounces, seed = 8, 99
    r = CudaRenderer(RendererConfig(max_bounces=bounces), device=0, seed=seed)
    r._check(lib.rdc_set_accel(r.ctx, native.ACCEL_BRUTE_FORCE), "rdc_set_accel")
    r.upload(scene)
    r._check(lib.rdc_reset(r.ctx), "rdc_reset")
    r.render_range(0, 2)
    ref1, seg1 = r.accumulator(scene), r.stats().segments
    r.render_range(2, 1)
    ref2, seg2 = r.accumulator(scene), r.stats().segments
    r.close()

    torch.cuda.set_device(0)
    acc = torch.zeros(scene.height * scene.width * 4, dtype=torch.float32, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    sc = scene.to_c()
    st, s1, msg = _static_call(lib, sc, acc.data_ptr(), 0, 2, bounces, seed, stream)
    assert st == 0, msg
    out1 = acc.cpu().numpy().reshape(scene.height, scene.width, 4)
    st, s2, msg = _static_call(lib, sc, acc.data_ptr(), 2, 1, bounces, seed, stream)
    assert st == 0, msg
    out2 = acc.cpu().numpy().reshape(scene.height, scene.width, 4)
    assert (s1, s2) == (seg1, seg2)
    assert bits_equal(out1, ref1) and bits_equal(out2, ref2)
