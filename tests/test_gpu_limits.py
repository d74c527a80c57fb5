"""The renderer at the limits the header states, against the CPU oracle.

- RDC_MAX_RESOLUTION per axis (16384 x 16384, 268 M pixels, a 4.3 GB
  accumulator): every pixel's sample count, the segment count against the
  oracle's over the same frame at 1 bounce, and a pixel sample (corners,
  edges, the last pixel, random ones) bit for bit at 3 bounces; the
  wavefront form at that size (one-sample waves of 2^28 paths, 23.6 GB of
  path records and queues) equal to the megakernel;
- RDC_MAX_BOUNCES (1024): paths that never escape a closed box run all their
  bounces, brute force, LBVH and the wavefront form, bit-identical to the
  oracle;
- RDC_MAX_BRUTE_OBJECTS (4096): brute force at the limit, its refusal one
  object above it, and the LBVH on the same scenes;
- RDC_MAX_OBJECTS (2^24): the LBVH build and traversal against the oracle's
  brute force on a ray sample.
"""
import numpy as np
import pytest

import oracle
from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from raydar_gb300.scene import Camera, Material, Object, Scene, World, resized
from tests.helpers import bits_equal

pytestmark = pytest.mark.gpu

SKY = World("SkyColor", np.array([0.53, 0.8, 0.92], np.float32), np.ones(3, np.float32))


def _render(scene, spp, bounces, seed, accel=native.ACCEL_AUTO):
    r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
    r._check(r.lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
    r.upload(scene)
    r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
    r.render_range(0, spp)
    acc, st = r.accumulator(scene), r.stats()
    r.close()
    return acc, st


def test_maximum_resolution():
    n = 16384
    scene = resized(scenegen.c1_plain().scene, n, n)
    acc, st = _render(scene, 1, 1, 31)
    assert acc.shape == (n, n, 4)
    assert np.all(acc[..., 3] == 1.0)
    _, segs = oracle.render(scene.to_c(), 0, 1, 1, 31, threads=16)
    assert st.segments == segs == n * n
    del acc
    acc, _ = _render(scene, 1, 3, 32)
    rng = np.random.default_rng(16384)
    edge = [0, n - 1, n * (n - 1), n * n - 1, n // 2 * n + n // 2, n - 2, n * n - 2]
    px = np.unique(np.concatenate([edge, rng.integers(0, n * n, 4000)])).astype(np.uint32)
    ref, _ = oracle.render_pixels(scene.to_c(), px, 0, 1, 3, 32)
    assert bits_equal(acc.reshape(-1, 4)[px], ref)


def test_wavefront_at_the_maximum_resolution():
    n = 16384
    scene = resized(scenegen.c2_default().scene, n, n)
    out = []
    for fn in ("rdc_render", "rdc_render_wavefront"):
        r = CudaRenderer(RendererConfig(max_bounces=2), seed=33)
        r.upload(scene)
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r._check(getattr(r.lib, fn)(r.ctx, 0, 1, 2, 33), fn)
        out.append((r.accumulator(scene), r.stats().segments))
        r.close()
    (a, sa), (b, sb) = out
    assert sa == sb and sa > n * n
    assert bits_equal(a, b)


def _closed_box(width=8, height=8):
    """A camera inside a large diffuse cube with a metal sphere: no ray escapes."""
    cam = Camera.new([0.0, 0.5, -2.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], width, height, 0.01, 1000.0, fov=70.0)
    objs = [Object("Cube", np.array([0.0, 0.0, 0.0], np.float32), 10.0,
                   Material(albedo=np.array([0.9, 0.85, 0.8], np.float32), roughness=1.0)),
            Object("Sphere", np.array([0.3, 0.0, 0.5], np.float32), 0.7,
                   Material(albedo=np.array([0.95, 0.95, 0.95], np.float32), roughness=0.1, metallic=1.0))]
    return Scene(cam, SKY, objs)


@pytest.mark.parametrize("accel", [native.ACCEL_BRUTE_FORCE, native.ACCEL_LBVH])
def test_maximum_bounces_in_a_closed_box(accel):
    scene = _closed_box()
    acc, st = _render(scene, 2, 1024, 41, accel)
    ref, segs = oracle.render(scene.to_c(), 0, 2, 1024, 41, threads=8)
    assert st.segments == segs == 8 * 8 * 2 * 1024
    assert bits_equal(acc, ref)


def test_maximum_bounces_in_the_wavefront_form():
    """1024 bounces through the LBVH at 5 samples: rdc_render takes the
    wavefront form (a graph of 2 x 1024 queue launches per wave)."""
    scene = _closed_box()
    acc, st = _render(scene, 5, 1024, 43, native.ACCEL_LBVH)
    assert st.kernel_launches > 2 * 1024
    ref, segs = oracle.render(scene.to_c(), 0, 5, 1024, 43, threads=8)
    assert st.segments == segs == 8 * 8 * 5 * 1024
    assert bits_equal(acc, ref)


def _sphere_grid(n, width=32, height=18):
    """n small spheres on a 64-wide grid, all materials, seen from above."""
    rng = np.random.default_rng(n)
    objs = []
    for i in range(n):
        gx, gz = i % 64, i // 64
        c = np.array([(gx - 31.5) * 0.3, 0.1 * (i % 3), (gz - 31.5) * 0.3], np.float32)
        kind = i % 4
        m = Material(albedo=rng.uniform(0.1, 0.9, 3).astype(np.float32),
                     roughness=(1.0, 0.5, 0.25, 0.0)[kind], metallic=1.0 if kind == 2 else 0.0,
                     transmission=1.0 if kind == 3 else 0.0)
        objs.append(Object("Sphere", c, float(np.float32(rng.uniform(0.05, 0.13))), m))
    cam = Camera.new([0.0, 14.0, -16.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], width, height, 0.01, 1000.0, fov=55.0)
    return Scene(cam, SKY, objs)


def test_brute_force_at_its_object_limit_and_the_lbvh_beside_it():
    scene = _sphere_grid(4096)
    ref, segs = oracle.render(scene.to_c(), 0, 1, 6, 51, threads=16)
    for accel in (native.ACCEL_BRUTE_FORCE, native.ACCEL_LBVH, native.ACCEL_AUTO):
        acc, st = _render(scene, 1, 6, 51, accel)
        assert st.accel == (native.ACCEL_BRUTE_FORCE if accel == native.ACCEL_BRUTE_FORCE else native.ACCEL_LBVH)
        assert st.segments == segs and bits_equal(acc, ref), accel


def test_brute_force_refuses_one_object_above_its_limit():
    scene = _sphere_grid(4097)
    r = CudaRenderer(RendererConfig(max_bounces=4), seed=1)
    r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_BRUTE_FORCE), "rdc_set_accel")
    st_up = r.lib.rdc_scene_upload(r.ctx, scene.to_c().ref())
    st_r = r.lib.rdc_render(r.ctx, 0, 1, 4, 1) if st_up == 0 else st_up
    r.close()
    assert st_r == 3  # RDC_ERR_LIMIT
    ref, segs = oracle.render(scene.to_c(), 0, 1, 4, 2, threads=16)
    acc, st = _render(scene, 1, 4, 2, native.ACCEL_AUTO)
    assert st.accel == native.ACCEL_LBVH and st.segments == segs and bits_equal(acc, ref)


def test_lbvh_at_the_object_limit():
    """RDC_MAX_OBJECTS (2^24) objects in the config-5 volume: the device
    build (its radix sort and prefix sums at their largest) and the traversal
    give the brute-force closest hit of the oracle on a ray sample."""
    from tests.test_gpu_bvh import _intersect, _ray_sample
    n_obj = 1 << 24
    w = scenegen.c5_large(seed=24, width=64, height=36, n_spheres=n_obj - (1 << 20), n_cubes=1 << 20)
    r = CudaRenderer(RendererConfig(), seed=0)
    r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_LBVH), "set_accel")
    r.upload(w.scene)
    st = r.stats()
    assert st.accel == native.ACCEL_LBVH and 0 < st.bvh_depth <= 64
    o, d = _ray_sample(w.scene, w.scene.packed, 24, np.random.default_rng(24))  # the oracle: ~0.4 s a ray
    got = _intersect(r, o, d)
    r.close()
    ref = oracle.intersect(w.scene.to_c(), o, d)
    for g, e in zip(got, ref):
        assert bits_equal(g, e)
    assert (got[1] >= 0).sum() > 12  # most rays hit something in a volume this dense
