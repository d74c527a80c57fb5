"""CUDA path vs the CPU oracle, through the C ABI.

Both sides draw the same Philox words for (seed, pixel, sample, bounce), both
evaluate the reference's float expressions in the reference's order without
FMA contraction, so the bar is bit equality: accumulators, hit t / normal /
index and scattered rays are compared byte for byte (stricter than the
1e-5 relative / 4 ulp tolerances the path is specified with).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from raydar_gb300 import native, scenegen
from raydar_gb300.scene import Scene
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _render_gpu(r, scene, s0, n, bounces, seed):
    r.seed = seed
    r.config.max_bounces = bounces
    r.upload(scene)
    r._check(r.lib.rdc_reset(r.ctx), "reset")
    r.render_range(s0, n)
    acc = r.accumulator(scene)
    return acc, r.stats().segments


def _ortho(scene, size):
    """The same scene seen through Projection::Orthographic (src/scene/camera.rs:8-11, 218-225)."""
    import copy
    s = copy.deepcopy(scene)
    s.camera.projection = "Orthographic"
    s.camera.size = float(np.float32(size))
    s.camera.update_matrices()
    return s


def _solid(scene):
    """World::SolidColor (src/scene/world.rs:6-14, 31)."""
    import copy

    from raydar_gb300.scene import World
    s = copy.deepcopy(scene)
    s.world = World("SolidColor", color=np.array([0.25, 0.5, 0.75], np.float32))
    return s


SCENES = {
    "c1_64x36": lambda: shrink(scenegen.c1_plain().scene, 64, 36),
    "c2_96x54": lambda: shrink(scenegen.c2_default().scene, 96, 54),
    "c4_48x48": lambda: shrink(scenegen.c4_diff().scene, 48, 48),
    "c2_ortho_96x54": lambda: _ortho(shrink(scenegen.c2_default().scene, 96, 54), 14.0),
    "c1_solid_world_64x36": lambda: _solid(shrink(scenegen.c1_plain().scene, 64, 36)),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_render_matches_oracle_bitwise(renderer, name):
    scene = SCENES[name]()
    acc, seg = _render_gpu(renderer, scene, 0, 4, 8, seed=1234)
    ref, ref_seg = oracle.render(scene.to_c(), 0, 4, 8, 1234, threads=8)
    assert seg == ref_seg
    diff = np.argwhere(acc.view(np.uint32) != ref.view(np.uint32))
    assert bits_equal(acc, ref), f"{len(diff)} channels differ, first {diff[:5].tolist()}"


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_reference_scenes_match_oracle_bitwise(renderer, golden_dir, name):
    scene = shrink(Scene.load(golden_dir / f"{name}.rscn"), 80, 45)
    acc, seg = _render_gpu(renderer, scene, 0, 3, 12, seed=7)
    ref, ref_seg = oracle.render(scene.to_c(), 0, 3, 12, 7, threads=8)
    assert seg == ref_seg
    assert bits_equal(acc, ref)


def test_progressive_split_is_bit_identical(renderer):
    scene = shrink(scenegen.c1_plain().scene, 40, 24)
    full, sf = _render_gpu(renderer, scene, 0, 5, 8, seed=3)
    renderer._check(renderer.lib.rdc_reset(renderer.ctx), "reset")
    renderer.render_range(0, 2)
    s1 = renderer.stats().segments
    renderer.render_range(2, 3)
    s2 = renderer.stats().segments
    assert bits_equal(renderer.accumulator(scene), full) and s1 + s2 == sf


def test_render_sample_loop_matches_render_frame():
    from raydar_gb300 import CudaRenderer, RendererConfig
    scene = shrink(scenegen.c1_plain().scene, 32, 18)
    a = CudaRenderer(RendererConfig(max_sample_count=4, max_bounces=8), seed=11)
    b = CudaRenderer(RendererConfig(max_sample_count=4, max_bounces=8), seed=11)
    img = a.render_frame(scene)
    b.new_frame(scene)
    last = None
    while True:
        nxt = b.render_sample(scene)
        if nxt is None:
            break
        last = nxt
    assert b.sample_count() == 4 and bits_equal(last, img)
    ref, _ = oracle.render(scene.to_c(), 0, 4, 8, 11)
    assert bits_equal(img, oracle.tonemap(ref, 4))
    a.close()
    b.close()


def _random_rays(scene, n, rng):
    o = rng.uniform(-8, 8, (n, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(0.05, 5, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    # axis-aligned directions (zero components) and unnormalised ones
    d[: n // 16] = np.array([0, -1, 0], np.float32)
    d[n // 16: n // 8, 0] = 0.0
    d[n // 8: n // 4] *= np.float32(3.0)
    return o, d


@pytest.mark.parametrize("name", ["c2_96x54", "c4_48x48"])
def test_fixed_ray_batch_intersection_matches_oracle(renderer, name):
    scene = SCENES[name]()
    renderer.upload(scene)
    rng = np.random.default_rng(42)
    n = 1 << 16
    o, d = _random_rays(scene, n, rng)
    t = np.zeros(n, np.float32)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), np.float32)
    fr = np.zeros(n, np.uint8)
    st = renderer.lib.rdc_intersect_rays(renderer.ctx, native.fptr(o), native.fptr(d), n, native.fptr(t),
                                         native.iptr(idx), native.fptr(nrm), native.u8ptr(fr))
    assert st == 0
    rt, ridx, rn, rf = oracle.intersect(scene.to_c(), o, d)
    assert np.array_equal(idx, ridx)
    assert (idx >= 0).mean() > 0.3
    assert bits_equal(t, rt) and bits_equal(nrm, rn) and np.array_equal(fr, rf)


def test_borderline_rays_match_oracle(renderer, golden_dir):
    """Rays on which one ulp decides the hit, taken from renders of the
    reference's benchmark scene: a primary ray tangent to sphere 24
    (discriminant exactly 0) and a ray leaving sphere 8 whose c term cancels to
    -8e-7.  A packed multiply fused into the following add (one rounding
    instead of two) drops both hits; the kernels must match the oracle here."""
    scene = shrink(Scene.load(golden_dir / "benchmark.rscn"), 80, 45)
    renderer.upload(scene)
    o = np.array([[-10.082242965698242, 4.5850090980529785, -10.082204818725586],
                  [-0.2938964068889618, 0.652721107006073, -3.8709042072296143]], np.float32)
    d = np.array([[0.907118022441864, -0.2591124475002289, 0.3316586911678314],
                  [-0.6680339574813843, -0.1301172971725464, 0.7326664924621582]], np.float32)
    n = len(o)
    t = np.zeros(n, np.float32)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), np.float32)
    fr = np.zeros(n, np.uint8)
    assert renderer.lib.rdc_intersect_rays(renderer.ctx, native.fptr(o), native.fptr(d), n, native.fptr(t),
                                           native.iptr(idx), native.fptr(nrm), native.u8ptr(fr)) == 0
    rt, ridx, rn, rf = oracle.intersect(scene.to_c(), o, d)
    assert ridx.tolist() == [24, 8]
    assert np.array_equal(idx, ridx) and bits_equal(t, rt) and bits_equal(nrm, rn)


def test_fixed_uniform_scatter_matches_oracle(renderer):
    scene = SCENES["c2_96x54"]()
    renderer.upload(scene)
    rng = np.random.default_rng(5)
    n = 1 << 15
    o, d = _random_rays(scene, n, rng)
    rt, ridx, _, _ = oracle.intersect(scene.to_c(), o, d)
    hit = ridx >= 0
    o, d, rt, ridx = o[hit], d[hit], rt[hit], ridx[hit]
    n = len(o)
    words = rng.integers(0, 2 ** 32, (n, 12), dtype=np.uint64).astype(np.uint32)
    oo = np.zeros((n, 3), np.float32)
    do = np.zeros((n, 3), np.float32)
    st = renderer.lib.rdc_scatter_fixed(renderer.ctx, native.fptr(np.ascontiguousarray(o)),
                                        native.fptr(np.ascontiguousarray(d)), native.fptr(np.ascontiguousarray(rt)),
                                        native.iptr(np.ascontiguousarray(ridx)), native.uptr(words), n,
                                        native.fptr(oo), native.fptr(do))
    assert st == 0
    ro, rd = oracle.scatter(scene.to_c(), o, d, rt, ridx, words)
    assert bits_equal(oo, ro) and bits_equal(do, rd)


def test_tonemap_matches_oracle(renderer):
    scene = SCENES["c1_64x36"]()
    acc, _ = _render_gpu(renderer, scene, 0, 3, 8, seed=2)
    renderer._sample_count = 3
    img = renderer.image(scene)
    assert bits_equal(img, oracle.tonemap(acc, 3))


def test_full_1080p_properties_and_spot_pixels(renderer):
    """configs[1] size (1920x1080, 12 bounces): one sample per pixel, checked by
    size-independent properties and 256 random pixels replayed by the oracle."""
    scene = scenegen.c2_default().scene
    acc, seg = _render_gpu(renderer, scene, 0, 2, 12, seed=99)
    npix = 1920 * 1080
    assert np.all(acc[..., 3] == 2.0)
    assert 2 * npix <= seg <= 2 * npix * 12
    assert np.isfinite(acc).all()
    px = np.random.default_rng(0).choice(npix, 256, replace=False).astype(np.uint32)
    ref, _ = oracle.render_pixels(scene.to_c(), px, 0, 2, 12, 99)
    assert bits_equal(acc.reshape(-1, 4)[px], ref)
    again, seg2 = _render_gpu(renderer, scene, 0, 2, 12, seed=99)
    assert bits_equal(again, acc) and seg2 == seg


def test_converged_image_matches_independent_oracle_stream(renderer):
    """Statistical parity with independent random streams (the reference's own
    RNG is unseeded, so this is how its converged image is compared): GPU
    64 seeds x 256 spp vs the oracle 32 other seeds x 512 spp, batch means
    combined in float64.  Per pixel and channel |difference| within 3 sigma of
    the batch variance for all but 1% (and none beyond 6 sigma); relative
    MSE < 1e-4.  The sigma floor 3e-5*|mean| covers float32 running-sum
    rounding inside one batch, which is all that varies on zero-variance
    pixels (no pixel jitter: a sky pixel's samples are all equal)."""
    scene = shrink(scenegen.c1_plain().scene, 40, 24)
    gpu = []
    for k in range(64):
        acc, _ = _render_gpu(renderer, scene, 0, 256, 8, seed=1000 + k)
        gpu.append(acc[..., :3].astype(np.float64) / 256)
    cpu = []
    for k in range(32):
        acc, _ = oracle.render(scene.to_c(), 0, 512, 8, 5000 + k, threads=16)
        cpu.append(acc[..., :3].astype(np.float64) / 512)
    gpu, cpu = np.array(gpu), np.array(cpu)
    gm, om = gpu.mean(0), cpu.mean(0)
    sigma = np.sqrt(gpu.var(0, ddof=1) / len(gpu) + cpu.var(0, ddof=1) / len(cpu)) + 3e-5 * np.abs(om) + 1e-7
    z = np.abs(gm - om) / sigma
    assert (z > 3).mean() < 0.01 and z.max() < 6, float(z.max())
    rel_mse = ((gm - om) ** 2).mean() / (om ** 2).mean()
    assert rel_mse < 1e-4, rel_mse


def test_scene_errors(renderer):
    lib = renderer.lib
    ctx = renderer.ctx
    assert lib.rdc_render(ctx, 0, 1, 1, 0) == 4  # RDC_ERR_NO_SCENE
    scene = shrink(scenegen.c1_plain().scene, 8, 8)
    scene.world.kind = "Transparent"
    sc = scene.to_c()
    assert lib.rdc_scene_upload(ctx, sc.ref()) == 2  # RDC_ERR_UNSUPPORTED
    assert b"Transparent" in lib.rdc_last_error(ctx)
    scene.world.kind = "SkyColor"
    sc = scene.to_c()
    sc.desc.object_count = native.MAX_OBJECTS + 1
    assert lib.rdc_scene_upload(ctx, sc.ref()) == 3  # RDC_ERR_LIMIT
    sc = scene.to_c()
    sc.desc.camera.resolution_x = 0
    assert lib.rdc_scene_upload(ctx, sc.ref()) == 1
    sc = scene.to_c()
    assert lib.rdc_scene_upload(ctx, sc.ref()) == 0
    assert lib.rdc_render(ctx, 0, 1, 2000, 0) == 3  # bounces above RDC_MAX_BOUNCES
    small = np.zeros(10, np.float32)
    assert lib.rdc_read_accum(ctx, native.fptr(small), small.size) == 1


def test_zero_objects_and_zero_bounces(renderer):
    scene = shrink(scenegen.c1_plain().scene, 16, 9)
    scene.objects = []
    acc, seg = _render_gpu(renderer, scene, 0, 2, 4, seed=1)
    ref, rseg = oracle.render(scene.to_c(), 0, 2, 4, 1)
    assert bits_equal(acc, ref) and seg == rseg == 16 * 9 * 2
    scene = shrink(scenegen.c1_plain().scene, 16, 9)
    acc, seg = _render_gpu(renderer, scene, 0, 3, 0, seed=1)
    assert seg == 0 and np.all(acc[..., :3] == 0) and np.all(acc[..., 3] == 3)


def test_device_min_max_signed_zero_semantics(renderer):
    """The oracle resolves fmin(-0,+0) to -0 and fmax(-0,+0) to +0; the cube
    slab test on the GPU uses fminf/fmaxf.  A cube whose face plane contains
    the ray origin produces t = +-0 on that axis: both sides must agree."""
    from raydar_gb300.scene import Camera, Material, Object, World
    cam = Camera.new([0, 0, -5], [0, 0, 0], [0, 1, 0], 4, 4, 0.01, 1000.0)
    scene = Scene(cam, World(), [Object("Cube", np.array([1, 1, 1], np.float32), 2.0, Material())])
    renderer.upload(scene)
    o = np.array([[0, 0, 0], [0, 0, 0], [2, 2, 2], [0, 1, 1]], np.float32)
    d = np.array([[1, 1, 1], [-1, -1, -1], [-1, 0, 0], [1, 0, 0]], np.float32)
    n = len(o)
    t = np.zeros(n, np.float32)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), np.float32)
    fr = np.zeros(n, np.uint8)
    assert renderer.lib.rdc_intersect_rays(renderer.ctx, native.fptr(o), native.fptr(d), n, native.fptr(t),
                                           native.iptr(idx), native.fptr(nrm), native.u8ptr(fr)) == 0
    rt, ridx, rn, rf = oracle.intersect(scene.to_c(), o, d)
    assert np.array_equal(idx, ridx) and bits_equal(t, rt) and bits_equal(nrm, rn)


def test_staging_wait_limit_reports_a_device_error_and_the_context_survives(renderer):
    """The shared-memory staging wait gives up after its bounded polls (here on
    a barrier nothing completes): RDC_ERR_DEVICE comes back once, then the
    context renders bit-identically to the oracle again."""
    st = renderer.lib.rdc_selftest_staging_timeout(renderer.ctx)
    assert st == 7, st  # RDC_ERR_DEVICE
    assert b"shared memory" in renderer.lib.rdc_last_error(renderer.ctx)
    scene = SCENES["c1_64x36"]()
    acc, seg = _render_gpu(renderer, scene, 0, 2, 8, seed=77)
    ref, ref_seg = oracle.render(scene.to_c(), 0, 2, 8, 77, threads=8)
    assert seg == ref_seg and bits_equal(acc, ref)
