"""Randomised parity: seeded scenes of every shape the scene model allows,
rendered by each GPU form and compared with the oracle bit for bit.

Each scene draws 1-300 objects (spheres and cubes in random runs, sizes over
three orders of magnitude, some overlapping or enclosing the camera),
materials at and between their extreme values (roughness and metallic 0 or
1, glass with IOR below and above 1, emission), a perspective or
orthographic camera anywhere around them and a sky or solid world.  Every
scene is rendered by the brute-force kernel (when it fits shared memory),
the LBVH kernel and the wavefront form; all must equal the oracle's
accumulator and segment count."""
import numpy as np
import pytest

import oracle
from raydar_gb300 import CudaRenderer, RendererConfig, native
from raydar_gb300.scene import Camera, Material, Object, Scene, World
from tests.helpers import bits_equal

pytestmark = pytest.mark.gpu

N_SCENES = 1000


def _random_scene(seed):
    rng = np.random.default_rng(seed)
    f32 = np.float32
    n = int(rng.choice([1, 2, 3, 7, 31, 64, 150, 300]))
    objs = []
    geom = "Sphere" if rng.random() < 0.5 else "Cube"
    for i in range(n):
        if rng.random() < 0.3:  # runs of one kind, switching now and then
            geom = "Cube" if geom == "Sphere" else "Sphere"
        c = rng.normal(scale=rng.choice([0.5, 3.0, 20.0]), size=3).astype(f32)
        size = float(f32(np.exp(rng.uniform(np.log(0.01), np.log(5.0)))))
        kind = rng.integers(0, 6)
        m = Material(albedo=rng.uniform(0, 1, 3).astype(f32))
        if kind == 0:
            m.roughness, m.metallic = float(f32(rng.choice([0.0, 1.0, rng.uniform()]))), 0.0
        elif kind == 1:
            m.roughness, m.metallic = float(f32(rng.choice([0.0, rng.uniform(0, 0.5)]))), 1.0
        elif kind == 2:
            m.transmission, m.roughness = 1.0, float(f32(rng.choice([0.0, rng.uniform(0, 0.3)])))
            m.ior = float(f32(rng.choice([1.5, 1.0, 0.7, 2.4])))
        elif kind == 3:
            m.emission_color = rng.uniform(0, 1, 3).astype(f32)
            m.emission_strength = float(f32(rng.uniform(0, 8)))
        elif kind == 4:
            m.transmission = float(f32(rng.uniform()))  # partly transmissive
            m.metallic = float(f32(rng.uniform()))
        objs.append(Object(geom, c, size, m))
    pos = rng.normal(scale=rng.choice([1.0, 8.0, 30.0]), size=3).astype(f32)
    tgt = rng.normal(scale=2.0, size=3).astype(f32)
    if np.allclose(pos, tgt):
        pos = pos + f32(1.0)
    w, h = int(rng.choice([17, 32, 40, 64])), int(rng.choice([9, 18, 23, 36]))
    ortho = rng.random() < 0.25
    cam = Camera.new(pos, tgt, [0.0, 1.0, 0.0], w, h, 0.01, 1000.0,
                     projection="Orthographic" if ortho else "Perspective",
                     fov=float(rng.uniform(20, 120)), size=float(rng.uniform(2, 20)))
    if rng.random() < 0.2:
        world = World("SolidColor", color=rng.uniform(0, 1, 3).astype(f32))
    else:
        world = World("SkyColor", rng.uniform(0, 1, 3).astype(f32), rng.uniform(0, 1, 3).astype(f32))
    spp, bounces = int(rng.integers(1, 4)), int(rng.choice([0, 1, 4, 12]))
    return Scene(cam, world, objs), spp, bounces


def _extreme_scene(seed):
    """Coordinates from 1e-4 to 1e7, object sizes from 1e-5 to 1e5 and cameras
    far from them: the fast paths' range guards and the IEEE fallbacks, and the
    LBVH's rounding-bound box growth, at their edges."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    scale = float(rng.choice([1e-4, 1e-2, 1.0, 1e3, 1e5, 1e7]))
    n = int(rng.choice([1, 5, 40, 200]))
    objs = []
    for i in range(n):
        c = (rng.normal(size=3) * scale).astype(f32)
        size = float(f32(scale * np.exp(rng.uniform(np.log(1e-5), np.log(1.0)))))
        m = Material(albedo=rng.uniform(0, 1, 3).astype(f32), roughness=float(f32(rng.uniform())),
                     metallic=float(f32(rng.choice([0.0, 1.0]))), transmission=float(f32(rng.choice([0.0, 1.0]))))
        objs.append(Object("Sphere" if rng.random() < 0.6 else "Cube", c, size, m))
    pos = (rng.normal(size=3) * scale * float(rng.choice([0.5, 3.0, 100.0]))).astype(f32)
    tgt = (rng.normal(size=3) * scale * 0.2).astype(f32)
    cam = Camera.new(pos, tgt, [0.0, 1.0, 0.0], 24, 16, 0.01, 1000.0, fov=float(rng.uniform(10, 100)))
    world = World("SkyColor", rng.uniform(0, 1, 3).astype(f32), rng.uniform(0, 1, 3).astype(f32))
    return Scene(cam, world, objs), int(rng.integers(1, 3)), int(rng.choice([1, 4, 12]))


def _gpu(scene, spp, bounces, seed, accel, wavefront=False):
    r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
    try:
        r._check(r.lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
        r.upload(scene)
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        if wavefront:
            r._check(r.lib.rdc_render_wavefront(r.ctx, 0, spp, bounces, seed), "rdc_render_wavefront")
        else:
            r.render_range(0, spp)
        return r.accumulator(scene), r.stats().segments
    finally:
        r.close()


@pytest.mark.parametrize("k", range(N_SCENES))
def test_random_scene_matches_the_oracle(k):
    scene, spp, bounces = _random_scene(1000 + k)
    seed = 77 + k
    ref, segs = oracle.render(scene.to_c(), 0, spp, bounces, seed, threads=8)
    forms = [(native.ACCEL_LBVH, False), (native.ACCEL_LBVH, True), (native.ACCEL_BRUTE_FORCE, False),
             (native.ACCEL_BRUTE_FORCE, True)]
    for accel, wf in forms:
        acc, s = _gpu(scene, spp, bounces, seed, accel, wf)
        assert s == segs, (accel, wf)
        assert bits_equal(acc, ref), (k, accel, wf, len(scene.objects))


@pytest.mark.parametrize("k", range(200))
def test_extreme_scale_scene_matches_the_oracle(k):
    scene, spp, bounces = _extreme_scene(7000 + k)
    seed = 11 + k
    ref, segs = oracle.render(scene.to_c(), 0, spp, bounces, seed, threads=8)
    for accel in (native.ACCEL_LBVH, native.ACCEL_BRUTE_FORCE):
        acc, s = _gpu(scene, spp, bounces, seed, accel)
        assert s == segs, (k, accel)
        assert bits_equal(acc, ref), (k, accel, len(scene.objects))


@pytest.mark.parametrize("k", range(100))
def test_random_scene_wavefront_in_several_waves_matches_the_oracle(k):
    """The wavefront form with 17-40 samples (waves of 16 and a remainder)
    from a first sample other than 0, through both accelerations."""
    scene, _, bounces = _random_scene(80000 + k)
    rng = np.random.default_rng(k)
    s0, spp = int(rng.integers(0, 5)), int(rng.integers(17, 41))
    seed = 500 + k
    ref, segs = oracle.render(scene.to_c(), s0, spp, bounces, seed, threads=8)
    for accel in (native.ACCEL_LBVH, native.ACCEL_BRUTE_FORCE):
        r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
        try:
            r._check(r.lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
            r.upload(scene)
            r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
            r._check(r.lib.rdc_render_wavefront(r.ctx, s0, spp, bounces, seed), "rdc_render_wavefront")
            acc, st = r.accumulator(scene), r.stats().segments
        finally:
            r.close()
        assert st == segs, (k, accel)
        assert bits_equal(acc, ref), (k, accel, len(scene.objects), spp)


@pytest.mark.parametrize("k", range(48))
def test_random_batch_matches_the_oracle(k):
    """A batch of 2-9 random scenes in one persistent launch: each equals the
    oracle's render with RNG stream = its batch index."""
    from raydar_gb300.batch import BatchRenderer
    rng = np.random.default_rng(5000 + k)
    items = []
    for j in range(int(rng.integers(2, 10))):
        scene, spp, bounces = _random_scene(20000 + 37 * k + j)
        items.append((scene, spp, bounces, 900 + 13 * k + j))
    br = BatchRenderer(items)
    try:
        br.render()
        total = br.stats().segments
        seg_sum = 0
        for i, (sc, spp, bounces, seed) in enumerate(items):
            ref, seg = oracle.render(sc.to_c(), 0, spp, bounces, seed, threads=8, stream=i)
            assert bits_equal(br.accumulator(i), ref), (k, i)
            seg_sum += seg
        assert total == seg_sum
    finally:
        br.close()


def _adjoint_case(k):
    scene, spp, _ = _random_scene(40000 + k)
    bounces = int(np.random.default_rng(k).choice([1, 3, 6, 16]))
    dl = np.random.default_rng(60 + k).uniform(-1, 1, (scene.height, scene.width, 3)).astype(np.float32)
    return scene, spp, bounces, 300 + k, dl


def _adjoint(scene, s0, spp, bounces, seed, dl, accel):
    r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
    try:
        r._check(r.lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
        r.forward(scene, spp, spp_begin=s0)
        return [np.asarray(g, np.float64) for g in r.backward(scene, dl)]
    finally:
        r.close()


@pytest.mark.parametrize("k", range(200))
def test_random_scene_adjoint_matches_the_oracle(k):
    """rdc_backward on random scenes (1-16 bounces, both accelerations)
    against the gradient oracle over the same paths, evaluated twice.  With
    each path's intermediates in float (the adjoint's precision) the
    relative L2 error must stay within 1e-4; in double, within the 1e-2 the
    gradients are specified with, on every scene whose two evaluations agree
    to 5e-3 and whose double replay kept every path.  The double evaluation
    departs from the float one where a path's derivative is ill-conditioned
    (hits a few ulp apart inside one object, where 1/t and grazing normals
    amplify rounding) or where replaying a float path in double loses a
    grazing hit (the oracle then drops that path): in 600 seeded scenes 13
    such, 10 with lost paths; the adjoint matched the float evaluation in all
    600 (worst 7e-6 relative, 2.6e-4 on a gradient of norm 5e-5).  (A float
    sum that cancels can also differ from double by ~1e-3: measured up to
    1.8e-3 on these scenes.)"""
    scene, spp, bounces, seed, dl = _adjoint_case(k)
    c = scene.to_c()
    o64 = oracle.gradient(c, 0, spp, bounces, seed, dl, threads=8)[:3]
    lost64 = oracle.gradient.lost_paths
    o32 = oracle.gradient(c, 0, spp, bounces, seed, dl, threads=8, fp32=True)[:3]
    assert oracle.gradient.lost_paths == 0  # the float replay is the float path itself
    for accel in (native.ACCEL_BRUTE_FORCE, native.ACCEL_LBVH):
        g = _adjoint(scene, 0, spp, bounces, seed, dl, accel)
        for name, gv, a, b in zip(("albedo", "roughness", "emission"), g, o64, o32):
            n32, e32 = float(np.linalg.norm(b)), float(np.linalg.norm(gv - b))
            assert e32 <= 1e-4 * n32 + 1e-6, (k, accel, name, "float", e32, n32)
            n64, e64 = float(np.linalg.norm(a)), float(np.linalg.norm(gv - a))
            if lost64 == 0 and float(np.linalg.norm(b - a)) <= 5e-3 * n64 + 1e-6:
                assert e64 <= 1e-2 * n64 + 1e-6, (k, accel, name, "double", e64, n64)


def test_an_ill_conditioned_path_follows_the_float_evaluation():
    """Random scene 89, sample 2 of pixel (18, 27): a path of 11 vertices,
    ten of them inside one partly metallic, partly transmissive object with
    hits 2e-5 to 1e-4 apart.  The roughness derivative of the object its
    first vertex hit is +1.66 in double and -0.88 in float; the adjoint
    gives the float value, through either acceleration."""
    scene, _, bounces, seed, dl = _adjoint_case(89)
    one = np.zeros_like(dl)
    one[27, 18] = dl[27, 18]
    c = scene.to_c()
    o64 = oracle.gradient(c, 2, 1, bounces, seed, one, threads=1)[1]
    o32 = oracle.gradient(c, 2, 1, bounces, seed, one, threads=1, fp32=True)[1]
    assert o64[43] > 1.0 and o32[43] < -0.5
    for accel in (native.ACCEL_BRUTE_FORCE, native.ACCEL_LBVH):
        gr = _adjoint(scene, 2, 1, bounces, seed, one, accel)[1]
        assert abs(gr[43] - o32[43]) <= 1e-5 * abs(o32[43]), (accel, gr[43], o32[43], o64[43])
        assert np.linalg.norm(gr - o32) <= 1e-4 * np.linalg.norm(o32)
