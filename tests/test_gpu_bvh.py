"""Device-built LBVH vs brute force and vs the oracle.

The LBVH must give exactly the brute-force closest hit (t, normal and object
index byte for byte, lowest index on ties): checked on a 1M-ray sample of the
100k-sphere / 10k-cube scene of config 5, and through whole renders compared
with the oracle and with the brute-force kernel."""
import copy

import numpy as np
import pytest

import oracle
from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from raydar_gb300.scene import Camera, Material, Object, Scene, World
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _intersect(r, o, d):
    n = len(o)
    t = np.zeros(n, np.float32)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), np.float32)
    fr = np.zeros(n, np.uint8)
    st = r.lib.rdc_intersect_rays(r.ctx, native.fptr(o), native.fptr(d), n, native.fptr(t), native.iptr(idx),
                                  native.fptr(nrm), native.u8ptr(fr))
    assert st == 0, r.lib.rdc_last_error(r.ctx)
    return t, idx, nrm, fr


def _ray_sample(scene, packed, n, rng):
    """Camera rays, rays from inside the volume, and rays leaving sphere surfaces."""
    k = n // 3
    cam = scene.camera
    o1 = np.tile(cam.position.astype(np.float32), (k, 1))
    tgt = np.stack([rng.uniform(-20, 20, k), rng.uniform(0, 10, k), rng.uniform(-20, 20, k)], 1)
    d1 = (tgt - o1).astype(np.float32)
    o2 = np.stack([rng.uniform(-22, 22, k), rng.uniform(-1, 11, k), rng.uniform(-22, 22, k)], 1).astype(np.float32)
    d2 = rng.normal(size=(k, 3)).astype(np.float32)
    sph = np.where(packed["geometry"] == 0)[0]
    pick = rng.choice(sph, n - 2 * k)
    nrm = rng.normal(size=(len(pick), 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    o3 = (packed["center"][pick] + nrm * (packed["radius"][pick, None] + 1e-4)).astype(np.float32)
    d3 = (nrm + rng.normal(size=nrm.shape)).astype(np.float32)
    o = np.ascontiguousarray(np.concatenate([o1, o2, o3]), np.float32)
    d = np.ascontiguousarray(np.concatenate([d1, d2, d3]), np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    return o, np.ascontiguousarray(d, np.float32)


def test_lbvh_equals_brute_force_on_1m_rays():
    w = scenegen.c5_large()
    r = CudaRenderer(RendererConfig(), seed=0)
    r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_LBVH), "set_accel")
    r.upload(w.scene)
    st = r.stats()
    assert st.accel == native.ACCEL_LBVH and 0 < st.bvh_depth <= 64
    o, d = _ray_sample(w.scene, w.scene.packed, 1 << 20, np.random.default_rng(7))
    tb, ib, nb, fb = _intersect(r, o, d)
    r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_BRUTE_FORCE), "set_accel")
    tf, i_f, nf, ff = _intersect(r, o, d)
    r.close()
    assert (i_f >= 0).mean() > 0.3
    bad = np.where(ib != i_f)[0]
    assert len(bad) == 0, f"{len(bad)} index mismatches, e.g. {bad[:5].tolist()}"
    assert bits_equal(tb, tf) and bits_equal(nb, nf) and np.array_equal(fb, ff)


def _mid_scene(n_spheres=2500, n_cubes=300, w=48, h=27):
    big = scenegen.c5_large(seed=9, width=w, height=h, n_spheres=n_spheres, n_cubes=n_cubes)
    return big.scene


def test_lbvh_render_matches_oracle():
    scene = _mid_scene()
    r = CudaRenderer(RendererConfig(max_bounces=8), seed=21)
    r.upload(scene)  # AUTO: above 512 objects -> LBVH
    r._check(r.lib.rdc_reset(r.ctx), "reset")
    r.render_range(0, 2)
    acc = r.accumulator(scene)
    st = r.stats()
    r.close()
    assert st.accel == native.ACCEL_LBVH and st.node_visits > 0 and st.prim_tests > 0
    ref, seg = oracle.render(scene.to_c(), 0, 2, 8, 21, threads=16)
    assert st.segments == seg
    assert bits_equal(acc, ref)


def test_lbvh_and_brute_force_renders_are_identical():
    scene = shrink(scenegen.c2_default().scene, 96, 54)
    out = {}
    for mode in (native.ACCEL_BRUTE_FORCE, native.ACCEL_LBVH):
        r = CudaRenderer(RendererConfig(max_bounces=12), seed=5)
        r._check(r.lib.rdc_set_accel(r.ctx, mode), "set_accel")
        r.upload(scene)
        r._check(r.lib.rdc_reset(r.ctx), "reset")
        r.render_range(0, 3)
        out[mode] = (r.accumulator(scene), r.stats())
        r.close()
    a, sa = out[native.ACCEL_BRUTE_FORCE]
    b, sb = out[native.ACCEL_LBVH]
    assert sa.accel == native.ACCEL_BRUTE_FORCE and sb.accel == native.ACCEL_LBVH
    assert bits_equal(a, b) and sa.segments == sb.segments


def test_lbvh_ties_pick_the_lowest_index():
    """600 identical spheres (one Morton code, every t equal) plus a cube: the
    reference's first-minimum rule must survive the tree order."""
    cam = Camera.new([0, 1, -6], [0, 1, 0], [0, 1, 0], 8, 8, 0.01, 1000.0, fov=30.0)
    objs = [Object("Cube", np.array([0, -5, 0], np.float32), 10.0, Material())]
    objs += [Object("Sphere", np.array([0, 1, 0], np.float32), 1.0, Material()) for _ in range(600)]
    scene = Scene(cam, World(), objs)
    r = CudaRenderer(RendererConfig(max_bounces=3), seed=1)
    r.upload(scene)
    rng = np.random.default_rng(3)
    o = np.tile(np.array([0, 1, -6], np.float32), (4096, 1))
    d = np.ascontiguousarray(np.array([0, 0, 1], np.float32) + rng.normal(scale=0.2, size=(4096, 3)), np.float32)
    t, idx, nrm, fr = _intersect(r, o, d)
    rt, ridx, rn, rf = oracle.intersect(scene.to_c(), o, d)
    assert r.stats().accel == native.ACCEL_LBVH
    assert set(np.unique(ridx[ridx >= 0]).tolist()) <= {0, 1}
    assert np.array_equal(idx, ridx) and bits_equal(t, rt) and bits_equal(nrm, rn)
    r._check(r.lib.rdc_reset(r.ctx), "reset")
    r.render_range(0, 2)
    ref, _ = oracle.render(scene.to_c(), 0, 2, 3, 1)
    assert bits_equal(r.accumulator(scene), ref)
    r.close()
