"""The kernels' IEEE fallback, through the C ABI, against the oracle.

The guarded fast path (exact reciprocal division, the pass-1 filters) runs only
where every operand is inside its range; a scene with a sphere centre beyond
2^50, or a ray with a direction component of 0 or below 2^-40 or an origin
beyond 2^50, takes the reference's own arithmetic everywhere (IEEE division,
the exact discriminant in pass 1).  Renders and ray batches on such inputs must
still match the oracle bit for bit (src/renderer/cpu.rs:34-98 with rounding
exactly as the reference's)."""
import copy

import numpy as np
import pytest

import oracle
from raydar_gb300 import native, scenegen
from raydar_gb300.scene import Material, Object
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu

F = np.float32


def _with_far_sphere(scene):
    """The same scene plus one sphere beyond the fast path's 2^50 guard (never visible)."""
    s = copy.deepcopy(scene)
    s.objects.append(Object("Sphere", np.array([2.0 ** 51, 0.0, 0.0], F), 1.0,
                            Material(albedo=np.array([0.5, 0.5, 0.5], F), roughness=1.0)))
    return s


def test_render_of_a_scene_outside_the_guards_matches_oracle(renderer):
    scene = _with_far_sphere(shrink(scenegen.c2_default().scene, 96, 54))
    renderer.seed = 321
    renderer.config.max_bounces = 8
    renderer.upload(scene)
    renderer._check(renderer.lib.rdc_reset(renderer.ctx), "reset")
    renderer.render_range(0, 3)
    acc = renderer.accumulator(scene)
    seg = renderer.stats().segments
    ref, ref_seg = oracle.render(scene.to_c(), 0, 3, 8, 321, threads=8)
    assert seg == ref_seg
    assert bits_equal(acc, ref)


def _odd_rays(scene, n, rng):
    """Rays the fast path does not take: direction components exactly 0,
    below 2^-40, or large; origins beyond 2^50; mixed with ordinary ones."""
    o = rng.uniform(-12.0, 12.0, (n, 3)).astype(F)
    o[:, 1] = rng.uniform(0.05, 6.0, n)
    d = rng.normal(size=(n, 3)).astype(F)
    k = n // 6
    rows = np.arange(k)
    d[rows, rng.integers(0, 3, k)] = 0.0                      # one component 0: parallel to a slab pair
    d[k:2 * k, 0] = 0.0
    d[k:2 * k, 2] = 0.0                                       # straight down / up
    d[2 * k + rows, rng.integers(0, 3, k)] = F(1e-13)         # one component below 2^-40
    d[3 * k:4 * k] *= F(40.0)                                 # |d| components above 16
    o[4 * k:5 * k, 0] = F(2.0 ** 51)                          # origin beyond 2^50
    d[4 * k:5 * k, 0] = -1.0
    return np.ascontiguousarray(o), np.ascontiguousarray(d)


@pytest.mark.parametrize("far", [False, True])
def test_ray_batch_off_the_fast_path_matches_oracle(renderer, far):
    scene = shrink(scenegen.c2_default().scene, 96, 54)
    if far:
        scene = _with_far_sphere(scene)
    renderer.upload(scene)
    n = 1 << 15
    o, d = _odd_rays(scene, n, np.random.default_rng(17 + far))
    t = np.zeros(n, F)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), F)
    fr = np.zeros(n, np.uint8)
    assert renderer.lib.rdc_intersect_rays(renderer.ctx, native.fptr(o), native.fptr(d), n, native.fptr(t),
                                           native.iptr(idx), native.fptr(nrm), native.u8ptr(fr)) == 0
    rt, ridx, rn, rf = oracle.intersect(scene.to_c(), o, d)
    assert (ridx >= 0).mean() > 0.15
    assert np.array_equal(idx, ridx)
    assert not np.isnan(rn).any()  # every ray has a direction: no NaN to compare
    assert bits_equal(t, rt) and bits_equal(nrm, rn) and np.array_equal(fr, rf)
