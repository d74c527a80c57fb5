"""Edge cases of the differentiation and material-update entry points:
rdc_update_materials equals a fresh upload (brute force and LBVH, no
rebuild), the adjoint on an LBVH scene matches the FP64 oracle, a SolidColor
world has no roughness gradient, and the bounce limit is enforced."""
import numpy as np
import pytest

import oracle
from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from raydar_gb300.scene import World, material_records
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _render(scene, spp, bounces, seed, materials=None, accel=native.ACCEL_AUTO):
    r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
    r._check(r.lib.rdc_set_accel(r.ctx, accel), "set_accel")
    r.upload(scene)
    if materials is not None:
        r.update_materials(materials)
    r._check(r.lib.rdc_reset(r.ctx), "reset")
    r.render_range(0, spp)
    acc = r.accumulator(scene)
    st = r.stats()
    r.close()
    return acc, st


@pytest.mark.parametrize("large", [False, True])
def test_update_materials_equals_a_fresh_upload(large):
    if large:
        scene = scenegen.c5_large(seed=4, width=32, height=18, n_spheres=1500, n_cubes=150).scene
    else:
        scene = shrink(scenegen.c2_default().scene, 48, 27)
    mats = material_records(scene)
    rng = np.random.default_rng(1)
    new = mats.copy()
    new["albedo"] = rng.uniform(0, 1, new["albedo"].shape).astype(np.float32)
    new["roughness"] = rng.uniform(0, 1, len(new)).astype(np.float32)
    a, sa = _render(scene, 2, 8, 3, materials=new)
    # the same materials uploaded with the geometry
    if large:
        fresh = scenegen.c5_large(seed=4, width=32, height=18, n_spheres=1500, n_cubes=150).scene
        for f in ("albedo", "roughness"):
            fresh.packed[f] = new[f]
    else:
        fresh = shrink(scenegen.c2_default().scene, 48, 27)
        for o, m in zip(fresh.objects, new):
            o.material.albedo = np.asarray(m["albedo"], np.float32).copy()
            o.material.roughness = float(m["roughness"])
    b, sb = _render(fresh, 2, 8, 3)
    assert sa.accel == sb.accel == (native.ACCEL_LBVH if large else native.ACCEL_BRUTE_FORCE)
    assert bits_equal(a, b) and sa.segments == sb.segments


def test_adjoint_on_an_lbvh_scene_matches_the_fp64_oracle():
    scene = scenegen.c5_large(seed=6, width=24, height=16, n_spheres=800, n_cubes=80).scene
    r = CudaRenderer(RendererConfig(max_bounces=6), seed=13)
    r.forward(scene, 4)
    assert r.stats().accel == native.ACCEL_LBVH
    dl = np.random.default_rng(2).uniform(-1, 1, (16, 24, 3)).astype(np.float32)
    ga, gr, ge = r.backward(scene, dl)
    r.close()
    oa, orr, oe, _ = oracle.gradient(scene.to_c(), 0, 4, 6, 13, dl, threads=16)
    for g, o in ((ga, oa), (gr, orr), (ge, oe)):
        if np.linalg.norm(o) > 0:
            assert np.linalg.norm(g - o) / np.linalg.norm(o) < 1e-2


def test_solid_color_world_has_only_the_lobe_choice_roughness_gradient():
    """Under a SolidColor world no direction changes a path's radiance, so the
    pathwise part of the roughness gradient is zero; what remains is the
    lobe-choice part (which lobe a coin picks changes what the path hits
    next), and the kernel's must equal the FP64 oracle's."""
    scene = shrink(scenegen.c4_diff().scene, 24, 24)
    scene.world = World("SolidColor", color=np.array([0.6, 0.7, 0.8], np.float32))
    r = CudaRenderer(RendererConfig(max_bounces=6), seed=2)
    r.forward(scene, 4)
    dl = np.ones((24, 24, 3), np.float32)
    ga, gr, ge = r.backward(scene, dl)
    r.close()
    assert np.abs(ga).sum() > 0 and np.abs(ge).sum() > 0
    oa, orr, oe, _, path = oracle.gradient(scene.to_c(), 0, 4, 6, 2, dl, threads=8, pathwise=True)
    assert np.all(path == 0.0) and np.abs(orr).sum() > 0
    assert np.linalg.norm(ga - oa) / np.linalg.norm(oa) < 1e-4
    assert np.linalg.norm(gr - orr) / np.linalg.norm(orr) < 1e-3


def test_adjoint_bounce_limit_and_material_count_are_checked():
    scene = shrink(scenegen.c4_diff().scene, 8, 8)
    r = CudaRenderer(RendererConfig(max_bounces=17), seed=1)
    r.upload(scene)
    img = np.zeros((8, 8, 3), np.float32)
    assert r.lib.rdc_forward(r.ctx, 0, 1, 17, 1, native.fptr(img)) == 3  # RDC_ERR_LIMIT
    mats = material_records(scene)
    with pytest.raises(native.RdcError):
        r.update_materials(mats[:-1])
    r.close()
