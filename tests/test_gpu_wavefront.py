"""Wavefront render (rdc_render_wavefront) against the megakernel (rdc_render):
the same accumulator bit for bit and the same segment count, for the config
scenes, a progressive split, the no-bounce case and waves of several
samples (full waves, a remainder, a first sample other than 0, an image
whose wave holds fewer than 16 samples)."""
import numpy as np
import pytest

from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _both(scene, s0, n, bounces, seed, accel=None):
    out = []
    for fn in ("rdc_render", "rdc_render_wavefront"):
        r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
        r._check(r.lib.rdc_set_render_form(r.ctx, native.FORM_MEGAKERNEL), "rdc_set_render_form")
        if accel is not None:
            r._check(r.lib.rdc_set_accel(r.ctx, accel), "set_accel")
        r.upload(scene)
        r._check(r.lib.rdc_reset(r.ctx), "reset")
        r._check(getattr(r.lib, fn)(r.ctx, s0, n, bounces, seed), fn)
        out.append((r.accumulator(scene), r.stats().segments))
        r.close()
    return out


@pytest.mark.parametrize("name,make", [
    ("c1", lambda: shrink(scenegen.c1_plain().scene, 64, 36)),
    ("c2", lambda: shrink(scenegen.c2_default().scene, 96, 54)),
    ("c4", lambda: shrink(scenegen.c4_diff().scene, 48, 48)),
])
def test_wavefront_equals_megakernel(name, make):
    (a, sa), (b, sb) = _both(make(), 0, 6, 12, 99)
    assert sa == sb
    assert bits_equal(a, b)


def test_wavefront_progressive_and_zero_bounces():
    scene = shrink(scenegen.c2_default().scene, 40, 24)
    (a, _), (b, _) = _both(scene, 3, 4, 8, 5)
    assert bits_equal(a, b)
    (a, sa), (b, sb) = _both(scene, 0, 2, 0, 5)
    assert sa == sb == 0 and bits_equal(a, b) and np.all(b[..., 3] == 2)


def test_wavefront_lbvh_equals_megakernel_lbvh_and_the_oracle():
    """LBVH scenes take the persistent LBVH intersect kernel: the same
    accumulator as the LBVH megakernel and the oracle's brute force."""
    import oracle
    scene = scenegen.c5_large(seed=4, width=40, height=24, n_spheres=3000, n_cubes=300).scene
    (a, sa), (b, sb) = _both(scene, 0, 3, 12, 21, accel=native.ACCEL_LBVH)
    assert sa == sb
    assert bits_equal(a, b)
    ref, segs = oracle.render(scene.to_c(), 0, 3, 12, 21, threads=8)
    assert segs == sb and bits_equal(b, ref)


def test_wavefront_lbvh_on_small_scenes_and_refill_thresholds():
    """One object (no tree nodes), a forced LBVH on a config scene, and
    refill thresholds from 1 to 32: all bit-identical to the megakernel."""
    one = shrink(scenegen.c1_plain().scene, 24, 16)
    one.objects = one.objects[:1]
    (a, sa), (b, sb) = _both(one, 0, 2, 6, 3, accel=native.ACCEL_LBVH)
    assert sa == sb and bits_equal(a, b)
    scene = shrink(scenegen.c2_default().scene, 48, 27)
    ref = None
    for mi in (1, 8, 16, 32):
        r = CudaRenderer(RendererConfig(max_bounces=12), seed=8)
        r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_LBVH), "set_accel")
        cfg = native.RdcLaunchConfig(256, 0, mi)
        r._check(r.lib.rdc_set_render_config(r.ctx, native.C.byref(cfg)), "cfg")
        r.upload(scene)
        r._check(r.lib.rdc_reset(r.ctx), "reset")
        r._check(r.lib.rdc_render_wavefront(r.ctx, 0, 2, 12, 8), "wavefront")
        acc = r.accumulator(scene)
        r.close()
        if ref is None:
            (ref, _), _ = _both(scene, 0, 2, 12, 8, accel=native.ACCEL_LBVH)
        assert bits_equal(acc, ref), mi


@pytest.mark.parametrize("w,h,s0,n,accel", [
    (40, 24, 0, 37, native.ACCEL_BRUTE_FORCE),   # waves of 16, 16, 5
    (40, 24, 5, 16, native.ACCEL_BRUTE_FORCE),   # one full wave from sample 5
    (40, 24, 3, 17, native.ACCEL_LBVH),          # 16 + 1
    (4096, 2048, 2, 11, native.ACCEL_BRUTE_FORCE),  # 2^23 pixels: waves of 4, 4, 3
    (4096, 4096, 0, 3, native.ACCEL_LBVH),       # 2^24 pixels: waves of 2, 1 through the LBVH
])
def test_wavefront_waves_of_several_samples(w, h, s0, n, accel):
    """A wave holds up to 16 consecutive samples of every pixel (at most 2^25
    paths) and adds each pixel's radiances in sample order."""
    scene = shrink(scenegen.c2_default().scene, w, h)
    (a, sa), (b, sb) = _both(scene, s0, n, 6, 17, accel=accel)
    assert sa == sb
    assert bits_equal(a, b)


def _render_form(scene, s0, n, bounces, seed, accel, form):
    r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
    try:
        r._check(r.lib.rdc_set_render_form(r.ctx, form), "rdc_set_render_form")
        r._check(r.lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
        r.upload(scene)
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r._check(r.lib.rdc_render(r.ctx, s0, n, bounces, seed), "rdc_render")
        st = r.stats()
        return r.accumulator(scene), st.segments, st.kernel_launches
    finally:
        r.close()


@pytest.mark.parametrize("accel,w,h,spp,expect", [
    (native.ACCEL_LBVH, 48, 27, 6, "wavefront"),          # a wave holds 6 samples: the wavefront
    (native.ACCEL_LBVH, 48, 27, 3, "megakernel"),         # 3 samples per wave: the megakernel
    (native.ACCEL_BRUTE_FORCE, 48, 27, 6, "wavefront"),   # a small image: the wavefront
    (native.ACCEL_BRUTE_FORCE, 48, 27, 3, "megakernel"),
    (native.ACCEL_BRUTE_FORCE, 640, 360, 4, "megakernel"),  # 230k pixels, above 1.5 per resident lane
    (native.ACCEL_LBVH, 640, 360, 4, "wavefront"),
])
def test_rdc_render_chooses_its_form_and_every_form_agrees(accel, w, h, spp, expect):
    """rdc_render in RDC_FORM_AUTO runs a scene as wavefront once a wave holds
    4 or more samples of every pixel and the scene uses the LBVH or the image
    has at most 1.5 pixels per resident megakernel lane, and as megakernel
    otherwise; the forced forms give the same accumulator."""
    scene = shrink(scenegen.c2_default().scene, w, h)
    auto, s_auto, l_auto = _render_form(scene, 1, spp, 8, 19, accel, native.FORM_AUTO)
    assert (l_auto > 1) == (expect == "wavefront"), l_auto
    for form in (native.FORM_MEGAKERNEL, native.FORM_WAVEFRONT):
        acc, segs, launches = _render_form(scene, 1, spp, 8, 19, accel, form)
        assert (launches == 1) == (form == native.FORM_MEGAKERNEL)
        assert segs == s_auto and bits_equal(acc, auto), form


def test_rdc_set_render_form_rejects_an_unknown_form():
    r = CudaRenderer(RendererConfig(), seed=0)
    try:
        assert r.lib.rdc_set_render_form(r.ctx, 3) == 1  # RDC_ERR_INVALID_ARGUMENT
        assert r.lib.rdc_set_render_form(None, native.FORM_AUTO) == 1
    finally:
        r.close()
