"""Wavefront render (rdc_render_wavefront) against the megakernel (rdc_render):
the same accumulator bit for bit and the same segment count, for the config
scenes, a progressive split and the no-bounce case."""
import numpy as np
import pytest

from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _both(scene, s0, n, bounces, seed):
    out = []
    for fn in ("rdc_render", "rdc_render_wavefront"):
        r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
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


def test_wavefront_refuses_lbvh_scenes():
    scene = shrink(scenegen.c2_default().scene, 32, 18)
    r = CudaRenderer(RendererConfig(), seed=1)
    r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_LBVH), "set_accel")
    r.upload(scene)
    assert r.lib.rdc_render_wavefront(r.ctx, 0, 1, 4, 1) == 2  # RDC_ERR_UNSUPPORTED
    r.close()
