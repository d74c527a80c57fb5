"""Batched persistent launch vs the oracle: every scene of a batch (uneven
resolution, spp, bounces and object count) must equal the oracle's render of
that scene with RNG stream = its batch index, bit for bit, under any launch
shape."""
import numpy as np
import pytest

import oracle
from raydar_gb300 import scenegen
from raydar_gb300.batch import BatchRenderer
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _items():
    ws = scenegen.c3_batch(seed=11, count=6)
    items = []
    for k, w in enumerate(ws):
        sc = shrink(w.scene, 24 + 8 * k, 16 + 4 * k)
        items.append((sc, 2 + (k % 3), 2 + 2 * (k % 4), 1000 + k))
    items.append((shrink(scenegen.c1_plain().scene, 17, 9), 3, 0, 77))   # zero bounces
    items.append((shrink(scenegen.c1_plain().scene, 5, 3), 0, 8, 78))    # zero samples
    return items


def test_batch_matches_oracle_per_scene():
    items = _items()
    br = BatchRenderer(items)
    br.render()
    total = br.stats().segments
    seg_sum = 0
    for i, (sc, spp, bounces, seed) in enumerate(items):
        ref, seg = oracle.render(sc.to_c(), 0, spp, bounces, seed, threads=8, stream=i)
        assert bits_equal(br.accumulator(i), ref), f"scene {i}"
        seg_sum += seg
    assert total == seg_sum
    br.close()


def test_batch_is_independent_of_launch_shape_and_replays():
    items = _items()[:4]
    br = BatchRenderer(items)
    br.render()
    first = [br.accumulator(i) for i in range(len(items))]
    for cfg in [(128, 1, 1), (256, 0, 16), (64, 2, 32)]:
        br.set_config(*cfg)
        br.render()
        for i in range(len(items)):
            assert bits_equal(br.accumulator(i), first[i]), (cfg, i)
    res = br.autotune()
    assert res["block_size"] in (128, 256) and res["ms"] > 0
    br.render()
    for i in range(len(items)):
        assert bits_equal(br.accumulator(i), first[i])
    br.close()


def test_config3_batch_at_full_resolution_matches_the_oracle():
    """The 64 seeded scenes of the batched workload (width 128..1024, 16:9 or
    1:1, 4..12 bounces, 4..200 spheres + 0..20 cubes) at their full
    resolution and bounce limit, with every scene's spp divided by 128 (at
    least 1) so the oracle finishes in seconds, under the launch shape the
    autotuner picks: each accumulator equals the oracle's render of that scene
    (RNG stream = its batch index) bit for bit, and the segment counts add up."""
    ws = scenegen.c3_batch()
    items = [(w.scene, max(1, w.spp // 128), w.max_bounces, 3000 + i) for i, w in enumerate(ws)]
    br = BatchRenderer(items)
    tune = br.autotune()
    br.render()
    total = br.stats().segments
    seg_sum = 0
    for i, (sc, spp, bounces, seed) in enumerate(items):
        ref, seg = oracle.render(sc.to_c(), 0, spp, bounces, seed, threads=16, stream=i)
        assert bits_equal(br.accumulator(i), ref), f"scene {i} ({sc.width}x{sc.height}, {spp} spp)"
        seg_sum += seg
    assert total == seg_sum
    assert tune["block_size"] in (64, 128, 256)
    br.close()
