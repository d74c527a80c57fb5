"""Contexts give back what they take: device memory after many create /
use / destroy cycles -- brute-force and LBVH uploads, renders, the wavefront
form, the adjoint buffers, the stage checks and batches -- equals the memory
before them (driver-wide free memory, read with cudaMemGetInfo through torch),
and a context keeps rendering the oracle's image after each kind of use."""
import numpy as np
import pytest

import oracle
from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen
from raydar_gb300.batch import BatchRenderer
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu


def _cycle(scenes):
    big, small = scenes
    r = CudaRenderer(RendererConfig(max_bounces=6), seed=5)
    try:
        r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_LBVH), "rdc_set_accel")
        r.upload(big)
        r.render_range(0, 1)
        r._check(r.lib.rdc_render_wavefront(r.ctx, 0, 1, 6, 5), "rdc_render_wavefront")
        r.forward(big, 1)
        r.backward(big, np.ones((big.height, big.width, 3), np.float32))
        r._check(r.lib.rdc_set_accel(r.ctx, native.ACCEL_BRUTE_FORCE), "rdc_set_accel")
        r.upload(small)
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r.render_range(0, 2)
        acc = r.accumulator(small)
    finally:
        r.close()
    br = BatchRenderer([(small, 1, 4, 1), (shrink(small, 24, 16), 2, 3, 2)])  # batches are brute force
    try:
        br.render()
        br.stats()
    finally:
        br.close()
    return acc


def test_contexts_return_their_device_memory():
    torch = pytest.importorskip("torch")
    big = scenegen.c5_large(seed=6, width=48, height=27, n_spheres=20000, n_cubes=2000).scene
    small = shrink(scenegen.c2_default().scene, 40, 24)
    ref, _ = oracle.render(small.to_c(), 0, 2, 6, 5, threads=8)
    acc = _cycle((big, small))  # first use: module load, kernels resident
    assert bits_equal(acc, ref)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(12):
        acc = _cycle((big, small))
        assert bits_equal(acc, ref)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    # a cycle allocates tens of MB (LBVH nodes and scratch, wavefront state, adjoint buffers, batch):
    # twelve of them leaking would show; allow the driver's own few MB of slack
    assert abs(free0 - free1) <= 8 << 20, (free0, free1)
