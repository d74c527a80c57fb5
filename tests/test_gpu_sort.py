"""The device radix sort and prefix sum of the LBVH build, through their
self-test entry points, against numpy's stable sort and cumulative sum.

A wrong sort would still give a correct hierarchy (the refit computes true
boxes) but a slower one, so the render parity tests cannot catch it; these
compare the sorted order itself, including the order of equal keys, which
the Karras construction's position tie-break relies on."""
import ctypes as C

import numpy as np
import pytest

from raydar_gb300 import CudaRenderer, RendererConfig

pytestmark = pytest.mark.gpu

U32P = C.POINTER(C.c_uint32)


def _p(a):
    return a.ctypes.data_as(U32P)


@pytest.fixture(scope="module")
def r():
    rr = CudaRenderer(RendererConfig(), device=0)
    yield rr
    rr.close()


@pytest.mark.parametrize("n,bits,distinct", [(1, 30, 1), (2, 30, 2), (2047, 30, 50), (2048, 30, 2048),
                                             (2049, 30, 300), (100_000, 30, 1 << 30), (110_000, 30, 5000),
                                             (1 << 20, 32, 1 << 31), (300_001, 10, 1024), (70_000, 7, 100)])
def test_radix_sort_is_numpy_stable_sort(r, n, bits, distinct):
    rng = np.random.default_rng(n + bits)
    keys = (rng.integers(0, distinct, n, dtype=np.uint64) % (1 << bits)).astype(np.uint32)
    if distinct >= (1 << 30):  # spread over the whole key range
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32) ^ np.uint32(0x9E3779B9)
    ko = np.empty_like(keys)
    vo = np.empty_like(vals)
    st = r.lib.rdc_selftest_radix_sort(r.ctx, _p(keys), _p(vals), n, bits, _p(ko), _p(vo))
    assert st == 0, r.lib.rdc_last_error(r.ctx)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ko, keys[order])
    assert np.array_equal(vo, vals[order])


def test_radix_sort_of_morton_codes_of_the_large_scene(r):
    """The LBVH's own input: 30-bit Morton codes of 110k object centres
    (many shared cells)."""
    from raydar_gb300 import scenegen
    w = scenegen.c5_large(width=32, height=18)
    c = w.scene.packed["center"].astype(np.float32)
    lo, hi = c.min(0), c.max(0)
    q = np.clip(((c - lo) / (hi - lo).max() * 1024.0), 0, 1023).astype(np.uint32)

    def spread(v):
        v = (v | (v << 16)) & 0x030000FF
        v = (v | (v << 8)) & 0x0300F00F
        v = (v | (v << 4)) & 0x030C30C3
        return (v | (v << 2)) & 0x09249249

    keys = ((spread(q[:, 0]) << 2) | (spread(q[:, 1]) << 1) | spread(q[:, 2])).astype(np.uint32)
    vals = np.arange(len(keys), dtype=np.uint32)
    ko, vo = np.empty_like(keys), np.empty_like(vals)
    assert r.lib.rdc_selftest_radix_sort(r.ctx, _p(keys), _p(vals), len(keys), 30, _p(ko), _p(vo)) == 0
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ko, keys[order]) and np.array_equal(vo, vals[order])


@pytest.mark.parametrize("n", [1, 5, 4095, 4096, 4097, 100_000, (1 << 20) + 3, 1 << 24])
def test_exclusive_scan_is_numpy_cumsum(r, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32) if n < 1000 else \
        rng.integers(0, 9, n, dtype=np.uint64).astype(np.uint32)
    out = np.empty_like(x)
    assert r.lib.rdc_selftest_exclusive_scan(r.ctx, _p(x), n, _p(out)) == 0, r.lib.rdc_last_error(r.ctx)
    ref = np.concatenate([[0], np.cumsum(x.astype(np.uint64))[:-1]]) % (1 << 32)
    assert np.array_equal(out, ref.astype(np.uint32))


def test_self_tests_reject_bad_arguments(r):
    k = np.zeros(4, np.uint32)
    assert r.lib.rdc_selftest_radix_sort(r.ctx, _p(k), _p(k), 4, 0, _p(k), _p(k)) != 0
    assert r.lib.rdc_selftest_radix_sort(r.ctx, _p(k), _p(k), 4, 33, _p(k), _p(k)) != 0
    assert r.lib.rdc_selftest_radix_sort(r.ctx, None, None, 4, 30, None, None) != 0
    assert r.lib.rdc_selftest_exclusive_scan(r.ctx, None, 4, None) != 0
    assert r.lib.rdc_selftest_radix_sort(r.ctx, _p(k), _p(k), 0, 30, _p(k), _p(k)) == 0
