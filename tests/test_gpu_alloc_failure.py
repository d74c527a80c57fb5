"""Out-of-memory handling, by host-side fault injection (no GPU fault).

With RDC_FAIL_ALLOC_AFTER=n in the environment, rdc_create lets the next n
device allocations of the library succeed and fails every later one with
cudaErrorMemoryAllocation, without calling cudaMalloc.  Walking n from 0 up
drives the failure through every allocating call in turn (context creation,
scene upload, the 8-bit read-back, the LBVH build, the adjoint's buffers, the
stage-check buffer, a batch upload).  Each call must return RDC_OK,
RDC_ERR_OUT_OF_MEMORY (with a message) or RDC_ERR_NO_SCENE (a render after a
failed upload), never anything else; a failed upload must leave no scene
behind (a later render is refused, not launched on freed buffers); and the
context must end with nothing faulted on the device.  Without the variable
the same sequence renders exactly what the oracle renders."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from raydar_gb300 import native, scenegen
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu

OK, NO_SCENE, OOM = native.RDC_OK, 4, 6
W, H, SPP, BOUNCES, SEED = 16, 9, 2, 6, 9


def _sequence(lib, sc, sc2):
    """Run the API sequence; returns [(call, status)] and the first render's accumulator."""
    out = []
    ctx = C.c_void_p()
    st = lib.rdc_create(C.byref(ctx), 0)
    out.append(("create", st))
    if st != OK:
        assert st == OOM and b"cudaMalloc" in lib.rdc_last_error(None)
        return out, None
    acc = np.zeros((H, W, 4), np.float32)
    try:
        def call(name, st):
            out.append((name, st))
            if st == OOM:
                assert len(lib.rdc_last_error(ctx)) > 0
            return st

        call("upload", lib.rdc_scene_upload(ctx, sc.ref()))
        call("reset", lib.rdc_reset(ctx))
        if call("render", lib.rdc_render(ctx, 0, SPP, BOUNCES, SEED)) == OK:
            call("read_accum", lib.rdc_read_accum(ctx, native.fptr(acc), acc.size))
        img8 = np.zeros((H, W, 4), np.uint8)
        call("read_rgba8", lib.rdc_read_rgba8(ctx, SPP, native.u8ptr(img8), img8.size))
        call("set_accel_lbvh", lib.rdc_set_accel(ctx, native.ACCEL_LBVH))
        call("render_lbvh", lib.rdc_render(ctx, 0, 1, BOUNCES, SEED))
        image = np.zeros((H, W, 3), np.float32)
        call("forward", lib.rdc_forward(ctx, 0, SPP, BOUNCES, SEED, native.fptr(image)))
        dl = np.ones((H, W, 3), np.float32)
        ga = np.zeros((sc.desc.object_count, 3), np.float32)
        gr = np.zeros(sc.desc.object_count, np.float32)
        ge = np.zeros((sc.desc.object_count, 3), np.float32)
        call("backward", lib.rdc_backward(ctx, native.fptr(dl), native.fptr(ga), native.fptr(gr), native.fptr(ge)))
        o = np.tile(np.array([[0.0, 1.5, -6.0]], np.float32), (8, 1))
        d = np.tile(np.array([[0.0, -0.2, 1.0]], np.float32), (8, 1))
        t, idx, nrm, fr = (np.zeros(8, np.float32), np.zeros(8, np.int32), np.zeros((8, 3), np.float32),
                           np.zeros(8, np.uint8))
        call("intersect", lib.rdc_intersect_rays(ctx, native.fptr(o), native.fptr(d), 8, native.fptr(t),
                                                 native.iptr(idx), native.fptr(nrm), native.u8ptr(fr)))
        items = (native.RdcBatchItem * 2)()
        for k, s in enumerate((sc, sc2)):
            items[k].scene = C.pointer(s.desc)
            items[k].spp, items[k].max_bounces, items[k].seed = 1, 4, 5 + k
        if call("batch_upload", lib.rdc_batch_upload(ctx, items, 2)) == OK:
            call("batch_render", lib.rdc_batch_render(ctx))
        call("synchronize", lib.rdc_synchronize(ctx))
    finally:
        lib.rdc_destroy(ctx)
    return out, acc


def test_every_allocation_failure_is_reported_and_leaves_a_usable_context():
    lib = native.load()
    scene = shrink(scenegen.c1_plain().scene, W, H)
    sc, sc2 = scene.to_c(), shrink(scenegen.c1_plain(seed=4).scene, 8, 8).to_c()
    failed_calls = set()
    try:
        for n in range(64):
            os.environ["RDC_FAIL_ALLOC_AFTER"] = str(n)
            statuses, _ = _sequence(lib, sc, sc2)
            for name, st in statuses:
                assert st in (OK, OOM, NO_SCENE), (n, name, st)
                if st == OOM:
                    failed_calls.add(name)
            d = dict(statuses)
            if d.get("upload") == OOM:
                assert d["reset"] == NO_SCENE and d["render"] == NO_SCENE, (n, statuses)
            assert d.get("synchronize", OK) == OK, (n, statuses)
            if all(st == OK for _, st in statuses):
                break  # the budget covers every allocation of the sequence
        else:
            pytest.fail("the sequence still failed with 64 allocations allowed")
    finally:
        os.environ.pop("RDC_FAIL_ALLOC_AFTER", None)
    assert {"create", "upload", "read_rgba8", "set_accel_lbvh", "backward", "intersect",
            "batch_upload"} <= failed_calls, failed_calls
    # no injection: the same sequence renders the oracle's image
    statuses, acc = _sequence(lib, sc, sc2)
    assert all(st == OK for _, st in statuses), statuses
    ref, _ = oracle.render(sc, 0, SPP, BOUNCES, SEED, threads=4)
    assert bits_equal(acc, ref)
