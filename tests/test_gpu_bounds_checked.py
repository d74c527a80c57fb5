"""The bounds-checked build (libraydar_cuda_checked.so, -DRDC_BOUNDS_CHECK=1):
the stand-in for a device memory checker.  Every data-dependent index into a
device array (materials, hit records, LBVH nodes and primitives, accumulators,
dL/dimage, gradient rows, wavefront queues) is range-checked; an index out of
range is counted and reported as RDC_ERR_DEVICE, never trapped.  A subprocess
runs every kernel family through the checked library -- brute-force renders,
the reference's benchmark scene, the LBVH, the wavefront form (brute force
and LBVH), a batch, the
adjoint on both accelerations, the single-stage checks and the allocation-
free render -- and must see no device error and the oracle's results."""
import json
import subprocess
import sys

import numpy as np
import pytest

import oracle
from raydar_gb300 import build, scenegen
from tests.conftest import GOLDEN, ROOT
from tests.helpers import bits_equal, shrink

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import ctypes as C, json, sys
from pathlib import Path
sys.path.insert(0, sys.argv[1])
import numpy as np
from raydar_gb300 import native
native.LIB_PATH = Path(sys.argv[2])
from raydar_gb300 import CudaRenderer, RendererConfig, scenegen
from raydar_gb300.batch import BatchRenderer
from raydar_gb300.scene import Scene, resized
out, status = {}, {}
lib = native.load()
assert "checked" in str(native.LIB_PATH)

def run(name, fn):
    try:
        fn()
        status[name] = "ok"
    except Exception as e:  # an RdcError carries the library's message
        status[name] = repr(e)

def render(name, scene, spp, bounces, seed, accel=native.ACCEL_AUTO, wavefront=False):
    r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=seed)
    r._check(lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
    r.upload(scene)
    r._check(lib.rdc_reset(r.ctx), "rdc_reset")
    if wavefront:
        r._check(lib.rdc_render_wavefront(r.ctx, 0, spp, bounces, seed), "rdc_render_wavefront")
    else:
        r.render_range(0, spp)
    out[name] = r.accumulator(scene)
    r._check(lib.rdc_synchronize(r.ctx), "rdc_synchronize")
    r.close()

c1 = resized(scenegen.c1_plain().scene, 24, 16)
bench = resized(Scene.load(sys.argv[3]), 48, 27)
big = scenegen.c5_large(seed=3, width=24, height=16, n_spheres=600, n_cubes=60).scene
c2 = resized(scenegen.c2_default().scene, 32, 18)
run("brute", lambda: render("brute", c1, 2, 8, 5))
run("benchmark_scene", lambda: render("benchmark_scene", bench, 1, 12, 6))
run("lbvh", lambda: render("lbvh", big, 1, 6, 9, accel=native.ACCEL_LBVH))
run("wavefront", lambda: render("wavefront", c2, 19, 12, 7, wavefront=True))  # waves of 16 + 3 samples
run("wavefront_lbvh", lambda: render("wavefront_lbvh", big, 18, 8, 14, accel=native.ACCEL_LBVH, wavefront=True))

def batch():
    items = [(c1, 2, 6, 11), (resized(scenegen.c1_plain(seed=4).scene, 16, 16), 1, 4, 12)]
    br = BatchRenderer(items)
    br.render()
    for i in range(len(items)):
        out[f"batch{i}"] = br.accumulator(i)
    br.close()
run("batch", batch)

def adjoint(name, scene, accel):
    r = CudaRenderer(RendererConfig(max_bounces=6), seed=13)
    r._check(lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
    r.forward(scene, 4)
    dl = np.random.default_rng(2).uniform(-1, 1, (scene.height, scene.width, 3)).astype(np.float32)
    ga, gr, ge = r.backward(scene, dl)
    out[name + "_ga"], out[name + "_gr"], out[name + "_ge"], out[name + "_dl"] = ga, gr, ge, dl
    r._check(lib.rdc_synchronize(r.ctx), "rdc_synchronize")
    r.close()
c4 = resized(scenegen.c4_diff().scene, 20, 20)
run("adjoint_brute", lambda: adjoint("adjoint_brute", c4, native.ACCEL_BRUTE_FORCE))
run("adjoint_lbvh", lambda: adjoint("adjoint_lbvh", big, native.ACCEL_LBVH))

def stages():
    r = CudaRenderer(RendererConfig(max_bounces=8), seed=1)
    r.upload(c1)
    rng = np.random.default_rng(3)
    o = np.tile(c1.camera.position.astype(np.float32), (256, 1))
    d = rng.normal(size=(256, 3)).astype(np.float32)
    d[:, 2] = np.abs(d[:, 2]) + 0.5
    t, idx = np.zeros(256, np.float32), np.zeros(256, np.int32)
    nrm, fr = np.zeros((256, 3), np.float32), np.zeros(256, np.uint8)
    r._check(lib.rdc_intersect_rays(r.ctx, native.fptr(o), native.fptr(d), 256, native.fptr(t), native.iptr(idx),
                                    native.fptr(nrm), native.u8ptr(fr)), "rdc_intersect_rays")
    out["isect_t"], out["isect_idx"], out["isect_o"], out["isect_d"] = t, idx, o, d
    r._check(lib.rdc_synchronize(r.ctx), "rdc_synchronize")
    r.close()
run("stages", stages)

def static():
    import torch
    acc = torch.zeros(c1.height * c1.width * 4, dtype=torch.float32, device="cuda:0")
    segs = C.c_uint64(0)
    err = C.create_string_buffer(256)
    st = lib.rdc_render_static(c1.to_c().ref(), C.c_void_p(acc.data_ptr()), 0, 2, 8, 5, None, C.byref(segs),
                               err, len(err))
    if st != 0:
        raise RuntimeError(err.value.decode())
    out["static"] = acc.cpu().numpy().reshape(c1.height, c1.width, 4)
run("static", static)
np.savez(sys.argv[4], **out)
print(json.dumps(status))
"""


@pytest.fixture(scope="module")
def checked_run(tmp_path_factory):
    lib = build.build_library(checked=True)
    npz = tmp_path_factory.mktemp("checked") / "out.npz"
    p = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT), str(lib), str(GOLDEN / "benchmark.rscn"), str(npz)],
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-3000:]
    status = json.loads(p.stdout.strip().splitlines()[-1])
    return status, dict(np.load(npz))


def test_no_kernel_family_sees_an_out_of_range_index(checked_run):
    status, _ = checked_run
    assert status and all(v == "ok" for v in status.values()), status


def test_checked_renders_equal_the_oracle(checked_run):
    from raydar_gb300.scene import Scene, resized
    _, out = checked_run
    c1 = resized(scenegen.c1_plain().scene, 24, 16)
    cases = [
        ("brute", c1, 2, 8, 5, 0), ("static", c1, 2, 8, 5, 0),
        ("benchmark_scene", resized(Scene.load(GOLDEN / "benchmark.rscn"), 48, 27), 1, 12, 6, 0),
        ("lbvh", scenegen.c5_large(seed=3, width=24, height=16, n_spheres=600, n_cubes=60).scene, 1, 6, 9, 0),
        ("wavefront", resized(scenegen.c2_default().scene, 32, 18), 19, 12, 7, 0),
        ("wavefront_lbvh", scenegen.c5_large(seed=3, width=24, height=16, n_spheres=600, n_cubes=60).scene,
         18, 8, 14, 0),
        ("batch0", c1, 2, 6, 11, 0), ("batch1", resized(scenegen.c1_plain(seed=4).scene, 16, 16), 1, 4, 12, 1),
    ]
    for name, scene, spp, bounces, seed, stream in cases:
        ref, _ = oracle.render(scene.to_c(), 0, spp, bounces, seed, threads=8, stream=stream)
        assert bits_equal(out[name], ref), name
    t, idx, _, _ = oracle.intersect(c1.to_c(), out["isect_o"], out["isect_d"])
    assert bits_equal(out["isect_t"], t) and bits_equal(out["isect_idx"], idx)


def test_checked_adjoint_equals_the_fp64_oracle(checked_run):
    from raydar_gb300.scene import resized
    _, out = checked_run
    scenes = {"adjoint_brute": resized(scenegen.c4_diff().scene, 20, 20),
              "adjoint_lbvh": scenegen.c5_large(seed=3, width=24, height=16, n_spheres=600, n_cubes=60).scene}
    for name, scene in scenes.items():
        oa, orr, oe, _ = oracle.gradient(scene.to_c(), 0, 4, 6, 13, out[name + "_dl"], threads=16)
        for g, o in ((out[name + "_ga"], oa), (out[name + "_gr"], orr), (out[name + "_ge"], oe)):
            if np.linalg.norm(o) > 0:
                assert np.linalg.norm(g - o) / np.linalg.norm(o) < 1e-3, name
