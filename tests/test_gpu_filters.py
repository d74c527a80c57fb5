"""The brute-force pass-1 filters on the device, through the C ABI, on rays
built to sit at their margins (src/renderer/cpu.rs:34-98 is the test they
must never disagree with).

`tests/test_brute_filters.py` checks the filters' float arithmetic restated
in numpy; this checks the kernels themselves (their FMAs, the packed pairs,
the record layout the host writes) against the oracle's closest hit: every
ray's hit index, t, normal and face are compared bit for bit.  The scene has
one run of spheres at three coordinate scales and one run of 24 cubes (long
enough for the cube filter); each object gets rays that graze it at
1e-3..1e-7 relative of its radius from both sides, rays that start on its
surface (a bounce leaving it), and for cubes rays aimed at edges and
corners, starting on faces and inside.  The same rays go through the LBVH,
whose grown boxes rest on the same rounding bounds."""
import numpy as np
import pytest

import oracle
from raydar_gb300 import native
from raydar_gb300.scene import Camera, Material, Object, Scene, World
from tests.helpers import bits_equal

pytestmark = pytest.mark.gpu

F = np.float32


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _scene(rng):
    mat = Material(albedo=np.array([0.5, 0.5, 0.5], F), roughness=1.0)
    objs = []
    for i in range(48):
        scale = (2.0, 40.0, 1500.0)[i % 3]
        c = rng.uniform(-scale, scale, 3).astype(F)
        r = float(F(np.exp(rng.uniform(np.log(0.01), np.log(3.0)))))
        objs.append(Object("Sphere", c, r, mat))
    for i in range(24):
        scale = (2.0, 40.0, 800.0)[i % 3]
        c = rng.uniform(-scale, scale, 3).astype(F)
        objs.append(Object("Cube", c, float(F(rng.uniform(0.05, 4.0))), mat))
    cam = Camera.new([0.0, 2.0, -10.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], 64, 36, 0.01, 1000.0, fov=45.0)
    return Scene(cam, World("SkyColor", np.array([0.53, 0.8, 0.92], F), np.array([1.0, 1.0, 1.0], F)), objs)


def _sphere_rays(rng, c, r, k):
    c = c.astype(np.float64)
    out_o, out_d = [], []
    for rel in (1e-3, 1e-5, 1e-7):
        o = c + _unit(rng.normal(size=(k, 3))) * (r * rng.uniform(1.5, 50.0, k))[:, None]
        p = _unit(np.cross(c - o, rng.normal(size=(k, 3))))
        rho = r * (1 + rel * rng.uniform(-1, 1, k))
        d = _unit((c + p * rho[:, None]) - o) * rng.uniform(0.25, 3.0, (k, 1))
        d[: k // 2] *= -1  # half of them with the sphere behind the origin
        out_o.append(o)
        out_d.append(d)
    o = c + _unit(rng.normal(size=(k, 3))) * r  # on the surface, any direction
    out_o.append(o)
    out_d.append(_unit(rng.normal(size=(k, 3))) * rng.uniform(0.25, 3.0, (k, 1)))
    return np.concatenate(out_o), np.concatenate(out_d)


def _cube_rays(rng, c, side, k):
    c = c.astype(np.float64)
    h = side / 2.0
    out_o, out_d = [], []
    # aimed at an edge or corner point, perturbed by ~1e-6 of the half side
    t = c + h * np.sign(rng.normal(size=(k, 3))) * (1 + rng.uniform(-1e-6, 1e-6, (k, 3)))
    ax = rng.integers(0, 3, k)
    t[np.arange(k), ax] = c[ax] + h * rng.uniform(-1, 1, k)
    o = c + _unit(rng.normal(size=(k, 3))) * h * rng.uniform(2.0, 40.0, (k, 1))
    out_o.append(o)
    out_d.append(t - o)
    # on a face, any direction
    o = c + h * rng.uniform(-1, 1, (k, 3))
    ax = rng.integers(0, 3, k)
    o[np.arange(k), ax] = c[ax] + h * np.sign(rng.normal(size=k))
    out_o.append(o)
    out_d.append(rng.normal(size=(k, 3)))
    # inside
    out_o.append(c + h * rng.uniform(-0.999, 0.999, (k, 3)))
    out_d.append(rng.normal(size=(k, 3)))
    d = np.concatenate(out_d)
    d = _unit(d) * rng.uniform(0.25, 3.0, (len(d), 1))
    return np.concatenate(out_o), d


@pytest.mark.parametrize("accel", ["brute_force", "lbvh"])
def test_filters_never_drop_a_hit_on_the_device(accel):
    """Brute force: the pass-1 filters.  LBVH: the grown leaf and node boxes
    (rdc_bvh.cuh), on the same rays."""
    from raydar_gb300 import CudaRenderer, RendererConfig

    rng = np.random.default_rng(2024)
    scene = _scene(rng)
    renderer = CudaRenderer(RendererConfig(), seed=0)
    mode = native.ACCEL_LBVH if accel == "lbvh" else native.ACCEL_BRUTE_FORCE
    renderer._check(renderer.lib.rdc_set_accel(renderer.ctx, mode), "set_accel")
    renderer.upload(scene)
    assert renderer.stats().accel == mode
    os_, ds = [], []
    for ob in scene.objects:
        if ob.geometry == "Sphere":
            o, d = _sphere_rays(rng, ob.center, ob.size, 600)
        else:
            o, d = _cube_rays(rng, ob.center, ob.size, 800)
        os_.append(o)
        ds.append(d)
    o = np.ascontiguousarray(np.concatenate(os_), F)
    d = np.concatenate(ds)
    d[np.abs(d) < 2.0 ** -30] = 2.0 ** -30  # inside the guarded fast path
    d = np.ascontiguousarray(d, F)
    n = len(o)
    t = np.zeros(n, F)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), F)
    fr = np.zeros(n, np.uint8)
    assert renderer.lib.rdc_intersect_rays(renderer.ctx, native.fptr(o), native.fptr(d), n, native.fptr(t),
                                           native.iptr(idx), native.fptr(nrm), native.u8ptr(fr)) == 0
    rt, ridx, rn, rf = oracle.intersect(scene.to_c(), o, d)
    assert (ridx >= 0).mean() > 0.3
    bad = np.flatnonzero(idx != ridx)
    assert bad.size == 0, f"{bad.size} of {n} rays differ in hit index, first {bad[:5]}: {idx[bad[:5]]} vs {ridx[bad[:5]]}"
    assert bits_equal(t, rt) and bits_equal(nrm, rn) and np.array_equal(fr, rf)
    renderer.close()
