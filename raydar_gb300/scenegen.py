"""Seeded synthetic scenes for the benchmark and parity workloads, written in
Raydar's `.rscn` format.

The reference ships no benchmark inputs, so these stand in for them:

  c1_plain      320x180, 64 spp, 8 bounces: 8 spheres (r ~ U[0.3,1.0]) on a
                diffuse ground, materials cycling Diffuse, Metal, Glass,
                Specular; camera at (0,1.5,-6) looking at the origin, fov 45.
  c2_default    1920x1080, 1024 spp, 12 bounces: 64 spheres (r log-uniform in
                [0.1,1.5]) and 16 cubes (edge U[0.3,2]) on the 20x20 ground,
                mix 40% diffuse / 25% metal / 20% glass / 15% specular.
  c3_batch      64 scenes of uneven resolution, spp, bounces and object count.
  c4_diff       512x512, 128 spp, 6 bounces: 32 spheres + 2 emissive spheres.

The material classes are parameter regimes of the reference's single
Material (src/scene/material.rs:4-13): Diffuse {roughness 1}, Specular
{roughness 0.5, the Material::default}, Metal {metallic 1, roughness
U[0,0.5]}, Glass {transmission 1, ior 1.5, roughness 0}; albedo U[0.1,0.9]^3.

The reference Cube has one side length (src/scene/objects.rs:46-50), so the
"20 x 0.2 x 20 ground slab" is a 20-unit cube whose top face is y = 0
(centre (0,-10,0)): identical from any camera above the ground.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .scene import Camera, Material, Object, Scene, World

SKY_TOP = (0.53, 0.8, 0.92)
SKY_BOTTOM = (1.0, 1.0, 1.0)


@dataclass
class Workload:
    name: str
    scene: Scene
    spp: int
    max_bounces: int


def _mat(kind: str, rng: np.random.Generator) -> Material:
    albedo = rng.uniform(0.1, 0.9, 3).astype(np.float32)
    if kind == "D":
        return Material(albedo=albedo, roughness=1.0)
    if kind == "S":
        return Material(albedo=albedo, roughness=0.5)
    if kind == "M":
        return Material(albedo=albedo, roughness=float(np.float32(rng.uniform(0.0, 0.5))), metallic=1.0)
    if kind == "G":
        return Material(albedo=albedo, roughness=0.0, transmission=1.0, ior=1.5)
    raise ValueError(kind)


def _ground(half_extent: float = 10.0) -> Object:
    side = 2.0 * half_extent
    return Object("Cube", np.array([0.0, -half_extent, 0.0], np.float32), side,
                  Material(albedo=np.array([0.5, 0.5, 0.5], np.float32), roughness=1.0))


def _place(rng, radii, extent, placed, inset=True, strict=True, max_tries=2000):
    """Rejection-sample non-overlapping footprints (x, z): centres in
    [-extent + r, extent - r] (inset) or [-extent, extent].  With strict=False
    an object that finds no free spot in max_tries keeps its last draw (dense
    batch scenes cannot all fit on the ground without touching)."""
    out = []
    for r in radii:
        lo, hi = (-extent + r, extent - r) if inset else (-extent, extent)
        for _ in range(max_tries):
            x, z = rng.uniform(lo, hi, 2)
            if all((x - px) ** 2 + (z - pz) ** 2 >= (r + pr) ** 2 for px, pz, pr in placed):
                break
        else:
            if strict:
                raise RuntimeError("could not place object without overlap")
        placed.append((x, z, r))
        out.append((x, z))
    return out


def _camera(w, h, pos, target, fov) -> Camera:
    return Camera.new(pos, target, [0.0, 1.0, 0.0], w, h, 0.01, 1000.0, fov=fov)


def c1_plain(seed: int = 1, width: int = 320, height: int = 180) -> Workload:
    rng = np.random.default_rng(seed)
    radii = rng.uniform(0.3, 1.0, 8)
    xz = _place(rng, radii, 3.0, [], inset=False)  # x, z ~ U[-3, 3]
    objs = [_ground()]
    cycle = "DMGS"
    for i, (r, (x, z)) in enumerate(zip(radii, xz)):
        objs.append(Object("Sphere", np.array([x, r, z], np.float32), float(np.float32(r)),
                           _mat(cycle[i % 4], rng)))
    cam = _camera(width, height, [0.0, 1.5, -6.0], [0.0, 0.0, 0.0], 45.0)
    return Workload("c1_plain", Scene(cam, World("SkyColor", np.array(SKY_TOP, np.float32),
                                                 np.array(SKY_BOTTOM, np.float32)), objs), 64, 8)


def _mix_kinds(rng, n, mix=(("D", 0.40), ("M", 0.25), ("G", 0.20), ("S", 0.15))):
    kinds = [k for k, _ in mix]
    p = np.array([w for _, w in mix])
    return list(rng.choice(kinds, size=n, p=p / p.sum()))


def c2_default(seed: int = 2, width: int = 1920, height: int = 1080, n_spheres: int = 64,
               n_cubes: int = 16, max_tries: int = 2000) -> Workload:
    rng = np.random.default_rng(seed)
    radii = np.exp(rng.uniform(np.log(0.1), np.log(1.5), n_spheres))
    edges = rng.uniform(0.3, 2.0, n_cubes)
    placed: list = []
    # footprints: spheres by radius, cubes by their half diagonal
    xz_s = _place(rng, radii, 10.0, placed, strict=False, max_tries=max_tries)
    xz_c = _place(rng, edges * np.sqrt(0.5), 10.0, placed, strict=False, max_tries=max_tries)
    kinds = _mix_kinds(rng, n_spheres + n_cubes)
    objs = [_ground()]
    for i, (r, (x, z)) in enumerate(zip(radii, xz_s)):
        objs.append(Object("Sphere", np.array([x, r, z], np.float32), float(np.float32(r)),
                           _mat(kinds[i], rng)))
    for j, (e, (x, z)) in enumerate(zip(edges, xz_c)):
        objs.append(Object("Cube", np.array([x, e / 2, z], np.float32), float(np.float32(e)),
                           _mat(kinds[n_spheres + j], rng)))
    cam = _camera(width, height, [0.0, 4.0, -17.0], [0.0, 0.5, 0.0], 45.0)
    sky = World("SkyColor", np.array(SKY_TOP, np.float32), np.array(SKY_BOTTOM, np.float32))
    return Workload("c2_default", Scene(cam, sky, objs), 1024, 12)


def c3_batch(seed: int = 3, count: int = 64) -> list[Workload]:
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        w = int(rng.choice(np.arange(128, 1025, 64)))
        h = w * 9 // 16 if rng.random() < 0.5 else w
        spp = int(round(np.exp(rng.uniform(np.log(16), np.log(512)))))
        bounces = int(rng.integers(4, 13))
        ns = int(rng.integers(4, 201))
        nc = int(rng.integers(0, 21))
        sub = c2_default(seed=int(rng.integers(1 << 30)), width=w, height=h, n_spheres=ns, n_cubes=nc,
                         max_tries=200)
        out.append(Workload(f"c3_scene{k:02d}", sub.scene, spp, bounces))
    return out


def c4_diff(seed: int = 4, width: int = 512, height: int = 512) -> Workload:
    rng = np.random.default_rng(seed)
    radii = rng.uniform(0.2, 0.8, 34)
    xz = _place(rng, radii, 8.0, [])
    kinds = _mix_kinds(rng, 32)
    objs = [_ground(10.0)]
    for i in range(32):
        r = radii[i]
        x, z = xz[i]
        objs.append(Object("Sphere", np.array([x, r, z], np.float32), float(np.float32(r)),
                           _mat(kinds[i], rng)))
    for i in (32, 33):
        r = radii[i]
        x, z = xz[i]
        m = Material(albedo=np.ones(3, np.float32), roughness=1.0,
                     emission_color=np.ones(3, np.float32),
                     emission_strength=float(np.float32(rng.uniform(2.0, 8.0))))
        objs.append(Object("Sphere", np.array([x, r + 1.5, z], np.float32), float(np.float32(r)), m))
    cam = _camera(width, height, [0.0, 5.0, -13.0], [0.0, 0.5, 0.0], 45.0)
    sky = World("SkyColor", np.array(SKY_TOP, np.float32), np.array(SKY_BOTTOM, np.float32))
    return Workload("c4_diff", Scene(cam, sky, objs), 128, 6)


WORKLOADS = {"c1_plain": c1_plain, "c2_default": c2_default, "c4_diff": c4_diff}


def _packed_materials(rng, rec, kinds):
    """Fill the material fields of packed records for class letters D/M/G/S."""
    n = len(rec)
    rec["albedo"] = rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32)
    rec["ior"] = 1.5
    rec["roughness"] = np.where(kinds == "D", 1.0, np.where(kinds == "S", 0.5, 0.0)).astype(np.float32)
    metal = kinds == "M"
    rec["roughness"][metal] = rng.uniform(0.0, 0.5, metal.sum()).astype(np.float32)
    rec["metallic"] = metal.astype(np.float32)
    rec["transmission"] = (kinds == "G").astype(np.float32)


def c5_large(seed: int = 5, width: int = 1920, height: int = 1080, n_spheres: int = 100_000,
             n_cubes: int = 10_000) -> Workload:
    """100k spheres (radius log-uniform in [0.01, 0.2]) and 10k cubes (edge
    U[0.02, 0.3]) with centres uniform in a 40 x 10 x 40 box, the usual
    material mix; 1920x1080, 256 spp, 12 bounces (device-built LBVH)."""
    from .scene import OBJECT_DTYPE, PackedScene
    rng = np.random.default_rng(seed)
    n = n_spheres + n_cubes
    rec = np.zeros(n, OBJECT_DTYPE)
    rec["geometry"][:n_spheres] = 0
    rec["geometry"][n_spheres:] = 1
    rec["center"] = np.stack([rng.uniform(-20, 20, n), rng.uniform(0, 10, n), rng.uniform(-20, 20, n)], 1)
    rec["radius"][:n_spheres] = np.exp(rng.uniform(np.log(0.01), np.log(0.2), n_spheres))
    rec["side_length"][n_spheres:] = rng.uniform(0.02, 0.3, n_cubes)
    kinds = np.array(_mix_kinds(rng, n))
    _packed_materials(rng, rec, kinds)
    cam = _camera(width, height, [0.0, 6.0, -32.0], [0.0, 5.0, 0.0], 50.0)
    sky = World("SkyColor", np.array(SKY_TOP, np.float32), np.array(SKY_BOTTOM, np.float32))
    return Workload("c5_large", PackedScene(cam, sky, rec), 256, 12)
