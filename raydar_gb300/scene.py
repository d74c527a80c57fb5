"""Raydar's scene model and its `.rscn` JSON format, on the Python side.

Mirrors src/scene/{mod,camera,material,objects,world}.rs: a Scene holds a
Camera (with its four serialised matrices), a World and the Objects in
order.  `.rscn` is serde_json of that struct: vectors are {"x","y","z"},
matrices are four columns {"x","y","z","w"}, enums are externally tagged
({"Sphere": {...}}, {"Perspective": {"fov": 45.0}}, "Transparent").

All numbers are float32, as in the reference.  Camera matrices are taken as
stored, exactly as the reference does when it loads a file
(src/cli/mod.rs:32-40); `Camera.update_matrices()` recomputes them through
the library's rdc_camera_update_matrices (src/scene/camera.rs:210-231).
"""
from __future__ import annotations

import contextlib
import ctypes as C
import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional

import numpy as np

from . import native

f32 = np.float32

# Camera::update_matrices goes through the library unless a caller routes it
# elsewhere with `camera_matrices_from` (a function of an RdcCamera returning
# the view, projection and both inverse matrices as 16 column-major floats).
_matrices_fn = None


@contextlib.contextmanager
def camera_matrices_from(fn):
    """Within the block, compute camera matrices with `fn(RdcCamera) ->
    (view, proj, inverse_view, inverse_proj)` instead of the library's
    rdc_camera_update_matrices: lets a process that must not load the CUDA
    library (a CPU-only timing of the same scene) build scenes."""
    global _matrices_fn
    prev, _matrices_fn = _matrices_fn, fn
    try:
        yield
    finally:
        _matrices_fn = prev


def _v3(d) -> np.ndarray:
    return np.array([d["x"], d["y"], d["z"]], dtype=np.float32)


def _m4(d) -> np.ndarray:
    # column-major flat: x column first
    cols = [d[k] for k in ("x", "y", "z", "w")]
    return np.array([[c["x"], c["y"], c["z"], c["w"]] for c in cols], dtype=np.float32).reshape(16)


def _fmt(x) -> float:
    # Shortest decimal that parses back to the same float32 (as serde_json/ryu writes f32).
    return float(np.format_float_positional(f32(x), unique=True, trim="0")) if np.isfinite(x) else float(x)


def _jv3(v) -> dict:
    return {"x": _fmt(v[0]), "y": _fmt(v[1]), "z": _fmt(v[2])}


def _jm4(m) -> dict:
    m = np.asarray(m, dtype=np.float32).reshape(4, 4)
    return {k: {"x": _fmt(m[i, 0]), "y": _fmt(m[i, 1]), "z": _fmt(m[i, 2]), "w": _fmt(m[i, 3])}
            for i, k in enumerate(("x", "y", "z", "w"))}


@dataclass
class Camera:
    """src/scene/camera.rs:13-30."""
    position: np.ndarray
    target: np.ndarray
    up: np.ndarray
    resolution_x: int
    resolution_y: int
    projection: str = "Perspective"  # or "Orthographic"
    fov: float = 90.0                  # degrees (Perspective)
    size: float = 1.0                  # Orthographic
    near_clip: float = 0.01
    far_clip: float = 1000.0
    view_matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(16))
    proj_matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(16))
    inverse_view_matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(16))
    inverse_proj_matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(16))

    @staticmethod
    def new(position, target, up, resolution_x, resolution_y, near_clip, far_clip,
            projection="Perspective", fov=90.0, size=1.0) -> "Camera":
        """Camera::new (camera.rs:33-60): fields, then update_matrices."""
        cam = Camera(np.asarray(position, np.float32), np.asarray(target, np.float32),
                     np.asarray(up, np.float32), int(resolution_x), int(resolution_y),
                     projection, float(f32(fov)), float(f32(size)), float(f32(near_clip)),
                     float(f32(far_clip)))
        cam.update_matrices()
        return cam

    def to_c(self) -> native.RdcCamera:
        c = native.RdcCamera()
        c.position[:] = [float(x) for x in self.position]
        c.target[:] = [float(x) for x in self.target]
        c.up[:] = [float(x) for x in self.up]
        c.resolution_x = self.resolution_x
        c.resolution_y = self.resolution_y
        c.projection = (native.PROJECTION_PERSPECTIVE if self.projection == "Perspective"
                        else native.PROJECTION_ORTHOGRAPHIC)
        c.fov_degrees = self.fov
        c.ortho_size = self.size
        c.near_clip = self.near_clip
        c.far_clip = self.far_clip
        c.view_matrix[:] = [float(x) for x in self.view_matrix]
        c.proj_matrix[:] = [float(x) for x in self.proj_matrix]
        c.inverse_view_matrix[:] = [float(x) for x in self.inverse_view_matrix]
        c.inverse_proj_matrix[:] = [float(x) for x in self.inverse_proj_matrix]
        return c

    def update_matrices(self) -> None:
        """Camera::update_matrices (camera.rs:210-231) via the native library
        (or the function installed by `camera_matrices_from`)."""
        c = self.to_c()
        if _matrices_fn is not None:
            mats = [np.asarray(m, np.float32).reshape(16).copy() for m in _matrices_fn(c)]
            self.view_matrix, self.proj_matrix, self.inverse_view_matrix, self.inverse_proj_matrix = mats
            return
        lib = native.load()
        st = lib.rdc_camera_update_matrices(C.byref(c))
        if st != native.RDC_OK:
            raise native.RdcError(st, "rdc_camera_update_matrices: singular or invalid camera")
        self.view_matrix = np.array(c.view_matrix[:], np.float32)
        self.proj_matrix = np.array(c.proj_matrix[:], np.float32)
        self.inverse_view_matrix = np.array(c.inverse_view_matrix[:], np.float32)
        self.inverse_proj_matrix = np.array(c.inverse_proj_matrix[:], np.float32)

    def to_json(self) -> dict:
        proj = ({"Perspective": {"fov": _fmt(self.fov)}} if self.projection == "Perspective"
                else {"Orthographic": {"size": _fmt(self.size)}})
        return {
            "position": _jv3(self.position), "target": _jv3(self.target), "up": _jv3(self.up),
            "resolution_x": self.resolution_x, "resolution_y": self.resolution_y,
            "projection": proj, "near_clip": _fmt(self.near_clip), "far_clip": _fmt(self.far_clip),
            "view_matrix": _jm4(self.view_matrix), "proj_matrix": _jm4(self.proj_matrix),
            "inverse_view_matrix": _jm4(self.inverse_view_matrix),
            "inverse_proj_matrix": _jm4(self.inverse_proj_matrix),
        }

    @staticmethod
    def from_json(d: dict) -> "Camera":
        proj = d["projection"]
        if "Perspective" in proj:
            kind, fov, size = "Perspective", float(f32(proj["Perspective"]["fov"])), 1.0
        else:
            kind, fov, size = "Orthographic", 90.0, float(f32(proj["Orthographic"]["size"]))
        return Camera(_v3(d["position"]), _v3(d["target"]), _v3(d["up"]),
                      int(d["resolution_x"]), int(d["resolution_y"]), kind, fov, size,
                      float(f32(d["near_clip"])), float(f32(d["far_clip"])),
                      _m4(d["view_matrix"]), _m4(d["proj_matrix"]),
                      _m4(d["inverse_view_matrix"]), _m4(d["inverse_proj_matrix"]))


@dataclass
class World:
    """src/scene/world.rs:6-14."""
    kind: str = "SkyColor"  # SkyColor | SolidColor | Transparent
    top_color: np.ndarray = field(default_factory=lambda: np.array([0.53, 0.8, 0.92], np.float32))
    bottom_color: np.ndarray = field(default_factory=lambda: np.array([1.0, 1.0, 1.0], np.float32))
    color: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))

    def to_json(self):
        if self.kind == "SkyColor":
            return {"SkyColor": {"top_color": _jv3(self.top_color), "bottom_color": _jv3(self.bottom_color)}}
        if self.kind == "SolidColor":
            return {"SolidColor": _jv3(self.color)}
        return "Transparent"

    @staticmethod
    def from_json(d) -> "World":
        if d == "Transparent":
            return World("Transparent")
        if "SkyColor" in d:
            return World("SkyColor", _v3(d["SkyColor"]["top_color"]), _v3(d["SkyColor"]["bottom_color"]))
        return World("SolidColor", color=_v3(d["SolidColor"]))


@dataclass
class Material:
    """src/scene/material.rs:4-27 (defaults as Material::default)."""
    albedo: np.ndarray = field(default_factory=lambda: np.array([0.8, 0.8, 0.8], np.float32))
    roughness: float = 0.5
    metallic: float = 0.0
    emission_color: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    emission_strength: float = 0.0
    transmission: float = 0.0
    ior: float = 1.5

    def to_json(self):
        return {"albedo": _jv3(self.albedo), "roughness": _fmt(self.roughness),
                "metallic": _fmt(self.metallic), "emission_color": _jv3(self.emission_color),
                "emission_strength": _fmt(self.emission_strength),
                "transmission": _fmt(self.transmission), "ior": _fmt(self.ior)}

    @staticmethod
    def from_json(d) -> "Material":
        return Material(_v3(d["albedo"]), float(f32(d["roughness"])), float(f32(d["metallic"])),
                        _v3(d["emission_color"]), float(f32(d["emission_strength"])),
                        float(f32(d["transmission"])), float(f32(d["ior"])))


@dataclass
class Object:
    """src/scene/objects.rs:6-16, 40-50: geometry 'Sphere' (radius) or 'Cube' (side_length)."""
    geometry: str
    center: np.ndarray
    size: float  # radius or side_length
    material: Material = field(default_factory=Material)

    def to_json(self):
        if self.geometry == "Sphere":
            g = {"Sphere": {"center": _jv3(self.center), "radius": _fmt(self.size)}}
        else:
            g = {"Cube": {"center": _jv3(self.center), "side_length": _fmt(self.size)}}
        return {"geometry": g, "material": self.material.to_json()}

    @staticmethod
    def from_json(d) -> "Object":
        g = d["geometry"]
        if "Sphere" in g:
            return Object("Sphere", _v3(g["Sphere"]["center"]), float(f32(g["Sphere"]["radius"])),
                          Material.from_json(d["material"]))
        return Object("Cube", _v3(g["Cube"]["center"]), float(f32(g["Cube"]["side_length"])),
                      Material.from_json(d["material"]))


@dataclass
class Scene:
    """src/scene/mod.rs:13-18."""
    camera: Camera
    world: World
    objects: list

    # ---------------------------------------------------------------- io --
    def to_json(self) -> dict:
        return {"camera": self.camera.to_json(), "world": self.world.to_json(),
                "objects": [o.to_json() for o in self.objects]}

    @staticmethod
    def from_json(d: dict) -> "Scene":
        return Scene(Camera.from_json(d["camera"]), World.from_json(d["world"]),
                     [Object.from_json(o) for o in d["objects"]])

    def save(self, path) -> None:
        Path(path).write_text(json.dumps(self.to_json(), indent=2))

    @staticmethod
    def load(path) -> "Scene":
        return Scene.from_json(json.loads(Path(path).read_text()))

    # ------------------------------------------------------------ C view --
    def to_c(self) -> "SceneC":
        return SceneC(self)

    @property
    def width(self) -> int:
        return self.camera.resolution_x

    @property
    def height(self) -> int:
        return self.camera.resolution_y


class SceneC:
    """An rdc_scene_desc and the object array it points to (kept alive together)."""

    def __init__(self, scene: Scene):
        n = len(scene.objects)
        self.objects = (native.RdcObject * max(n, 1))()
        for i, o in enumerate(scene.objects):
            q = self.objects[i]
            q.geometry = native.GEOMETRY_SPHERE if o.geometry == "Sphere" else native.GEOMETRY_CUBE
            q.center[:] = [float(x) for x in o.center]
            q.radius = o.size if o.geometry == "Sphere" else 0.0
            q.side_length = o.size if o.geometry == "Cube" else 0.0
            m = o.material
            q.material.albedo[:] = [float(x) for x in m.albedo]
            q.material.roughness = m.roughness
            q.material.metallic = m.metallic
            q.material.emission_color[:] = [float(x) for x in m.emission_color]
            q.material.emission_strength = m.emission_strength
            q.material.transmission = m.transmission
            q.material.ior = m.ior
        self.desc = native.RdcSceneDesc()
        self.desc.camera = scene.camera.to_c()
        w = scene.world
        self.desc.world.kind = {"SkyColor": native.WORLD_SKY_COLOR, "SolidColor": native.WORLD_SOLID_COLOR,
                                "Transparent": native.WORLD_TRANSPARENT}[w.kind]
        self.desc.world.top_color[:] = [float(x) for x in w.top_color]
        self.desc.world.bottom_color[:] = [float(x) for x in w.bottom_color]
        self.desc.world.solid_color[:] = [float(x) for x in w.color]
        self.desc.objects = C.cast(self.objects, C.POINTER(native.RdcObject))
        self.desc.object_count = n

    def ref(self):
        return C.byref(self.desc)


def resized(scene: Scene, width: int, height: int) -> Scene:
    """The same scene at another resolution, the camera's matrices recomputed
    as the reference's Camera setters do (src/scene/camera.rs:140-152): what
    the editor does when its viewport changes size."""
    import copy
    s = copy.deepcopy(scene)
    s.camera.resolution_x = width
    s.camera.resolution_y = height
    s.camera.update_matrices()
    return s


def default_scene() -> Scene:
    """Scene::default (src/scene/mod.rs:20-67)."""
    cam = Camera.new([-3.09, 0.03, -1.16], [0, 0, 0], [0, 1, 0], 854, 480, 0.01, 1000.0, fov=90.0)
    objs = [
        Object("Sphere", np.array([0, 0.001, 0], np.float32), 1.0,
               Material(albedo=np.ones(3, np.float32), roughness=0.2, transmission=1.0)),
        Object("Cube", np.array([0, -101, 0], np.float32), 200.0,
               Material(albedo=np.array([0.34, 0.34, 0.44], np.float32))),
        Object("Cube", np.array([7, 3, 0], np.float32), 1.8,
               Material(emission_color=np.array([0.8, 0.5, 0.2], np.float32), emission_strength=30.0)),
    ]
    return Scene(cam, World(), objs)


# Packed rdc_object records (68 bytes, the C layout) for large generated scenes.
OBJECT_DTYPE = np.dtype([
    ("geometry", "<u4"), ("center", "<f4", 3), ("radius", "<f4"), ("side_length", "<f4"),
    ("albedo", "<f4", 3), ("roughness", "<f4"), ("metallic", "<f4"), ("emission_color", "<f4", 3),
    ("emission_strength", "<f4"), ("transmission", "<f4"), ("ior", "<f4"),
])
assert OBJECT_DTYPE.itemsize == C.sizeof(native.RdcObject)

MATERIAL_FIELDS = ("albedo", "roughness", "metallic", "emission_color", "emission_strength", "transmission", "ior")
MATERIAL_DTYPE = np.dtype([(f, OBJECT_DTYPE.fields[f][0]) for f in MATERIAL_FIELDS])
assert MATERIAL_DTYPE.itemsize == C.sizeof(native.RdcMaterial)


def material_records(scene) -> np.ndarray:
    """The objects' materials as rdc_material records (MATERIAL_DTYPE), in scene order."""
    if isinstance(scene, PackedScene):
        src = scene.packed
        out = np.empty(len(src), MATERIAL_DTYPE)
        for f in MATERIAL_FIELDS:
            out[f] = src[f]
        return out
    out = np.empty(len(scene.objects), MATERIAL_DTYPE)
    for i, o in enumerate(scene.objects):
        m = o.material
        out[i] = (m.albedo, m.roughness, m.metallic, m.emission_color, m.emission_strength, m.transmission, m.ior)
    return out


class PackedScene(Scene):
    """A Scene whose objects live in one numpy array of OBJECT_DTYPE records
    (generated scenes with 10^5 objects); `objects` is built lazily."""

    def __init__(self, camera: Camera, world: World, packed: np.ndarray):
        self.camera = camera
        self.world = world
        self.packed = packed
        self._objects = None

    @property
    def objects(self):
        if self._objects is None:
            out = []
            for r in self.packed:
                geo = "Sphere" if r["geometry"] == native.GEOMETRY_SPHERE else "Cube"
                size = float(r["radius"] if geo == "Sphere" else r["side_length"])
                m = Material(r["albedo"].copy(), float(r["roughness"]), float(r["metallic"]),
                             r["emission_color"].copy(), float(r["emission_strength"]),
                             float(r["transmission"]), float(r["ior"]))
                out.append(Object(geo, r["center"].copy(), size, m))
            self._objects = out
        return self._objects

    @objects.setter
    def objects(self, value):
        self._objects = value

    def to_c(self) -> "SceneC":
        return PackedSceneC(self)


class PackedSceneC(SceneC):
    def __init__(self, scene: PackedScene):
        n = len(scene.packed)
        self.objects = (native.RdcObject * max(n, 1))()
        C.memmove(self.objects, np.ascontiguousarray(scene.packed).ctypes.data, n * OBJECT_DTYPE.itemsize)
        self.desc = native.RdcSceneDesc()
        self.desc.camera = scene.camera.to_c()
        w = scene.world
        self.desc.world.kind = {"SkyColor": native.WORLD_SKY_COLOR, "SolidColor": native.WORLD_SOLID_COLOR,
                                "Transparent": native.WORLD_TRANSPARENT}[w.kind]
        self.desc.world.top_color[:] = [float(x) for x in w.top_color]
        self.desc.world.bottom_color[:] = [float(x) for x in w.bottom_color]
        self.desc.world.solid_color[:] = [float(x) for x in w.color]
        self.desc.objects = C.cast(self.objects, C.POINTER(native.RdcObject))
        self.desc.object_count = n
