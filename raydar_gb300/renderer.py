"""CudaRenderer: Raydar's `trait Renderer` (src/renderer/mod.rs:25-35) over the C ABI.

Same methods, argument meaning and semantics as CpuRenderer
(src/renderer/cpu.rs:118-183): render_frame renders max_sample_count samples
from a fresh frame and returns the 8-bit image; render_sample adds one sample
and returns the image, or None once max_sample_count is reached; new_frame
resets the accumulator.  Errors the C ABI reports are raised as RdcError
(the reference CPU backend cannot fail; its Vulkan backend panics).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import native
from .scene import Scene


@dataclass
class RendererConfig:
    """src/renderer/mod.rs:11-23."""
    max_sample_count: int = 1024
    max_bounces: int = 12


class Timer:
    """src/renderer/timing.rs:69-127 (durations in seconds)."""

    def __init__(self):
        self._start: Optional[float] = None
        self.duration: Optional[float] = None

    def start(self):
        self._start = time.perf_counter()

    def start_if_not_started(self):
        if self._start is None:
            self.start()

    def end(self):
        if self._start is not None:
            self.duration = time.perf_counter() - self._start

    def end_if_not_ended(self):
        if self.duration is None:
            self.end()

    def set(self, seconds: float):
        self.duration = seconds


class Profiler:
    """src/renderer/timing.rs:10-19."""

    def __init__(self):
        self.frame_timer = Timer()
        self.sample_timer = Timer()
        self.prepare_timer = Timer()
        self.render_timer = Timer()


class CudaRenderer:
    """The GB300 backend behind the reference's Renderer interface."""

    def __init__(self, config: Optional[RendererConfig] = None, device: int = 0, seed: int = 0):
        self.lib = native.load()
        self.config = config or RendererConfig()
        self.seed = int(seed)
        self._profiler = Profiler()
        self._sample_count = 0
        self._uploaded: Optional[bytes] = None
        self._scene_c = None
        ctx = C.c_void_p()
        st = self.lib.rdc_create(C.byref(ctx), device)
        if st != native.RDC_OK:
            raise native.RdcError(st, self.lib.rdc_last_error(None).decode())
        self.ctx = ctx

    # ------------------------------------------------------------ helpers --
    def _check(self, st: int, what: str):
        if st != native.RDC_OK:
            raise native.RdcError(st, f"{what}: {self.lib.rdc_last_error(self.ctx).decode()}")

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.rdc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, scene: Scene, force: bool = False):
        """Copy the scene to the device if it changed since the last call."""
        sc = scene.to_c()
        # the descriptor's objects pointer differs per to_c(): compare contents
        key = bytes(sc.desc.camera) + bytes(sc.desc.world) + bytes(sc.objects)[: sc.desc.object_count *
                                                                                C.sizeof(native.RdcObject)]
        if force or key != self._uploaded:
            self._check(self.lib.rdc_scene_upload(self.ctx, sc.ref()), "rdc_scene_upload")
            self._uploaded = key
            self._scene_c = sc

    def render_range(self, spp_begin: int, spp_count: int):
        self._check(self.lib.rdc_render(self.ctx, spp_begin, spp_count, self.config.max_bounces,
                                        self.seed), "rdc_render")

    def accumulator(self, scene: Scene) -> np.ndarray:
        out = np.empty((scene.height, scene.width, 4), np.float32)
        self._check(self.lib.rdc_read_accum(self.ctx, native.fptr(out), out.size), "rdc_read_accum")
        return out

    def image(self, scene: Scene) -> np.ndarray:
        out = np.empty((scene.height, scene.width, 4), np.uint8)
        self._check(self.lib.rdc_read_rgba8(self.ctx, self._sample_count, native.u8ptr(out), out.size),
                    "rdc_read_rgba8")
        return out

    def stats(self) -> native.RdcStats:
        s = native.RdcStats()
        self._check(self.lib.rdc_stats_get(self.ctx, C.byref(s)), "rdc_stats_get")
        return s

    def update_materials(self, materials: np.ndarray):
        """Replace the uploaded scene's materials (MATERIAL_DTYPE records, scene
        order) without re-uploading geometry (rdc_update_materials)."""
        from .scene import MATERIAL_DTYPE
        m = np.ascontiguousarray(materials, MATERIAL_DTYPE)
        self._check(self.lib.rdc_update_materials(self.ctx, m.ctypes.data_as(C.POINTER(native.RdcMaterial)),
                                                  len(m)), "rdc_update_materials")
        self._uploaded = None  # the cached scene no longer matches the device copy

    # ------------------------------------------------------ differentiation --
    def _dims(self):
        c = self._scene_c.desc.camera
        return int(c.resolution_y), int(c.resolution_x), int(self._scene_c.desc.object_count)

    def forward(self, scene: Optional[Scene], spp: int, spp_begin: int = 0) -> np.ndarray:
        """Mean-radiance image (H x W x 3) of samples [spp_begin, spp_begin+spp)
        with the configured bounce limit and seed (rdc_forward).  scene None:
        the scene on the device as it is (e.g. after update_materials)."""
        if scene is not None:
            self.upload(scene)
        h, w, _ = self._dims()
        out = np.empty((h, w, 3), np.float32)
        self._check(self.lib.rdc_forward(self.ctx, spp_begin, spp, self.config.max_bounces, self.seed,
                                         native.fptr(out)), "rdc_forward")
        return out

    def backward(self, scene: Optional[Scene], dl_dimage: np.ndarray):
        """(dL/dalbedo N x 3, dL/droughness N, dL/demission N x 3) for the image
        of the last forward(), given dL/dimage (H x W x 3) (rdc_backward)."""
        if self._scene_c is None:
            raise native.RdcError(4, "backward: no scene uploaded")  # RDC_ERR_NO_SCENE
        h, w, n = self._dims()
        dl = np.ascontiguousarray(dl_dimage, np.float32).reshape(h, w, 3)
        ga = np.zeros((n, 3), np.float32)
        gr = np.zeros(n, np.float32)
        ge = np.zeros((n, 3), np.float32)
        self._check(self.lib.rdc_backward(self.ctx, native.fptr(dl), native.fptr(ga), native.fptr(gr),
                                          native.fptr(ge)), "rdc_backward")
        return ga, gr, ge

    # ----------------------------------------------------- trait Renderer --
    def render_frame(self, scene: Scene) -> np.ndarray:
        """cpu.rs:119-133: new frame, all samples, tone-mapped image."""
        self.new_frame(scene)
        n = self.config.max_sample_count
        if self._sample_count < n:
            self._profiler.prepare_timer.end_if_not_ended()
            self._profiler.render_timer.start_if_not_started()
            self.render_range(self._sample_count, n - self._sample_count)
            st = self.stats()  # synchronises
            self._sample_count = n
            self._profiler.render_timer.end()
            self._profiler.frame_timer.end()
            self._profiler.sample_timer.set(st.device_ms / 1e3 / max(1, st.paths // max(1, scene.width * scene.height)))
        return self.image(scene)

    def new_frame(self, scene: Scene):
        """cpu.rs:135-140."""
        self._profiler.frame_timer.start()
        self._profiler.prepare_timer.start()
        self._profiler.prepare_timer.duration = None
        self._profiler.render_timer = Timer()
        self.upload(scene)
        self._check(self.lib.rdc_reset(self.ctx), "rdc_reset")
        self._sample_count = 0

    def render_sample(self, scene: Scene) -> Optional[np.ndarray]:
        """cpu.rs:142-158: one more sample, or None once max_sample_count is reached."""
        if self._sample_count >= self.config.max_sample_count:
            return None
        self.upload(scene)
        self._profiler.prepare_timer.end_if_not_ended()
        self._profiler.render_timer.start_if_not_started()
        self.render_range(self._sample_count, 1)
        st = self.stats()
        self._sample_count += 1
        if self._sample_count == self.config.max_sample_count:
            self._profiler.render_timer.end()
            self._profiler.frame_timer.end()
        self._profiler.sample_timer.set(st.device_ms / 1e3)
        return self.image(scene)

    def profiler(self) -> Profiler:
        return self._profiler

    def sample_count(self) -> int:
        return self._sample_count

    def max_sample_count(self) -> int:
        return self.config.max_sample_count

    def max_bounces(self) -> int:
        return self.config.max_bounces

    def set_max_sample_count(self, count: int):
        self.config.max_sample_count = int(count)

    def set_max_bounces(self, bounces: int):
        self.config.max_bounces = int(bounces)
