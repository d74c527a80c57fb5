"""Batched rendering: many scenes in one persistent launch (rdc_batch_*).

`BatchRenderer` holds a context with one uploaded batch.  Item i is rendered
with RNG stream i and its own seed; render() replays the batch's CUDA graph
(clear + persistent kernel).  `autotune()` runs the library's launch-shape
search (block size, resident blocks per SM = paths in flight, refill
threshold) and can cache the result in a JSON file keyed by GPU and batch
signature.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import native
from .scene import Scene


class BatchRenderer:
    def __init__(self, items: Sequence[tuple], device: int = 0):
        """items: (scene, spp, max_bounces, seed) tuples."""
        self.lib = native.load()
        ctx = C.c_void_p()
        st = self.lib.rdc_create(C.byref(ctx), device)
        if st != native.RDC_OK:
            raise native.RdcError(st, self.lib.rdc_last_error(None).decode())
        self.ctx = ctx
        self.scenes = [it[0] for it in items]
        self._keep = [sc.to_c() for sc in self.scenes]
        arr = (native.RdcBatchItem * len(items))()
        for i, (sc, spp, bounces, seed) in enumerate(items):
            arr[i].scene = C.pointer(self._keep[i].desc)
            arr[i].spp = int(spp)
            arr[i].max_bounces = int(bounces)
            arr[i].seed = int(seed)
        self.items = list(items)
        self._check(self.lib.rdc_batch_upload(self.ctx, arr, len(items)), "rdc_batch_upload")

    def _check(self, st, what):
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

    def render(self):
        self._check(self.lib.rdc_batch_render(self.ctx), "rdc_batch_render")

    def stats(self) -> native.RdcStats:
        s = native.RdcStats()
        self._check(self.lib.rdc_stats_get(self.ctx, C.byref(s)), "rdc_stats_get")
        return s

    def accumulator(self, i: int) -> np.ndarray:
        sc: Scene = self.scenes[i]
        out = np.empty((sc.height, sc.width, 4), np.float32)
        self._check(self.lib.rdc_batch_read_accum(self.ctx, i, native.fptr(out), out.size), "rdc_batch_read_accum")
        return out

    def config(self) -> native.RdcLaunchConfig:
        c = native.RdcLaunchConfig()
        self._check(self.lib.rdc_batch_get_config(self.ctx, C.byref(c)), "rdc_batch_get_config")
        return c

    def set_config(self, block_size: int, blocks_per_sm: int, refill_min_idle: int):
        c = native.RdcLaunchConfig(block_size, blocks_per_sm, refill_min_idle)
        self._check(self.lib.rdc_batch_set_config(self.ctx, C.byref(c)), "rdc_batch_set_config")

    def signature(self) -> str:
        h = hashlib.sha1()
        for sc, spp, b, _ in self.items:
            h.update(f"{sc.width}x{sc.height}:{len(sc.objects)}:{spp}:{b};".encode())
        return h.hexdigest()[:16]

    def autotune(self, cache: Optional[Path] = None) -> dict:
        """Pick the fastest launch shape (cached per GPU + batch signature)."""
        key = None
        if cache is not None:
            import torch  # noqa: F401  (GPU name only)
            gpu = torch.cuda.get_device_name(0) if torch.cuda.is_available() else "gpu"
            key = f"{gpu}/{self.signature()}"
            if Path(cache).exists():
                d = json.loads(Path(cache).read_text())
                if key in d:
                    c = d[key]
                    self.set_config(c["block_size"], c["blocks_per_sm"], c["refill_min_idle"])
                    return dict(c, cached=True)
        best = native.RdcLaunchConfig()
        ms = C.c_float(0)
        self._check(self.lib.rdc_batch_autotune(self.ctx, C.byref(best), C.byref(ms)), "rdc_batch_autotune")
        res = {"block_size": best.block_size, "blocks_per_sm": best.blocks_per_sm,
               "refill_min_idle": best.refill_min_idle, "ms": ms.value}
        if cache is not None:
            d = json.loads(Path(cache).read_text()) if Path(cache).exists() else {}
            d[key] = res
            Path(cache).write_text(json.dumps(d, indent=1))
        return dict(res, cached=False)
