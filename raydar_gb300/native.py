"""ctypes binding of the C ABI in include/raydar_cuda.h (libraydar_cuda.so).

There is no fallback: if the shared library has not been built, loading it
raises.  The structures below mirror the header field for field.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libraydar_cuda.so"

RDC_OK = 0
STATUS_NAMES = {
    0: "RDC_OK",
    1: "RDC_ERR_INVALID_ARGUMENT",
    2: "RDC_ERR_UNSUPPORTED",
    3: "RDC_ERR_LIMIT",
    4: "RDC_ERR_NO_SCENE",
    5: "RDC_ERR_CUDA",
    6: "RDC_ERR_OUT_OF_MEMORY",
    7: "RDC_ERR_DEVICE",
}
GEOMETRY_SPHERE, GEOMETRY_CUBE = 0, 1
WORLD_SKY_COLOR, WORLD_SOLID_COLOR, WORLD_TRANSPARENT = 0, 1, 2
PROJECTION_PERSPECTIVE, PROJECTION_ORTHOGRAPHIC = 0, 1
MAX_RESOLUTION = 16384
MAX_OBJECTS = 1 << 24
MAX_BRUTE_OBJECTS = 4096
ACCEL_AUTO, ACCEL_BRUTE_FORCE, ACCEL_LBVH = 0, 1, 2
FORM_AUTO, FORM_MEGAKERNEL, FORM_WAVEFRONT = 0, 1, 2
MAX_BOUNCES = 1024

F3 = C.c_float * 3
F16 = C.c_float * 16


class RdcCamera(C.Structure):
    _fields_ = [
        ("position", F3), ("target", F3), ("up", F3),
        ("resolution_x", C.c_uint32), ("resolution_y", C.c_uint32),
        ("projection", C.c_uint32), ("fov_degrees", C.c_float), ("ortho_size", C.c_float),
        ("near_clip", C.c_float), ("far_clip", C.c_float),
        ("view_matrix", F16), ("proj_matrix", F16),
        ("inverse_view_matrix", F16), ("inverse_proj_matrix", F16),
    ]


class RdcWorld(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("top_color", F3), ("bottom_color", F3), ("solid_color", F3)]


class RdcMaterial(C.Structure):
    _fields_ = [
        ("albedo", F3), ("roughness", C.c_float), ("metallic", C.c_float),
        ("emission_color", F3), ("emission_strength", C.c_float),
        ("transmission", C.c_float), ("ior", C.c_float),
    ]


class RdcObject(C.Structure):
    _fields_ = [
        ("geometry", C.c_uint32), ("center", F3), ("radius", C.c_float),
        ("side_length", C.c_float), ("material", RdcMaterial),
    ]


class RdcSceneDesc(C.Structure):
    _fields_ = [
        ("camera", RdcCamera), ("world", RdcWorld),
        ("objects", C.POINTER(RdcObject)), ("object_count", C.c_uint32),
    ]


class RdcStats(C.Structure):
    _fields_ = [
        ("segments", C.c_uint64), ("paths", C.c_uint64), ("device_ms", C.c_float),
        ("sample_count", C.c_uint32), ("kernel_launches", C.c_uint32),
        ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
        ("node_visits", C.c_uint64), ("prim_tests", C.c_uint64), ("accel", C.c_uint32), ("bvh_depth", C.c_uint32),
    ]


class RdcBatchItem(C.Structure):
    _fields_ = [("scene", C.POINTER(RdcSceneDesc)), ("spp", C.c_uint32), ("max_bounces", C.c_uint32),
                ("seed", C.c_uint64)]


class RdcLaunchConfig(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("refill_min_idle", C.c_uint32)]


# name -> (restype, argtypes).  Every exported symbol of include/raydar_cuda.h.
_P = C.c_void_p
_FP = C.POINTER(C.c_float)
SIGNATURES = {
    "rdc_version": (C.c_char_p, []),
    "rdc_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "rdc_destroy": (None, [_P]),
    "rdc_last_error": (C.c_char_p, [_P]),
    "rdc_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "rdc_synchronize": (C.c_int, [_P]),
    "rdc_scene_upload": (C.c_int, [_P, C.POINTER(RdcSceneDesc)]),
    "rdc_reset": (C.c_int, [_P]),
    "rdc_set_accel": (C.c_int, [_P, C.c_uint32]),
    "rdc_set_render_form": (C.c_int, [_P, C.c_uint32]),
    "rdc_render": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64]),
    "rdc_render_static": (C.c_int, [C.POINTER(RdcSceneDesc), C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                    C.c_uint64, C.c_void_p, C.POINTER(C.c_uint64), C.c_char_p, C.c_size_t]),
    "rdc_read_accum": (C.c_int, [_P, _FP, C.c_size_t]),
    "rdc_batch_upload": (C.c_int, [_P, C.POINTER(RdcBatchItem), C.c_uint32]),
    "rdc_batch_render": (C.c_int, [_P]),
    "rdc_batch_read_accum": (C.c_int, [_P, C.c_uint32, _FP, C.c_size_t]),
    "rdc_batch_set_config": (C.c_int, [_P, C.POINTER(RdcLaunchConfig)]),
    "rdc_batch_get_config": (C.c_int, [_P, C.POINTER(RdcLaunchConfig)]),
    "rdc_set_render_config": (C.c_int, [_P, C.POINTER(RdcLaunchConfig)]),
    "rdc_forward": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _FP]),
    "rdc_update_materials": (C.c_int, [_P, C.POINTER(RdcMaterial), C.c_uint32]),
    "rdc_render_wavefront": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64]),
    "rdc_scene_parse_rscn": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(RdcSceneDesc), C.POINTER(RdcObject),
                                       C.c_uint32, C.POINTER(C.c_uint32)]),
    "rdc_scene_write_rscn": (C.c_int, [C.POINTER(RdcSceneDesc), C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "rdc_backward": (C.c_int, [_P, _FP, _FP, _FP, _FP]),
    "rdc_get_render_config": (C.c_int, [_P, C.POINTER(RdcLaunchConfig)]),
    "rdc_batch_autotune": (C.c_int, [_P, C.POINTER(RdcLaunchConfig), C.POINTER(C.c_float)]),
    "rdc_write_accum": (C.c_int, [_P, _FP, C.c_size_t, C.c_uint32]),
    "rdc_read_rgba8": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint8), C.c_size_t]),
    "rdc_stats_get": (C.c_int, [_P, C.POINTER(RdcStats)]),
    "rdc_intersect_rays": (C.c_int, [_P, _FP, _FP, C.c_uint32, _FP, C.POINTER(C.c_int32), _FP,
                                     C.POINTER(C.c_uint8)]),
    "rdc_scatter_fixed": (C.c_int, [_P, _FP, _FP, _FP, C.POINTER(C.c_int32), C.POINTER(C.c_uint32),
                                    C.c_uint32, _FP, _FP]),
    "rdc_measure_fp32_issue": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "rdc_measure_fp32x2_issue": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "rdc_selftest_staging_timeout": (C.c_int, [_P]),
    "rdc_selftest_radix_sort": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32,
                                          C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "rdc_selftest_exclusive_scan": (C.c_int, [_P, C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32)]),
    "rdc_camera_update_matrices": (C.c_int, [C.POINTER(RdcCamera)]),
}

_lib = None


def load() -> C.CDLL:
    """Load libraydar_cuda.so (built by raydar_gb300.build); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class RdcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_FP)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def uptr(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def u8ptr(a: np.ndarray):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint8))
