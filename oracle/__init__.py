"""ctypes binding of the CPU oracle (oracle/_build/liboracle_raydar.so).

TEST INFRASTRUCTURE ONLY: the checker the CUDA backend is compared with.
Only tests/, the smoke check and the benchmark's CPU-baseline leg load it.
The oracle restates src/renderer/cpu.rs, src/utils/mod.rs,
src/scene/world.rs and src/scene/camera.rs:210-231 of the reference; see
raydar_oracle.hpp for the line-by-line map and the parity status.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle_raydar.so"

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} missing: run `make -C oracle` (or __graft_entry__.build())")
    lib = C.CDLL(str(LIB_PATH))
    P = C.c_void_p
    FP = C.POINTER(C.c_float)
    U32P = C.POINTER(C.c_uint32)
    lib.oracle_render.argtypes = [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, FP,
                                  C.POINTER(C.c_uint64), C.c_int]
    lib.oracle_render_pixels.argtypes = [P, U32P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                         C.c_uint64, C.c_uint32, FP, C.POINTER(C.c_uint64)]
    lib.oracle_intersect.argtypes = [P, FP, FP, C.c_uint32, FP, C.POINTER(C.c_int32), FP,
                                     C.POINTER(C.c_uint8)]
    lib.oracle_scatter.argtypes = [P, FP, FP, FP, C.POINTER(C.c_int32), U32P, C.c_uint32, FP, FP]
    lib.oracle_tonemap.argtypes = [FP, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint8)]
    lib.oracle_tonemap.restype = None
    lib.oracle_camera_matrices.argtypes = [P, FP, FP, FP, FP]
    lib.oracle_philox4x32_10.argtypes = [U32P, U32P, U32P]
    lib.oracle_philox4x32_10.restype = None
    lib.oracle_bounce_words.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, U32P]
    lib.oracle_bounce_words.restype = None
    lib.oracle_uniforms.argtypes = [U32P, C.c_uint32, FP, FP]
    lib.oracle_uniforms.restype = None
    DP = C.POINTER(C.c_double)
    for fn in (lib.oracle_gradient, lib.oracle_gradient_f32):
        fn.argtypes = [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, FP, DP, DP, DP, DP,
                       C.c_int, C.POINTER(C.c_uint64), DP]
    _lib = lib
    return lib


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _u(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _desc(scene_c):
    return C.cast(C.pointer(scene_c.desc), C.c_void_p)


def render(scene_c, s0, n, max_bounces, seed, accum=None, threads=1, stream=0):
    """Accumulate samples [s0, s0+n) of every pixel; returns (accum HxWx4, segments)."""
    lib = load()
    w, h = scene_c.desc.camera.resolution_x, scene_c.desc.camera.resolution_y
    acc = np.zeros((h, w, 4), np.float32) if accum is None else np.ascontiguousarray(accum, np.float32).copy()
    seg = C.c_uint64(0)
    rc = lib.oracle_render(_desc(scene_c), s0, n, max_bounces, seed, stream, _f(acc), C.byref(seg), threads)
    if rc != 0:
        raise RuntimeError(f"oracle_render failed ({rc})")
    return acc, seg.value


def gradient(scene_c, s0, n, max_bounces, seed, dl_dimage, threads=1, stream=0, pathwise=False, fp32=False):
    """FP64 reference gradient of sum(dl_dimage * image), image = mean radiance
    (HxWx3) of samples [s0, s0+n).  Returns (g_albedo Nx3, g_roughness N,
    g_emission Nx3, image HxWx3), all float64; with pathwise=True also the
    roughness gradient's pathwise part alone (N) as a fifth item (the part a
    small central difference with common random numbers sees when no coin
    flips).  fp32=True: the same derivative with each path's intermediates
    in float (the sums over paths in double), the precision the CUDA adjoint
    works in."""
    lib = load()
    w, h = scene_c.desc.camera.resolution_x, scene_c.desc.camera.resolution_y
    nobj = scene_c.desc.object_count
    dl = np.ascontiguousarray(dl_dimage, np.float32).reshape(h, w, 3)
    ga = np.zeros((nobj, 3), np.float64)
    gr = np.zeros(nobj, np.float64)
    ge = np.zeros((nobj, 3), np.float64)
    img = np.zeros((h, w, 3), np.float64)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    gp = np.zeros(nobj, np.float64)
    lost = C.c_uint64(0)
    fn = lib.oracle_gradient_f32 if fp32 else lib.oracle_gradient
    rc = fn(_desc(scene_c), s0, n, max_bounces, seed, stream, _f(dl), dp(ga), dp(gr), dp(ge), dp(img), threads,
            C.byref(lost), dp(gp))
    if rc != 0:
        raise RuntimeError(f"oracle_gradient failed ({rc})")
    gradient.lost_paths = lost.value
    if pathwise:
        return ga, gr, ge, img, gp
    return ga, gr, ge, img


def render_pixels(scene_c, pixels, s0, n, max_bounces, seed, accum=None, stream=0):
    lib = load()
    px = np.ascontiguousarray(pixels, np.uint32)
    acc = np.zeros((len(px), 4), np.float32) if accum is None else np.ascontiguousarray(accum, np.float32).copy()
    seg = C.c_uint64(0)
    rc = lib.oracle_render_pixels(_desc(scene_c), _u(px), len(px), s0, n, max_bounces, seed, stream,
                                  _f(acc), C.byref(seg))
    if rc != 0:
        raise RuntimeError(f"oracle_render_pixels failed ({rc})")
    return acc, seg.value


def intersect(scene_c, origins, directions):
    lib = load()
    o = np.ascontiguousarray(origins, np.float32)
    d = np.ascontiguousarray(directions, np.float32)
    n = len(o)
    t = np.zeros(n, np.float32)
    idx = np.zeros(n, np.int32)
    nrm = np.zeros((n, 3), np.float32)
    fr = np.zeros(n, np.uint8)
    lib.oracle_intersect(_desc(scene_c), _f(o), _f(d), n, _f(t), idx.ctypes.data_as(C.POINTER(C.c_int32)),
                         _f(nrm), fr.ctypes.data_as(C.POINTER(C.c_uint8)))
    return t, idx, nrm, fr


def scatter(scene_c, origins, directions, t, index, words):
    lib = load()
    o = np.ascontiguousarray(origins, np.float32)
    d = np.ascontiguousarray(directions, np.float32)
    tt = np.ascontiguousarray(t, np.float32)
    ii = np.ascontiguousarray(index, np.int32)
    ww = np.ascontiguousarray(words, np.uint32)
    n = len(o)
    oo = np.zeros((n, 3), np.float32)
    do = np.zeros((n, 3), np.float32)
    rc = lib.oracle_scatter(_desc(scene_c), _f(o), _f(d), _f(tt), ii.ctypes.data_as(C.POINTER(C.c_int32)),
                            _u(ww), n, _f(oo), _f(do))
    if rc != 0:
        raise RuntimeError(f"oracle_scatter failed ({rc})")
    return oo, do


def tonemap(accum, sample_count):
    lib = load()
    a = np.ascontiguousarray(accum, np.float32)
    out = np.zeros(a.shape, np.uint8)
    lib.oracle_tonemap(_f(a), a.size // 4, sample_count, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def camera_matrices(camera_c):
    lib = load()
    mats = [np.zeros(16, np.float32) for _ in range(4)]
    rc = lib.oracle_camera_matrices(C.cast(C.pointer(camera_c), C.c_void_p), *[_f(m) for m in mats])
    if rc != 0:
        raise RuntimeError("oracle_camera_matrices: singular matrix")
    return mats  # view, proj, inverse_view, inverse_proj


def philox(ctr, key):
    lib = load()
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib.oracle_philox4x32_10(_u(c), _u(k), _u(out))
    return out


def bounce_words(seed, stream, pixel, sample, bounce):
    lib = load()
    out = np.zeros(12, np.uint32)
    lib.oracle_bounce_words(seed, stream, pixel, sample, bounce, _u(out))
    return out


def uniforms(words):
    lib = load()
    w = np.ascontiguousarray(words, np.uint32)
    a = np.zeros(len(w), np.float32)
    b = np.zeros(len(w), np.float32)
    lib.oracle_uniforms(_u(w), len(w), _f(a), _f(b))
    return a, b
