"""The host-side record layout the brute-force kernels read (rdc_flatten.hpp),
checked on the CPU through the C++ itself: a small shim over `flatten` is
compiled with the library's host flags and called with seeded scenes.

The pass-1 filters are only as safe as two per-object constants the host
writes: the sphere filter's s = c.c - q must lie at or below its exact value
(q >= r^2 + 2^-16 (2 c.c + r^2) + 2^-70), and a cube run's header R must
bound |centre| + half side * sqrt(3) over the run.  Both are checked here in
exact rational arithmetic, together with where each float lands (sphere
pairs: centres, s, c.c, r*r; cube pairs: min and max per axis; odd runs
repeat their last object)."""
import ctypes as C
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from raydar_gb300 import build, native
from raydar_gb300.scene import Camera, Material, Object, Scene, World

F = np.float32

SHIM = r"""
#include <cstring>
#include <vector>
#include "rdc_flatten.hpp"
extern "C" int probe_flatten(const rdc_scene_desc* sc, float* rec_out, uint32_t rec_cap, int* runs_out,
                             uint32_t runs_cap, uint32_t* nrec, uint32_t* nruns) {
    const rdc::FlatCounts fc = rdc::flat_counts(sc);
    *nrec = fc.nrec;
    *nruns = fc.nruns;
    if (fc.nrec > rec_cap || fc.nruns > runs_cap) return 1;
    std::vector<float4> rec(fc.nrec), hit(sc->object_count ? sc->object_count : 1);
    std::vector<rdc::MatDev> mat(sc->object_count ? sc->object_count : 1);
    std::vector<int4> runs(fc.nruns);
    const bool fast = rdc::flatten(sc, rec.data(), hit.data(), mat.data(), runs.data());
    std::memcpy(rec_out, rec.data(), fc.nrec * sizeof(float4));
    std::memcpy(runs_out, runs.data(), fc.nruns * sizeof(int4));
    return fast ? 0 : 2;
}
"""


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("flatten_probe")
    src = d / "probe.cpp"
    src.write_text(SHIM)
    so = d / "probe.so"
    cmd = [cxx, *build.HOST_CXX, "-shared", "-I", str(build.INCLUDE), "-I", str(build.CSRC), "-I",
           build._cuda_include(), str(src), "-o", str(so)]
    subprocess.run(cmd, check=True, capture_output=True)
    lib = C.CDLL(str(so))
    lib.probe_flatten.restype = C.c_int
    lib.probe_flatten.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    return lib


def _flatten(lib, scene):
    sc = scene.to_c()
    cap = 4 * len(scene.objects) + 64
    rec = np.zeros((cap, 4), F)
    runs = np.zeros((cap, 4), np.int32)
    nrec, nruns = C.c_uint32(0), C.c_uint32(0)
    st = lib.probe_flatten(C.addressof(sc.desc), rec.ctypes.data, cap, runs.ctypes.data, cap,
                           C.byref(nrec), C.byref(nruns))
    assert st in (0, 2)
    return rec[: nrec.value], runs[: nruns.value], st == 0


def _scene(rng, kinds):
    mat = Material(albedo=np.array([0.5, 0.5, 0.5], F), roughness=1.0)
    objs = []
    for k in kinds:
        scale = float(rng.choice([1.0, 50.0, 3000.0]))
        c = rng.uniform(-scale, scale, 3).astype(F)
        size = float(F(np.exp(rng.uniform(np.log(1e-3), np.log(20.0)))))
        objs.append(Object("Sphere" if k == "S" else "Cube", c, size, mat))
    cam = Camera.new([0.0, 1.0, -5.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], 16, 9, 0.01, 1000.0, fov=45.0)
    return Scene(cam, World("SkyColor", np.array([0.5, 0.7, 1.0], F), np.array([1.0, 1.0, 1.0], F)), objs)


def _q(x):
    return Fraction(float(x))


def test_sphere_and_cube_records(probe):
    rng = np.random.default_rng(31)
    # runs: 7 spheres, 11 cubes, 4 spheres, 5 cubes (odd runs repeat their last object)
    kinds = "S" * 7 + "C" * 11 + "S" * 4 + "C" * 5
    scene = _scene(rng, kinds)
    rec, runs, fast = _flatten(probe, scene)
    assert fast
    objs = scene.objects
    assert [tuple(r[:3]) for r in runs] == [(0, 0, 7), (1, 7, 18), (0, 18, 22), (1, 22, 27)]
    for geom, first, end, off in runs:
        n = end - first
        if geom == 0:  # spheres: 3 float4 per pair
            assert n == 0 or off + 3 * ((n + 1) // 2) <= len(rec)
            for j in range(n + (n & 1)):
                o = objs[first + min(j, n - 1)]  # an odd run repeats its last sphere
                p, h = divmod(j, 2)
                A, B, Cr = rec[off + 3 * p], rec[off + 3 * p + 1], rec[off + 3 * p + 2]
                c = o.center.astype(F)
                assert (A[h], A[2 + h], B[h]) == (c[0], c[1], c[2])
                rr = F(o.size) * F(o.size)
                cc = (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]  # the reference's float c.c
                assert Cr[h] == cc and Cr[2 + h] == rr
                # s <= c.c - q exactly, q >= r^2 + 2^-16 (2 c.c + r^2) + 2^-70, with c.c exact
                cce = sum(_q(x) * _q(x) for x in c)
                q_min = _q(rr) + (2 * cce + _q(rr)) / 2 ** 16 + Fraction(1, 2 ** 70)
                s = _q(B[2 + h])
                assert s <= cce - q_min
                # and not loose by more than a float rounding of the larger term
                assert cce - q_min - s <= (abs(cce) + q_min) * Fraction(1, 2 ** 22) + Fraction(1, 2 ** 60)
        else:  # cubes: a header (R, 0, 0, 0), then 3 float4 per pair
            R = _q(rec[off][0])
            bound = 0
            for i in range(first, end):
                o = objs[i]
                c = o.center.astype(np.float64)
                h = float(F(o.size) * F(0.5))
                bound = max(bound, float(np.sqrt((c * c).sum())) + h * np.sqrt(3.0))
            assert R >= Fraction(bound) and R <= Fraction(bound) * Fraction(10002, 10000) + 1
            for j in range(n + (n & 1)):
                o = objs[first + min(j, n - 1)]
                p, h = divmod(j, 2)
                c = o.center.astype(F)
                hs = F(o.size) * F(0.5)
                for ax in range(3):
                    row = rec[off + 1 + 3 * p + ax]
                    assert row[h] == c[ax] - hs and row[2 + h] == c[ax] + hs


def test_range_guards_turn_the_fast_path_off(probe):
    rng = np.random.default_rng(5)
    scene = _scene(rng, "SSCC")
    scene.objects[0].center = np.array([2.0 ** 51, 0.0, 0.0], F)  # beyond the sphere guard (2^50)
    _, _, fast = _flatten(probe, scene)
    assert not fast
    scene = _scene(rng, "SSCC")
    scene.objects[2].size = 0.0  # a cube side must be > 0
    _, _, fast = _flatten(probe, scene)
    assert not fast


def _header_define(name):
    import re
    txt = (build.INCLUDE / "raydar_cuda.h").read_text()
    return int(re.search(rf"#define {name} (\d+)u", txt).group(1))


def test_worst_case_layout_fits_the_static_scratch(probe):
    """rdc_render_static keeps the flattened scene in a fixed device array.
    Its record region must hold the layout of any scene of up to
    RDC_STATIC_MAX_OBJECTS objects: alternating spheres and cubes (every run
    of length one: 3 records per sphere, 4 per cube with the run header) is
    the densest, 3584 records for 1024 objects."""
    nmax = _header_define("RDC_STATIC_MAX_OBJECTS")
    scratch = _header_define("RDC_STATIC_SCRATCH_BYTES")
    # counters 256 B; per object slot: hit 16 B, material 64 B, run 16 B; the rest is records
    rec_capacity = (scratch - 256 - nmax * (16 + 64 + 16)) // 16
    rng = np.random.default_rng(77)
    for kinds in ("SC" * (nmax // 2), "CS" * (nmax // 2), "C" + "SC" * ((nmax - 1) // 2)):
        rec, runs, _ = _flatten(probe, _scene(rng, kinds))
        assert len(runs) == len(kinds)
        assert len(rec) == sum(3 if k == "S" else 4 for k in kinds)
        assert len(rec) <= rec_capacity, (len(rec), rec_capacity)
    # any mix: never more than 4 records per object
    for _ in range(20):
        n = int(rng.integers(1, nmax + 1))
        kinds = "".join(rng.choice(["S", "C"], n, p=[0.5, 0.5]))
        rec, _, _ = _flatten(probe, _scene(rng, kinds))
        assert len(rec) <= 4 * n <= rec_capacity
