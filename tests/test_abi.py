"""The C ABI surface: the library loads and exports every entry point that
include/raydar_cuda.h declares, and argument checks fail cleanly (no GPU needed)."""
import ctypes as C
import re

import pytest

from raydar_gb300 import native
from tests.conftest import ROOT


def _declared():
    text = (ROOT / "include" / "raydar_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rdc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = native.load()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), f"{n} not exported by libraydar_cuda.so"
        assert n in native.SIGNATURES, f"{n} has no ctypes signature"
    assert set(native.SIGNATURES) == set(names)


RUST_SYS = ROOT / "rust" / "raydar-cuda-sys" / "src" / "lib.rs"
RUST_RENDERER = ROOT / "rust" / "src" / "renderer" / "cuda.rs"
RUST_PATCH = ROOT / "rust" / "raydar-cuda.patch"


def _header_prototypes():
    """name -> (return type, [parameter types]) of every header entry point."""
    text = (ROOT / "include" / "raydar_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for ret, name, params in re.findall(r"([A-Za-z_][A-Za-z0-9_ ]*?\**)\s*\b(rdc_[a-z0-9_]+)\s*\(([^)]*)\)\s*;",
                                         text):
        types = []
        for prm in params.split(","):
            prm = " ".join(prm.split())
            if prm in ("", "void"):
                continue
            m = re.match(r"(.*?[\s*])([A-Za-z_][A-Za-z0-9_]*)$", prm)
            types.append(" ".join(m.group(1).replace("*", " * ").split()))
        out[name] = (" ".join(ret.replace("*", " * ").split()), types)
    return out


_C_TO_RUST = {
    "rdc_status": "rdc_status", "void": None, "int": "c_int", "uint32_t": "u32", "uint64_t": "u64",
    "size_t": "usize", "float": "f32", "double": "f64", "uint8_t": "u8", "int32_t": "i32", "char": "c_char",
}


def _c_type_to_rust(t):
    """'const rdc_object *' -> '*const rdc_object', 'void * *' -> '*mut *mut c_void'."""
    parts = t.split()
    stars = parts.count("*")
    const = parts[0] == "const"
    base = [p for p in parts if p not in ("const", "*")][0]
    rust = "c_void" if (base == "void" and stars) else _C_TO_RUST.get(base, base)
    for k in range(stars):
        rust = ("*const " if (const and k == 0) else "*mut ") + rust
    return rust


def _rust_externs():
    text = RUST_SYS.read_text()
    block = text[text.index('extern "C" {'):]
    block = re.sub(r"//[^\n]*", "", block)
    out = {}
    for name, params, ret in re.findall(r"pub fn (rdc_[a-z0-9_]+)\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block):
        types = [" ".join(p.split(":", 1)[1].split()) for p in params.split(",") if p.strip()]
        out[name] = (" ".join(ret.split()) if ret else None, types)
    return out


def test_the_rust_binding_declares_every_entry_point_with_the_header_signature():
    """rust/raydar-cuda-sys/src/lib.rs (the FFI crate the --cuda backend links)
    names every function the header declares, and nothing else, with each
    parameter's type the header's."""
    protos, externs = _header_prototypes(), _rust_externs()
    assert set(externs) == set(_declared()) == set(protos)
    for name, (ret, params) in protos.items():
        rret, rparams = externs[name]
        assert rret == _c_type_to_rust(ret) or (ret == "void" and rret is None), (name, ret, rret)
        assert [_c_type_to_rust(p) for p in params] == rparams, (name, params, rparams)


_RUST_PRIM = {"f32": (4, 4), "u32": (4, 4), "i32": (4, 4), "u64": (8, 8), "f64": (8, 8), "usize": (8, 8)}


def _rust_structs():
    text = RUST_SYS.read_text()
    out = {}
    for name, body in re.findall(r"pub struct (rdc_[a-z_]+) \{(.*?)\}", text, re.S):
        out[name] = re.findall(r"pub ([a-z_0-9]+): ([^,]+),", body)
    return out


def _rust_layout(structs, name, cache):
    """Offsets, size and alignment of a repr(C) struct from its parsed fields."""
    if name in cache:
        return cache[name]
    off, align, fields = 0, 1, []
    for fname, ftype in structs[name]:
        ftype = ftype.strip()
        m = re.match(r"\[(\w+); (\d+)\]", ftype)
        if m:
            (esz, eal), n = _rust_prim_or_struct(structs, m.group(1), cache), int(m.group(2))
            sz, al = esz * n, eal
        else:
            sz, al = _rust_prim_or_struct(structs, ftype, cache)
        off = (off + al - 1) // al * al
        fields.append((fname, off))
        off += sz
        align = max(align, al)
    size = (off + align - 1) // align * align
    cache[name] = (fields, size, align)
    return cache[name]


def _rust_prim_or_struct(structs, t, cache):
    if t.startswith("*"):
        return 8, 8
    if t in _RUST_PRIM:
        return _RUST_PRIM[t]
    fields, size, align = _rust_layout(structs, t, cache)
    return size, align


def test_rust_structures_have_the_header_layout(tmp_path):
    """Every repr(C) structure of the FFI crate has the header struct's fields
    in the same order at the same offsets, and the same size (the header's
    offsets from a program gcc compiles against it); the crate's compile-time
    size assertions state the same sizes."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    structs = _rust_structs()
    assert set(structs) == {"rdc_camera", "rdc_world", "rdc_material", "rdc_object", "rdc_scene_desc", "rdc_stats",
                            "rdc_batch_item", "rdc_launch_config"}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "raydar_cuda.h"', "int main(void) {"]
    for name, fields in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for fname, _ in fields:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    c = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True)
             .stdout.splitlines())
    cache = {}
    asserted = dict(re.findall(r"size_of::<(rdc_[a-z_]+)>\(\) == (\d+)", RUST_SYS.read_text()))
    for name in structs:
        fields, size, _ = _rust_layout(structs, name, cache)
        assert int(c[name]) == size == int(asserted[name]), name
        for fname, off in fields:
            assert int(c[f"{name}.{fname}"]) == off, (name, fname)


def test_the_cuda_backend_uses_only_declared_entry_points_and_the_patch_wires_it():
    """src/renderer/cuda.rs calls only functions the crate declares and
    implements every method of trait Renderer (src/renderer/mod.rs:25-35);
    the patch adds the module, the --cuda flag and the branch that builds it
    (src/cli/mod.rs:50-54), the renderer's name (src/main.rs:36) and the
    dependency."""
    rs = RUST_RENDERER.read_text()
    used = set(re.findall(r"ffi::(rdc_[a-z0-9_]+)\(", rs))
    assert used and used <= set(_rust_externs())
    for m in ("render_frame", "render_sample", "new_frame", "profiler", "sample_count", "max_sample_count",
              "max_bounces", "set_max_sample_count", "set_max_bounces"):
        assert re.search(rf"fn {m}\(", rs), m
    patch = RUST_PATCH.read_text()
    added = "\n".join(ln[1:] for ln in patch.splitlines() if ln.startswith("+") and not ln.startswith("+++"))
    for needle in ("pub mod cuda;", "pub cuda: bool", "Box::new(CudaRenderer::new(config))",
                   'if args.common.cuda { "CUDA" }', 'raydar-cuda-sys = { path = "raydar-cuda-sys" }'):
        assert needle in added, needle
    touched = set(re.findall(r"^\+\+\+ b/(\S+)", patch, re.M))
    assert touched == {"Cargo.toml", "src/renderer/mod.rs", "src/cli/mod.rs", "src/main.rs"}


def test_enum_constants_agree_across_the_header_and_both_bindings():
    """RDC_ACCEL_* and RDC_FORM_* (and RDC_FORM_AUTO_WAVE_SAMPLES) have the
    same values in include/raydar_cuda.h, the ctypes binding and the Rust
    crate."""
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "raydar_cuda.h").read_text(), flags=re.S)
    header = {}
    for body in re.findall(r"enum\s*\{([^}]*)\}", text):
        for name, val in re.findall(r"(RDC_(?:ACCEL|FORM)_[A-Z_]+)\s*=\s*(\d+)", body):
            header[name] = int(val)
    header.update({n: int(v) for n, v in re.findall(r"#define\s+(RDC_FORM_AUTO_WAVE_SAMPLES)\s+(\d+)u", text)})
    assert {"RDC_ACCEL_AUTO", "RDC_ACCEL_LBVH", "RDC_FORM_AUTO", "RDC_FORM_MEGAKERNEL", "RDC_FORM_WAVEFRONT",
            "RDC_FORM_AUTO_WAVE_SAMPLES"} <= set(header)
    rust = {n: int(v) for n, v in re.findall(r"pub const (RDC_(?:ACCEL|FORM)_[A-Z_]+): u32 = (\d+);",
                                               RUST_SYS.read_text())}
    for name, val in header.items():
        assert rust.get(name) == val, name
        py = getattr(native, name[len("RDC_"):], None)
        if py is not None:
            assert py == val, name
    assert native.FORM_WAVEFRONT == header["RDC_FORM_WAVEFRONT"] and native.ACCEL_LBVH == header["RDC_ACCEL_LBVH"]


def test_version_string():
    assert b"sm_103a" in native.load().rdc_version()


def test_create_on_a_missing_device_fails_with_a_message():
    lib = native.load()
    ctx = C.c_void_p()
    st = lib.rdc_create(C.byref(ctx), 999)
    assert st != native.RDC_OK and not ctx.value
    assert len(lib.rdc_last_error(None)) > 0


@pytest.mark.parametrize("name,args", [
    ("rdc_render", (None, 0, 1, 1, 0)),
    ("rdc_reset", (None,)),
    ("rdc_scene_upload", (None, None)),
    ("rdc_synchronize", (None,)),
])
def test_null_context_is_rejected(name, args):
    lib = native.load()
    assert getattr(lib, name)(*args) == 1  # RDC_ERR_INVALID_ARGUMENT


def test_destroy_accepts_null():
    native.load().rdc_destroy(None)


def test_camera_update_rejects_bad_input():
    lib = native.load()
    cam = native.RdcCamera()
    assert lib.rdc_camera_update_matrices(None) == 1
    assert lib.rdc_camera_update_matrices(C.byref(cam)) == 1  # zero resolution
