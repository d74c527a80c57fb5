"""The host-only C++ (the .rscn reader and writer, the camera matrices) and
the CPU oracle under AddressSanitizer and UndefinedBehaviorSanitizer, on the
CPU: tests/sanitize/host_checks.cpp parses the reference scenes and
thousands of truncated and corrupted variants, recomputes random cameras and
runs every oracle entry point; any sanitizer report or failed check fails
the test.  (The device code has its own stand-in: the bounds-checked build.)"""
import os
import shutil
import subprocess

import pytest

from tests.conftest import GOLDEN, ROOT


def test_host_code_and_oracle_are_clean_under_asan_and_ubsan(tmp_path):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = None
    for nvcc in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if nvcc and os.path.exists(nvcc):
            cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
            break
    if cuda_inc is None:
        pytest.skip("no CUDA headers")
    exe = tmp_path / "host_checks"
    src = [ROOT / "tests" / "sanitize" / "host_checks.cpp", ROOT / "raydar_gb300" / "csrc" / "rdc_rscn.cpp",
           ROOT / "raydar_gb300" / "csrc" / "rdc_camera.cpp", ROOT / "oracle" / "oracle_capi.cpp"]
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-ffp-contract=off", "-pthread",
           "-I", str(ROOT / "include"), "-I", str(ROOT / "raydar_gb300" / "csrc"), "-I", cuda_inc,
           *map(str, src), "-o", str(exe)]
    b = subprocess.run(cmd, capture_output=True, text=True)
    if b.returncode != 0 and "sanitizer" in (b.stderr + b.stdout).lower():
        pytest.skip("this compiler has no sanitizer runtime")
    assert b.returncode == 0, b.stderr[-3000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe), str(GOLDEN / "default.rscn"), str(GOLDEN / "benchmark.rscn")],
                       capture_output=True, text=True, env=env, timeout=600)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-4000:]
    assert "host checks: ok" in r.stdout
    assert "runtime error" not in out and "AddressSanitizer" not in out, out[-4000:]
