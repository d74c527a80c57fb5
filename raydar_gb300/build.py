"""Build recipe for the native parts: the sm_103a CUDA library and the CPU oracle.

Everything is built in-tree (outputs are git-ignored):
  raydar_gb300/libraydar_cuda.so     the product: kernels + the C ABI of include/raydar_cuda.h
  raydar_gb300/libraydar_cuda_checked.so
                                     the same sources with device bounds checks
                                     (-DRDC_BOUNDS_CHECK=1: out-of-range indices are counted and
                                     reported as RDC_ERR_DEVICE, never trap); built on demand by
                                     its test, the stand-in for a memory checker
  oracle/_build/liboracle_raydar.so  test infrastructure: the CPU restatement of the reference
  raydar_gb300/_build/*.o            intermediate objects and the ptxas resource report

Translation units are compiled in parallel; no cmake, one -gencode.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = PKG / "libraydar_cuda.so"
LIB_CHECKED = PKG / "libraydar_cuda_checked.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle_raydar.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: the reference (Rust) never contracts a*b+c; IEEE division and
# square root and no flush-to-zero, so every float matches the CPU path.
NVCC_DEVICE = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true",
               "-prec-sqrt=true", "-ftz=false", "-Xptxas", "-v", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off"]
HOST_CXX = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build raydar_gb300")
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _run(cmd: list[str], log: Path | None = None) -> None:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if log is not None:
        log.write_text(p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError(f"build step failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile csrc/*.cu and csrc/*.cpp for sm_103a and link libraydar_cuda.so
    (checked: the bounds-checked libraydar_cuda_checked.so)."""
    build_dir = PKG / "_build_checked" if checked else BUILD
    lib = LIB_CHECKED if checked else LIB
    extra = ["-DRDC_BOUNDS_CHECK=1"] if checked else []
    build_dir.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    incs = ["-I", str(INCLUDE), "-I", str(CSRC)]
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = build_dir / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append(([nvcc, *ARCH, *NVCC_DEVICE, *extra, *incs, "-c", str(src), "-o", str(obj)],
                         build_dir / (src.stem + ".ptxas.txt")))
    cxx = os.environ.get("CXX", "g++")
    for src in sorted(CSRC.glob("*.cpp")):
        obj = build_dir / (src.stem + ".cpp.o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append(([cxx, *HOST_CXX, *extra, *incs, "-I", _cuda_include(), "-c", str(src), "-o", str(obj)],
                         None))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_run, cmd, log) for cmd, log in jobs]:
            fut.result()
    if force or jobs or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-Xcompiler", "-fPIC",
              "-lpthread", "-ldl", "-lrt"])
    if verbose:
        for f in sorted(build_dir.glob("*.ptxas.txt")):
            sys.stdout.write(f.read_text())
    return lib


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) with -ffp-contract=off."""
    (ORACLE_DIR / "_build").mkdir(exist_ok=True)
    deps = [ORACLE_DIR / "oracle_capi.cpp", ORACLE_DIR / "raydar_oracle.hpp", ORACLE_DIR / "raydar_oracle_grad.hpp",
            ORACLE_DIR / "Makefile", INCLUDE / "raydar_cuda.h"]
    if force or _stale(ORACLE_LIB, deps):
        _run(["make", "-s", "-C", str(ORACLE_DIR)])
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_library, force)
        b = ex.submit(build_oracle, force)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB, ORACLE_LIB)
