"""Build of the CUDA library `librast_gb300.so` (sm_103a), in-tree.

The library is compiled straight from `csrc/*.cu` with nvcc: one object per
translation unit, compiled in parallel, then linked into one shared object
under `_build/`.  Every unit is compiled with `-fmad=false` and IEEE division
and square root: the rasteriser's FP32 results are defined operation by
operation, and a contracted multiply-add would change winning primitives.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "librast_gb300.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "--expt-relaxed-constexpr",
    "--extended-lambda",
    "-Xcompiler",
    "-fPIC,-O2",
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def library_path() -> Path:
    return BUILD_DIR / LIB_NAME


def up_to_date() -> bool:
    lib = library_path()
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every `csrc/*.cu` for sm_103a and link `_build/librast_gb300.so`."""
    if not force and up_to_date():
        return library_path()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    procs = []
    objs = []
    for src in sources():
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            print(out.decode(errors="replace"))
        if p.returncode != 0:
            errors.append(src.name)
    if errors:
        raise RuntimeError(f"nvcc failed for {errors}")
    tmp = BUILD_DIR / (LIB_NAME + ".tmp")
    link = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, library_path())
    return library_path()


if __name__ == "__main__":
    print(build(force=True, verbose=True))
