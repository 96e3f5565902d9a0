"""Builds libmpm_gb300.so (the engine's CUDA kernels and C ABI) in-tree.

The library is compiled with nvcc for sm_103a only and placed in
``taichi_elements_gb300/_build/``.  Translation units are compiled in
parallel and linked with the static CUDA runtime, so the .so depends on the
driver only.  A rebuild happens when any source or header is newer than the
library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libmpm_gb300.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["mpm_kernels.cu", "mpm_adjoint.cu", "mpm_io.cu", "mpm_voxelize.cu", "mpm_render.cu"]


def nvcc_path() -> str:
    cand = os.environ.get("NVCC")
    if cand:
        return cand
    for p in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the GB300 engine cannot be built")


def library_path() -> Path:
    return BUILD_DIR / LIB_NAME


def _deps() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def common_flags() -> list[str]:
    return ARCH_FLAGS + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler",
        "-fPIC",
        "-I",
        str(INCLUDE),
        "-I",
        str(CSRC),
    ]


def build_library(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile the engine library if needed and return its path."""
    lib = library_path()
    if not force and not _stale(lib):
        return lib
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    flags = common_flags() + list(extra_flags or [])

    def compile_one(src: str) -> Path:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        cmd = [nvcc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(SOURCES))) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
